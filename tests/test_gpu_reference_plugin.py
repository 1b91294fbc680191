"""The reference's own CUDA plugin (src/cuda_box.cu, compiled unmodified for sm_103a by
oracle/ref.mk) under its host loop, beside the engine's plain FP64 mode on the same instances:
same status, iteration counts within one check interval, objectives within 1e-10 relative."""
import numpy as np
import pytest

import boxqp
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('seed', [1, 2])
def test_reference_cuda_plugin_agrees_with_fp64_engine(engine, seed):
    if not O.REF_CUBIN.exists():
        pytest.skip('the reference CUDA module was not built (no reference checkout where build() ran)')
    if not O.build_ref_cuda():
        pytest.skip('the driver-API harness did not compile')
    inst = boxqp.planted('graph10k', seed=seed, n=3000, lower_triplets=True)
    status, st, x_ref, _ = O.ref_cuda_solve(inst['rowptr'], inst['col'], inst['val'], inst['hrow'], inst['hcol'],
                                            inst['hval'], inst['c'], inst['lower'], inst['upper'], tol=1e-7)
    o = boxqp.options_struct(1e-7, 30.0, 200000, 'fp64')
    x, ours = engine.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
    assert status == boxqp.STATUS_NAMES[ours.status] == 'optimal'
    assert abs(int(st['iterations']) - int(ours.iterations)) <= 25
    assert abs(st['objective'] - ours.objective) <= 1e-10 * (1 + abs(st['objective']))
    assert np.max(np.abs(x - x_ref)) < 1e-5
