"""bqp_check_device_noalloc: the device verification for callers that cannot allocate.

Some callers must not allocate device memory while they verify a solution -- a serving loop
where cudaMalloc/cudaFree would synchronize the device and stall the solves in flight, or a
process whose device memory another allocator has already reserved, where cudaMalloc fails.
This entry point takes its scratch from a static device array in the library instead.  The
test calls it through the C-ABI twice in a row, on two different problems, and compares each
result with the allocating entry point bqp_check_device on the same device arrays.

This file is collected last (tests/test_zz_*), so a run that stops at the first failure has
already run every other test.
"""
import numpy as np
import pytest

import boxqp

pytestmark = pytest.mark.gpu

FIELDS = ('objective', 'primal_residual', 'stationarity_residual', 'dual_bound', 'relative_gap')


def device_arrays(torch, inst, x):
    return {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
            [('rowptr', inst['rowptr']), ('col', inst['col']), ('val', inst['val']), ('x', x), ('c', inst['c']),
             ('l', inst['lower']), ('u', inst['upper'])]}


def call(fn, n, d, tol=1e-6):
    st = boxqp.Stats()
    rc = fn(n, d['rowptr'].data_ptr(), d['col'].data_ptr(), d['val'].data_ptr(), d['x'].data_ptr(),
            d['c'].data_ptr(), d['l'].data_ptr(), d['u'].data_ptr(), tol, 0.0, 0, st)
    return rc, st


def test_noalloc_check_matches_allocating_check_on_two_calls():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    lib = boxqp.lib()
    rng = np.random.default_rng(5)
    cases = [boxqp.planted('graph10k', seed=31, n=20000), boxqp.planted('grid', seed=32, n=64 * 64)]
    for inst in cases:  # two calls in a row, different sizes: the shared scratch is cleared each time
        x = np.clip(inst['xstar'] + 1e-4 * rng.standard_normal(inst['n']), inst['lower'], inst['upper'])
        d = device_arrays(torch, inst, x)
        rc_ref, ref = call(lib.bqp_check_device, inst['n'], d)
        rc, got = call(lib.bqp_check_device_noalloc, inst['n'], d)
        assert rc_ref == 0 and rc == 0
        for f in FIELDS:
            assert getattr(got, f) == pytest.approx(getattr(ref, f), rel=1e-12, abs=1e-300), f
        assert got.verified == ref.verified


def test_noalloc_check_rejects_sizes_beyond_its_static_scratch():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    lib = boxqp.lib()
    dummy = torch.zeros(8, dtype=torch.float64, device='cuda')
    st = boxqp.Stats()
    p = dummy.data_ptr()
    rc = lib.bqp_check_device_noalloc(4194305, p, p, p, p, p, p, p, 1e-6, 0.0, 0, st)
    assert rc == 1
    assert b'4194304' in lib.bqp_box_last_error(None)
