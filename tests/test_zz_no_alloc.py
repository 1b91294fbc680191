"""bqp_check_device_noalloc: the device verification for callers that cannot allocate.

Some callers must not allocate device memory while they verify a solution -- a serving loop
where cudaMalloc/cudaFree would synchronize the device and stall the solves in flight, or a
process whose device memory another allocator has already reserved, where cudaMalloc fails.
This entry point takes its scratch from a static device array in the library instead.  The
test calls it through the C-ABI twice in a row, on two different problems, and compares each
result with the allocating entry point bqp_check_device on the same device arrays.

Further cases: the largest size the static scratch takes (n = 4,194,304 rows, the most blocks
of partials), a size beyond it (rejected with a message), and the entry point's first calls in
a fresh process under lazy module loading.

This file is collected last (tests/test_zz_*), so a run that stops at the first failure has
already run every other test.
"""
import os
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

import boxqp

ROOT = Path(__file__).resolve().parents[1]

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
        torch.cuda.synchronize()  # the arrays' copies are done before the checks read them
        rc_ref, ref = call(lib.bqp_check_device, inst['n'], d)
        rc, got = call(lib.bqp_check_device_noalloc, inst['n'], d)
        assert rc_ref == 0 and rc == 0
        for f in FIELDS:
            assert getattr(got, f) == pytest.approx(getattr(ref, f), rel=1e-12, abs=1e-300), f
        assert got.verified == ref.verified


def test_noalloc_check_at_its_largest_size():
    """n = 4,194,304, the limit: the launch uses the most blocks of partials the static array
    holds.  A diagonal Hessian keeps the arrays cheap; both entry points see the same device
    arrays and must agree."""
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    lib = boxqp.lib()
    n = 4194304
    rng = np.random.default_rng(9)
    diag = rng.uniform(0.5, 2.0, n)
    inst = {'rowptr': np.arange(n + 1, dtype=np.int32), 'col': np.arange(n, dtype=np.int32), 'val': diag,
            'c': rng.uniform(-1, 1, n), 'lower': np.full(n, -1.0), 'upper': np.full(n, 1.0)}
    x = np.clip(-inst['c'] / diag + 1e-7 * rng.standard_normal(n), -1.0, 1.0)
    d = device_arrays(torch, inst, x)
    torch.cuda.synchronize()
    for _ in range(2):
        rc_ref, ref = call(lib.bqp_check_device, n, d)
        rc, got = call(lib.bqp_check_device_noalloc, n, d)
        assert rc_ref == 0 and rc == 0
        for f in FIELDS:
            assert getattr(got, f) == pytest.approx(getattr(ref, f), rel=1e-12, abs=1e-300), f
        assert got.verified == ref.verified


def test_noalloc_check_first_calls_in_a_fresh_process_with_lazy_loading():
    """A fresh process with CUDA_MODULE_LOADING=LAZY: the set-up happens on the entry point's
    first call, and two calls in a row still equal the allocating check."""
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    script = textwrap.dedent('''
        import sys
        sys.path[:0] = [sys.argv[1], sys.argv[1] + '/hypergrey-sih-26_gb300', sys.argv[1] + '/tests']
        import numpy as np
        import torch
        import boxqp
        from test_zz_no_alloc import FIELDS, call, device_arrays
        lib = boxqp.lib()
        inst = boxqp.planted('graph10k', seed=41, n=5000)
        d = device_arrays(torch, inst, inst['xstar'])
        torch.cuda.synchronize()
        got = [call(lib.bqp_check_device_noalloc, inst['n'], d) for _ in range(2)]
        rc_ref, ref = call(lib.bqp_check_device, inst['n'], d)
        assert rc_ref == 0 and all(rc == 0 for rc, _ in got), (rc_ref, [rc for rc, _ in got])
        for _, st in got:
            for f in FIELDS:
                a, b = getattr(st, f), getattr(ref, f)
                assert abs(a - b) <= 1e-12 * abs(b) + 1e-300, (f, a, b)
            assert st.verified == ref.verified == 1
        print('fresh-process ok')
    ''')
    env = dict(os.environ, CUDA_MODULE_LOADING='LAZY')
    proc = subprocess.run([sys.executable, '-c', script, str(ROOT)], capture_output=True, text=True, env=env,
                          timeout=300)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    assert 'fresh-process ok' in proc.stdout


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
