"""GPU ADMM inner solve (C-ABI bqp_admm_*) against the CPU restatement of the reference's
inner CG (oracle/admm_pcg.py, qp_admm.cpp:153-161, 262-273).

Tolerances: K v to 1e-12 relative (summation order differs); the CG solve to 1e-9 relative in x
with the iteration count within max(3, 5 %) (the reference's long double dot products are not
reproduced, and CG amplifies rounding: near the stopping threshold a few iterations move); the final max|r| at or below the accuracy
when the solve converged."""
import numpy as np
import pytest

import boxqp
from boxqp.admm import AdmmSystem
from oracle.admm_pcg import AdmmSystemOracle

pytestmark = pytest.mark.gpu


def close_counts(a, b):
    return abs(a - b) <= max(3, int(0.05 * b))


def case(seed, n, m, per_row):
    """H: a planted graph Hessian; A: m sparse rows of per_row normal entries (some equality-like
    rows get rho x 100, as the reference's set-up does)."""
    inst = boxqp.planted('graph10k', seed=seed, n=n)
    rng = np.random.default_rng(seed)
    rowptr, col, val = [0], [], []
    for _ in range(m):
        cols = np.sort(rng.choice(n, size=per_row, replace=False))
        col.extend(cols.tolist())
        val.extend(rng.normal(size=per_row).tolist())
        rowptr.append(len(col))
    a = (np.array(rowptr, np.int32), np.array(col, np.int32), np.array(val))
    h = (inst['rowptr'], inst['col'], inst['val'])
    rho = np.where(rng.random(m) < 0.1, 10.0, 0.1)
    return h, a, rho, rng


@pytest.mark.parametrize('seed,n,m,per_row', [(1, 400, 150, 6), (2, 2000, 900, 12)])
def test_admm_inner_solve_matches_restatement(seed, n, m, per_row):
    h, a, rho, rng = case(seed, n, m, per_row)
    sigma = 1e-8
    gpu = AdmmSystem(*h, *a, n)
    ref = AdmmSystemOracle(h, a, n)
    gpu.set_rho(rho, sigma)
    ref.set_rho(rho, sigma)
    v = rng.normal(size=n)
    kv, kv_ref = gpu.apply(v), ref.apply(v)
    assert np.max(np.abs(kv - kv_ref)) <= 1e-12 * np.max(np.abs(kv_ref))
    rhs = rng.normal(size=n)
    x0 = rng.normal(size=n) * 0.1
    for accuracy in (1e-6, 1e-10):
        x, inner, resid = gpu.solve(rhs, x0, accuracy, 2 * n + 20)
        xr, inner_r, resid_r = ref.solve(rhs, x0, accuracy, 2 * n + 20)
        assert close_counts(inner, inner_r), (inner, inner_r)
        assert resid <= accuracy and resid_r <= accuracy
        assert np.max(np.abs(x - xr)) <= 1e-9 * max(1.0, np.max(np.abs(xr))) + 10 * accuracy
        # repeated solves are deterministic
        x2, inner2, resid2 = gpu.solve(rhs, x0, accuracy, 2 * n + 20)
        assert np.array_equal(x, x2) and inner2 == inner and resid2 == resid
    # the iteration cap and max_inner = 0
    x, inner, _ = gpu.solve(rhs, x0, 0.0, 3)
    xr, inner_r, _ = ref.solve(rhs, x0, 0.0, 3)
    assert inner == inner_r == 3 and np.max(np.abs(x - xr)) <= 1e-10 * max(1.0, np.max(np.abs(xr)))
    x, inner, _ = gpu.solve(rhs, x0, 1e-6, 0)
    assert inner == 0 and np.array_equal(x, x0)
    # a new rho rebuilds the preconditioner and the system
    rho2 = rho * 3.0
    gpu.set_rho(rho2, 1e-6)
    ref.set_rho(rho2, 1e-6)
    x, inner, resid = gpu.solve(rhs, x0, 1e-8, 2 * n + 20)
    xr, inner_r, _ = ref.solve(rhs, x0, 1e-8, 2 * n + 20)
    assert close_counts(inner, inner_r) and resid <= 1e-8
    gpu.close()


def test_admm_rejects_bad_input():
    h, a, rho, _ = case(3, 100, 20, 4)
    bad_col = (a[0], np.where(a[1] == a[1][0], 100, a[1]).astype(np.int32), a[2])
    with pytest.raises(ValueError):
        AdmmSystem(*h, *bad_col, 100)
    gpu = AdmmSystem(*h, *a, 100)
    with pytest.raises(ValueError):
        gpu.set_rho(np.zeros(20), 1e-8)
    gpu.close()


def test_gpu_inner_solve_inside_the_reference_admm_loop():
    """The restated ADMM loop of the reference (oracle/admm_pcg.py, pinned bit for bit to
    solve_qp_admm by tests/test_admm_oracle.py) with its x-update solved on the GPU reaches the
    reference's primal after the fixture's iterations to 1e-5 (each inner solve stops at the
    reference's accuracy, about 1e-7 relative, and rounds differently)."""
    from pathlib import Path
    from oracle.admm_pcg import solve_qp_admm_restated
    data = np.load(Path(__file__).resolve().parent / 'golden' / 'reference_admm.npz')
    names = sorted({k.split('.')[0] for k in data.files})
    for name in names:
        p = {k.split('.', 1)[1]: data[k] for k in data.files if k.startswith(name + '.')}
        n = int(p['n'])
        cache = {}

        def inner(system, rhs, x0, accuracy, max_inner):
            h, a, rho, sigma = system
            if 's' not in cache:
                cache['s'] = AdmmSystem(*h, *a, n)
                cache['s'].set_rho(rho, sigma)
            x, _, _ = cache['s'].solve(rhs, x0, accuracy, max_inner)
            return x

        x = solve_qp_admm_restated(n, p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'],
                                   p['a_rowptr'], p['a_col'], p['a_val'], p['row_lower'], p['row_upper'],
                                   int(p['iterations']), scaling=bool(p['scaling']), inner=inner)
        cache['s'].close()
        assert np.max(np.abs(x - p['x'])) <= 1e-5, (name, float(np.max(np.abs(x - p['x']))))


def test_device_admm_iterations_reach_the_reference_primal():
    """bqp_admm_iterate runs whole ADMM iterations of the reference's loop on the device (rhs, inner
    solve, relaxed z/y and x updates) from the reference's scaled set-up (restated by
    oracle/admm_pcg.py): the primal after the fixture's iterations matches the reference's
    solve_qp_admm to 1e-5, and iterations split over two calls give the same bits as one call."""
    from pathlib import Path
    from oracle.admm_pcg import scale_qp_admm
    data = np.load(Path(__file__).resolve().parent / 'golden' / 'reference_admm.npz')
    for name in sorted({k.split('.')[0] for k in data.files}):
        p = {k.split('.', 1)[1]: data[k] for k in data.files if k.startswith(name + '.')}
        n, its = int(p['n']), int(p['iterations'])
        sp = scale_qp_admm(n, p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], p['a_rowptr'],
                           p['a_col'], p['a_val'], p['row_lower'], p['row_upper'], bool(p['scaling']))
        s = AdmmSystem(*sp['h'], *sp['a'], n)
        s.set_rho(sp['rho'], sp['sigma'])
        x, z, y, inner = s.iterate(sp['c'], sp['lo'], sp['up'], sp['x'], sp['z'], sp['y'], 0, its)
        assert inner > 0
        assert np.max(np.abs(x * sp['variable'] - p['x'])) <= 1e-5, name
        k = its // 2
        x1, z1, y1, _ = s.iterate(sp['c'], sp['lo'], sp['up'], sp['x'], sp['z'], sp['y'], 0, k)
        x2, z2, y2, _ = s.iterate(sp['c'], sp['lo'], sp['up'], x1, z1, y1, k, its - k)
        assert np.array_equal(x2, x) and np.array_equal(z2, z) and np.array_equal(y2, y), name
        s.close()


def test_gpu_cg_stops_on_breakdown():
    """The device loop leaves at a non-positive d'K d as the reference does: x unchanged, no
    iteration counted, max|r| of the start returned."""
    n = 5
    h = (np.zeros(n + 1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    a = (np.zeros(3, np.int32), np.zeros(0, np.int32), np.zeros(0))
    s = AdmmSystem(*h, *a, n)
    s.set_rho(np.array([0.1, 0.1]), 0.0)
    x0 = np.arange(n, dtype=float)
    x, inner, resid = s.solve(np.ones(n), x0, 1e-9, 50)
    assert inner == 0 and np.array_equal(x, x0) and resid == 1.0
    s.close()
