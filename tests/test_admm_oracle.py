"""The CPU restatement of the reference's ADMM inner solve (oracle/admm_pcg.py), without a GPU:
its system matrix equals H + sigma I + A' diag(rho) A formed densely, and its CG reaches the
requested residual."""
import numpy as np

from oracle.admm_pcg import AdmmSystemOracle


def random_case(seed, n=60, m=40, density=0.1):
    rng = np.random.default_rng(seed)
    # H: a symmetric diagonally dominant graph Laplacian plus a diagonal
    dense_h = np.zeros((n, n))
    for _ in range(3 * n):
        i, j = rng.integers(0, n, 2)
        if i != j:
            w = rng.uniform(0.1, 1.0)
            dense_h[i, j] -= w
            dense_h[j, i] -= w
            dense_h[i, i] += w
            dense_h[j, j] += w
    dense_h += np.diag(rng.uniform(0.0, 1.0, n))
    dense_a = np.where(rng.random((m, n)) < density, rng.normal(size=(m, n)), 0.0)

    def csr(dense):
        rowptr, col, val = [0], [], []
        for row in dense:
            nz = np.nonzero(row)[0]
            col.extend(nz.tolist())
            val.extend(row[nz].tolist())
            rowptr.append(len(col))
        return np.array(rowptr, np.int32), np.array(col, np.int32), np.array(val)

    return dense_h, dense_a, csr(dense_h), csr(dense_a), rng


def test_restated_system_and_cg():
    dense_h, dense_a, h, a, rng = random_case(3)
    n, m = dense_h.shape[0], dense_a.shape[0]
    rho = np.where(rng.random(m) < 0.2, 10.0, 0.1)
    sigma = 1e-8
    o = AdmmSystemOracle(h, a, n)
    o.set_rho(rho, sigma)
    k = dense_h + sigma * np.eye(n) + dense_a.T @ np.diag(rho) @ dense_a
    v = rng.normal(size=n)
    assert np.allclose(o.apply(v), k @ v, rtol=1e-12, atol=1e-12)
    assert np.allclose(o.precond, np.diag(k), rtol=1e-13, atol=0)
    rhs = rng.normal(size=n)
    x, inner, resid = o.solve(rhs, np.zeros(n), 1e-10, 2 * n + 20)
    assert resid <= 1e-10 and 0 < inner <= 2 * n + 20
    assert np.allclose(x, np.linalg.solve(k, rhs), rtol=1e-8, atol=1e-8)
    x0, inner0, _ = o.solve(rhs, np.ones(n), 1e-10, 0)
    assert inner0 == 0 and np.array_equal(x0, np.ones(n))


def _golden_admm(file='reference_admm.npz'):
    from pathlib import Path
    data = np.load(Path(__file__).resolve().parent / 'golden' / file)
    names = sorted({k.split('.')[0] for k in data.files})
    return [(name, {k.split('.', 1)[1]: data[k] for k in data.files if k.startswith(name + '.')}) for name in names]


def test_restated_admm_loop_matches_reference_golden():
    """The restated ADMM loop (scaling, x-update by the restated inner CG, relaxed z/y updates)
    reproduces the reference's solve_qp_admm primal after a few iterations (fixture made by
    tests/golden/make_golden.py from the reference itself): bit for bit where numpy's long double
    is the x87 80-bit type the reference's dot products use, else to 1e-12."""
    from oracle.admm_pcg import solve_qp_admm_restated
    exact = np.finfo(np.longdouble).nmant == 63
    for name, p in _golden_admm():
        x = solve_qp_admm_restated(int(p['n']), p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'],
                                   p['a_rowptr'], p['a_col'], p['a_val'], p['row_lower'], p['row_upper'],
                                   int(p['iterations']), scaling=bool(p['scaling']))
        if exact:
            assert np.array_equal(x, p['x']), name
        else:
            assert np.max(np.abs(x - p['x'])) <= 1e-12, name


def test_restated_admm_loop_with_rho_adaptation_matches_reference_golden():
    """120-230 iterations, across the reference's rho adaptation at iterations 100 and 200
    (qp_admm.cpp:265-271: residual-balanced rho_base, a new rho and preconditioner when it moves
    by more than 5x): the restated loop reproduces solve_qp_admm's primal as above, and the
    adaptation changes rho_base at least once in every case."""
    from oracle.admm_pcg import solve_qp_admm_restated
    exact = np.finfo(np.longdouble).nmant == 63
    for name, p in _golden_admm('reference_admm_adapt.npz'):
        info = {}
        x = solve_qp_admm_restated(int(p['n']), p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'],
                                   p['a_rowptr'], p['a_col'], p['a_val'], p['row_lower'], p['row_upper'],
                                   int(p['iterations']), scaling=bool(p['scaling']), info=info)
        assert info['rho_base'][0] != 0.1, name
        if exact:
            assert np.array_equal(x, p['x']), name
        else:
            assert np.max(np.abs(x - p['x'])) <= 1e-12, name


def test_restated_rho_adaptation_rule():
    """adapt_rho keeps rho_base while the balanced candidate stays within a factor 5 and clamps it
    to [1e-6, 1e6]: a case with Ax = z (no primal residual) drives it to the floor."""
    from oracle.admm_pcg import AdmmSystemOracle, adapt_rho
    n = 3
    h = (np.array([0, 1, 2, 3], np.int32), np.array([0, 1, 2], np.int32), np.array([1.0, 1.0, 1.0]))
    a = (np.array([0, 1, 2, 3], np.int32), np.array([0, 1, 2], np.int32), np.array([1.0, 1.0, 1.0]))
    system = AdmmSystemOracle(h, a, n)
    x = np.array([0.5, -0.25, 0.125])
    sp = {'a': a, 'h': h, 'c': np.array([1.0, 0.0, -1.0])}
    # primal 0 -> sqrt(1e-16 / dual) * rho_base is far below rho_base / 5
    assert adapt_rho(sp, system, x, x.copy(), np.zeros(n), 0.1) == max(1e-6, 0.1 * np.sqrt(1e-16 / (1.5 / 2.0)))
    # primal and dual residuals balanced: rho_base stays
    z = x + np.array([1.5, 0.0, 0.0])
    assert adapt_rho(sp, system, x, z, np.zeros(n), 0.1) == 0.1


def test_restated_cg_stops_on_breakdown():
    """A zero system (H = 0, A = 0, sigma = 0) breaks down at once: d'K d is not positive, the
    reference leaves the CG loop before any update (qp_admm.cpp:264)."""
    n = 5
    h = (np.zeros(n + 1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    a = (np.zeros(3, np.int32), np.zeros(0, np.int32), np.zeros(0))
    o = AdmmSystemOracle(h, a, n)
    with np.errstate(divide='ignore', invalid='ignore'):
        o.set_rho(np.array([0.1, 0.1]), 0.0)
        x0 = np.arange(n, dtype=float)
        x, inner, resid = o.solve(np.ones(n), x0, 1e-9, 50)
    assert inner == 0 and np.array_equal(x, x0) and resid == 1.0


def test_restated_admm_with_kkt_polish_matches_reference_golden():
    """The whole restated solve_qp_admm (checks every 25 iterations, rho adaptation, and the KKT
    polish in its diagonal-Hessian form, qp_admm.cpp:165-205) on diagonal-Hessian QPs whose ADMM
    does not verify by iteration 250: the polish at 250 verifies, and status, iteration count,
    primal and row duals equal the reference's (tests/golden/reference_admm_polish.npz)."""
    from oracle.admm_pcg import solve_qp_admm_full_restated
    exact = np.finfo(np.longdouble).nmant == 63
    for name, p in _golden_admm('reference_admm_polish.npz'):
        status, iterations, x, y, chk, polished = solve_qp_admm_full_restated(
            int(p['n']), p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], p['a_rowptr'],
            p['a_col'], p['a_val'], p['row_lower'], p['row_upper'], float(p['tol']))
        assert status == str(p['status']) == 'optimal' and iterations == int(p['iterations']) == 250, name
        assert polished, name
        if exact:
            assert np.array_equal(x, p['x']) and np.array_equal(y, p['row_dual']), name
        else:
            assert np.max(np.abs(x - p['x'])) <= 1e-12, name
