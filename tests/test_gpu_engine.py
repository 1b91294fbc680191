"""GPU engine parity against the CPU oracle and the reference's golden results (needs a GPU).

Tolerances (the bar for floating point):
  * BQP_PRECISION_FP64_EXACT: bit-identical iterates, statuses and iteration counts.
  * BQP_PRECISION_FP64 (FMA, multiply by 1/L): same status, iterations within one check
    interval, objective relative difference <= 1e-10, primal max difference <= 1e-6.
  * BQP_PRECISION_MIXED: verified at the requested KKT tolerance by the FP64 oracle checker on
    the host, objective relative error vs the planted optimum <= 1e-7, active set identical to
    the planted one wherever the planted dual margin exceeds 1e-6.
"""
import hashlib

import numpy as np
import pytest

import boxqp
from oracle import oracle as O
from golden_cases import args, inputs

pytestmark = pytest.mark.gpu


def digest(x):
    return hashlib.sha256(np.ascontiguousarray(x, np.float64).tobytes()).hexdigest()


def solve(engine, inst, precision, tol, iteration_limit=200000, time_limit=60.0):
    o = boxqp.options_struct(tol, time_limit, iteration_limit, precision)
    return engine.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)


def planted_args(inst):
    return inst['hrow'], inst['hcol'], inst['hval'], inst['c'], inst['lower'], inst['upper']


def active_set_ok(inst, x, margin=1e-6):
    z = inst['z']
    at_lo = z > margin
    at_up = z < -margin
    return (np.all(x[at_lo] == inst['lower'][at_lo]) and np.all(x[at_up] == inst['upper'][at_up]) and
            np.all((x[~(at_lo | at_up)] > inst['lower'][~(at_lo | at_up)]) &
                   (x[~(at_lo | at_up)] < inst['upper'][~(at_lo | at_up)])))


@pytest.mark.parametrize('name', ['graph2k_s100', 'graph2k_s103', 'graph2k_tol1e-8', 'graph2k_limit60',
                                  'graph2k_limit0', 'tridiagonal_1000', 'grid32_tol1e-08', 'batch_i0',
                                  'graph10k_s0', 'graph2k_open', 'grid32_open', 'graph2k_fixed',
                                  'graph2k_zero_rows', 'single_var'] + [f'kkt5_{i:02d}' for i in range(15)])
def test_exact_mode_reproduces_reference_bits(engine, golden, name):
    d, xs = golden
    rec = next(c for c in d['cases'] if c['name'] == name)
    p, inst = inputs(rec)
    if inst is None:  # a stored problem (the reference's own test problems): through the mirrored API
        q = boxqp.QuadraticProblem(cost=p['cost'], lower=p['lower'], upper=p['upper'], hessian_row=p['hrow'],
                                   hessian_col=p['hcol'], hessian_val=p['hval'], maximize=rec['maximize'],
                                   offset=rec['offset'])
        r = boxqp.solve_accelerated_box(q, boxqp.QpOptions(tolerance=rec['tol'], precision='fp64_exact',
                                                           iteration_limit=rec['iteration_limit'], time_limit=600.0),
                                        engine=engine)
        status, iterations, x, objective = r.status, r.iterations, r.primal, r.objective
    else:
        x, st = solve(engine, inst, 'fp64_exact', rec['tol'], rec['iteration_limit'], 600.0)
        status, iterations, objective = boxqp.STATUS_NAMES[st.status], st.iterations, st.objective
    assert status == rec['status']
    assert iterations == rec['iterations']
    assert digest(x) == rec['x_sha256']
    if name in xs:
        assert np.array_equal(x, xs[name])
    assert objective == pytest.approx(rec['objective'], rel=1e-13, abs=1e-13)


@pytest.mark.parametrize('name', ['v2_psd_300', 'two_var', 'two_var_maximize'])
def test_reference_api_known_answers(engine, golden, name):
    """The reference's own test problems through the mirrored solve_accelerated_box."""
    d, xs = golden
    rec = next(c for c in d['cases'] if c['name'] == name)
    p, _ = inputs(rec)
    q = boxqp.QuadraticProblem(cost=p['cost'], lower=p['lower'], upper=p['upper'], hessian_row=p['hrow'],
                               hessian_col=p['hcol'], hessian_val=p['hval'], maximize=rec['maximize'],
                               offset=rec['offset'])
    r = boxqp.solve_accelerated_box(q, boxqp.QpOptions(tolerance=rec['tol'], precision='fp64_exact'), engine=engine)
    assert r.status == rec['status'] and r.optimality_verified
    assert r.iterations == rec['iterations']
    assert r.objective == pytest.approx(rec['objective'], rel=1e-12, abs=1e-12)
    assert np.array_equal(r.primal, xs[name])


@pytest.mark.parametrize('seed', [0, 1])
def test_fp64_mode_matches_oracle(engine, seed):
    inst = boxqp.planted('graph10k', seed=seed, lower_triplets=True)
    status, xo, so = O.solve_box(*planted_args(inst), tol=1e-6, threads=8)
    x, st = solve(engine, inst, 'fp64', 1e-6)
    assert boxqp.STATUS_NAMES[st.status] == status == 'optimal'
    assert abs(st.iterations - so['iterations']) <= 25
    assert st.objective == pytest.approx(so['objective'], rel=1e-10)
    assert np.max(np.abs(x - xo)) <= 1e-6
    chk = O.check(*planted_args(inst), x, tol=1e-6)
    assert chk['verified'] == 1.0


@pytest.mark.parametrize('preset,n,seed,tol', [('graph10k', 0, 3, 1e-6), ('graph10k', 0, 4, 1e-8),
                                               ('grid', 64 * 64, 2, 1e-6), ('grid', 64 * 64, 2, 1e-8),
                                               ('graph1m', 50000, 1, 1e-6), ('batch', 0, 3, 1e-6)])
def test_mixed_mode_meets_tolerance_against_fp64_oracle(engine, preset, n, seed, tol):
    inst = boxqp.planted(preset, seed=seed, n=n, lower_triplets=True)
    x, st = solve(engine, inst, 'mixed', tol)
    assert boxqp.STATUS_NAMES[st.status] == 'optimal', st.as_dict()
    chk = O.check(*planted_args(inst), x, tol=tol)
    assert chk['verified'] == 1.0, chk
    assert chk['stationarity_residual'] <= tol
    assert abs(chk['objective'] - inst['fstar']) / (1 + abs(inst['fstar'])) <= 1e-7
    assert st.objective == pytest.approx(chk['objective'], rel=1e-12)
    assert active_set_ok(inst, x)


def test_plugin_box_iteration_reproduces_cpu_loop(golden):
    """make_cuda_box + the reference's host loop == the CPU branch, iterate for iterate."""
    inst = boxqp.planted('graph10k', seed=21, n=3000, lower_triplets=True)
    L = boxqp.gershgorin(inst['rowptr'], inst['val'])
    box = boxqp.make_cuda_box(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], L)
    x = np.maximum(inst['lower'], np.minimum(inst['upper'], 0.0))
    w = x.copy()
    t = 1.0
    for k in range(4):
        # 25 iterations on each side, then compare the primal as the reference's check would
        tt = t
        for _ in range(25):
            nt = (1 + np.sqrt(1 + 4 * tt * tt)) / 2
            beta = (tt - 1) / nt
            tt = nt
            box.step(beta)
        t = O.fista_steps(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], L, x,
                          w, t, 25)
        assert t == tt
        assert np.array_equal(box.primal(), x)
    box.close()


def test_batch_results_equal_solo_results(engine):
    """Each solve is bit-identical alone and inside a batch of unequal solves."""
    insts = [boxqp.planted('batch', seed=3, index=i) for i in range(12)]
    solo = []
    for inst in insts:
        x, st = solve(engine, inst, 'mixed', 1e-6)
        solo.append((x, st.iterations, st.objective))
    ids = []
    for inst in insts:
        o = boxqp.options_struct(1e-6, 60.0, 200000, 'mixed')
        ids.append(engine.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o))
    for inst, ident, (xs, its, obj) in zip(insts, ids, solo):
        assert engine.wait(ident, 120.0)
        x, st = engine.fetch(ident, inst['n'])
        engine.release(ident)
        assert boxqp.STATUS_NAMES[st.status] == 'optimal'
        assert np.array_equal(x, xs) and st.iterations == its and st.objective == obj


def test_resolve_resident_is_reproducible(engine):
    inst = boxqp.planted('graph10k', seed=8, n=20000)
    o = boxqp.options_struct(1e-6, 60.0, 200000, 'mixed')
    ident = engine.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
    assert engine.wait(ident, 120.0)
    x1, s1 = engine.fetch(ident, inst['n'])
    engine.resolve([ident])
    assert engine.wait(ident, 120.0)
    x2, s2 = engine.fetch(ident, inst['n'])
    engine.release(ident)
    assert np.array_equal(x1, x2) and s1.iterations == s2.iterations
    assert s2.device_end_ns > s2.device_start_ns > 0


def test_iteration_and_time_limits(engine):
    inst = boxqp.planted('grid', seed=2, n=128 * 128)
    x, st = solve(engine, inst, 'fp64', 1e-12, iteration_limit=37)
    assert boxqp.STATUS_NAMES[st.status] == 'iteration_limit' and st.iterations == 37
    big = boxqp.planted('graph1m', seed=3, n=300000)
    x, st = solve(engine, big, 'fp64', 1e-300, iteration_limit=10 ** 9, time_limit=0.05)
    assert boxqp.STATUS_NAMES[st.status] == 'time_limit'
    assert 0.05 <= st.device_seconds < 5.0
    assert np.all(np.isfinite(x))


def test_check_device_matches_oracle_checker():
    torch = pytest.importorskip('torch')
    inst = boxqp.planted('graph10k', seed=9, n=5000, lower_triplets=True)
    rng = np.random.default_rng(2)
    x = np.clip(inst['xstar'] + 1e-5 * rng.standard_normal(inst['n']), inst['lower'], inst['upper'])
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
           [('rowptr', inst['rowptr']), ('col', inst['col']), ('val', inst['val']), ('x', x), ('c', inst['c']),
            ('l', inst['lower']), ('u', inst['upper'])]}
    st = boxqp.Stats()
    rc = boxqp.lib().bqp_check_device(inst['n'], dev['rowptr'].data_ptr(), dev['col'].data_ptr(),
                                      dev['val'].data_ptr(), dev['x'].data_ptr(), dev['c'].data_ptr(),
                                      dev['l'].data_ptr(), dev['u'].data_ptr(), 1e-6, 0.0, 0, st)
    assert rc == 0
    ref = O.check(*planted_args(inst), x, tol=1e-6)
    assert st.objective == pytest.approx(ref['objective'], rel=1e-13)
    assert st.stationarity_residual == pytest.approx(ref['stationarity_residual'], rel=1e-9)
    assert st.primal_residual == pytest.approx(ref['primal_residual'], abs=1e-15)
    assert st.dual_bound == pytest.approx(ref['dual_bound'], rel=1e-12)
    assert bool(st.verified) == bool(ref['verified'])


def _gate_expected(rowptr, col, val):
    """Per-row restatement of bqp_gate_device's contract: FP64 sums in column order."""
    n = rowptr.shape[0] - 1
    lip, indefinite, nondominant = 0.0, 0, 0
    diag = np.zeros(n)
    for r in range(n):
        a, b = int(rowptr[r]), int(rowptr[r + 1])
        total, radius, d, nd = 0.0, 0.0, 0.0, 0
        for k in range(a, b):
            v = float(val[k])
            total += abs(v)
            if col[k] == r:
                d = v if nd == 0 else (0.0 + d if nd == 1 else d) + v
                nd += 1
            else:
                radius += abs(v)
        lip = max(lip, total)
        if d < 0 or (d == 0 and radius > 0):
            indefinite = 1
        if d < radius:
            nondominant = 1
        diag[r] = d
    return lip, indefinite, nondominant, diag


def _rows_to_csr(rows):
    rowptr = np.zeros(len(rows) + 1, np.int32)
    rowptr[1:] = np.cumsum([len(c) for c, _ in rows])
    col = np.concatenate([np.asarray(c, np.int32) for c, _ in rows])
    val = np.concatenate([np.asarray(v, np.float64) for _, v in rows])
    return rowptr, col, val


def _gate_rows(rng, n, degree, mode, long_rows=()):
    """Rows with random off-diagonal values (not FP32-representable, so the FP32 bracket of the
    radius has width); the diagonal is the FP64 column-order radius itself ('equal': every row
    falls inside the bracket and sums again in FP64), one unit below it in one row ('below'), or
    the radius plus a clear margin ('margin')."""
    rows = []
    for r in range(n):
        m = int(long_rows[r]) if r < len(long_rows) else int(rng.integers(1, 2 * degree))
        cols = np.unique(rng.integers(0, n, m))
        cols = cols[cols != r]
        vals = rng.uniform(-1.0, 1.0, cols.shape[0]) * 10.0 ** rng.integers(-3, 3)
        radius = 0.0
        for v in vals:
            radius += abs(float(v))
        d = radius + (0.5 if mode == 'margin' else 0.0)
        cols = np.append(cols, r)
        vals = np.append(vals, d)
        order = np.argsort(cols, kind='stable')
        rows.append((cols[order], vals[order]))
    if mode == 'below':
        cols, vals = rows[n // 2]
        k = int(np.nonzero(cols == n // 2)[0][0])
        vals[k] = np.nextafter(vals[k], 0.0)
    return rows


def test_gate_device_matches_the_row_restatement():
    """bqp_gate_device (the engine's admission pass on caller arrays): the Gershgorin bound bit for
    bit against bqp_gershgorin, the dominance and indefiniteness flags and the stored diagonal
    against a per-row FP64 restatement, on rows whose diagonal equals the FP64 radius (the FP32
    bracket cannot decide them), one unit below it, with a margin, with negative or zero
    diagonals, with duplicate diagonal entries, and with rows longer than a staging window."""
    torch = pytest.importorskip('torch')
    from ctypes import byref, c_double, c_int32
    rng = np.random.default_rng(7)
    cases = {}
    for mode in ('equal', 'below', 'margin'):
        cases[mode] = _rows_to_csr(_gate_rows(rng, 3000, 8, mode))
        cases[mode + '_long'] = _rows_to_csr(_gate_rows(rng, 3000, 8, mode, long_rows=[2500, 900, 30] * 3))
    rows = _gate_rows(rng, 500, 6, 'margin')
    c0, v0 = rows[7]
    v0 = v0.copy()
    v0[np.nonzero(c0 == 7)[0][0]] = -1.0
    cases['negative'] = _rows_to_csr(rows[:7] + [(c0, v0)] + rows[8:])
    rows = _gate_rows(rng, 500, 6, 'margin')
    c1, v1 = rows[11]
    v1 = v1.copy()
    v1[np.nonzero(c1 == 11)[0][0]] = 0.0
    cases['zero_diagonal'] = _rows_to_csr(rows[:11] + [(c1, v1)] + rows[12:])
    rows = _gate_rows(rng, 500, 6, 'margin')
    rows[3] = (np.array([], np.int32), np.array([]))  # an empty row
    c2, v2 = rows[5]
    k = int(np.nonzero(c2 == 5)[0][0])
    rows[5] = (np.insert(c2, k, 5), np.insert(v2, k, [-0.25]))  # two diagonal entries in one row
    cases['duplicates_empty'] = _rows_to_csr(rows)
    lib = boxqp.lib()
    for name, (rowptr, col, val) in cases.items():
        n = rowptr.shape[0] - 1
        d = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (rowptr, col, val)]
        diag = torch.zeros(n, dtype=torch.float64, device='cuda')
        torch.cuda.synchronize()
        lip, ind, nond = c_double(), c_int32(), c_int32()
        rc = lib.bqp_gate_device(n, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), diag.data_ptr(),
                                 byref(lip), byref(ind), byref(nond))
        assert rc == 0, name
        want_lip, want_ind, want_nond, want_diag = _gate_expected(rowptr, col, val)
        assert lip.value == boxqp.gershgorin(rowptr, val) == want_lip, name
        assert (ind.value, nond.value) == (want_ind, want_nond), name
        assert np.array_equal(diag.cpu().numpy(), want_diag), name
    assert _gate_expected(*cases['equal'])[2] == 0 and _gate_expected(*cases['below'])[2] == 1
    assert _gate_expected(*cases['negative'])[1] == 1 and _gate_expected(*cases['zero_diagonal'])[1] == 1


def test_hessian_entries_are_checked_by_the_admission_pass(engine):
    """The submission scans rows, costs and bounds on the host (errors at once); the Hessian's
    entries are checked by the device's admission pass, which reports, in the reference's order
    (src/accelerated_qp.cpp:14-28), an entry out of range or not finite as invalid_argument
    ('Invalid Hessian'), a non-convex Hessian as unsupported_curvature and a zero Hessian as the
    CPU LP path's error, through bqp_wait / bqp_fetch; the context keeps serving afterwards."""
    inst = boxqp.planted('graph10k', seed=4, n=3000)
    base = [np.array(a, copy=True) for a in (inst['rowptr'], inst['col'], inst['val'], inst['c'],
                                             inst['lower'], inst['upper'])]
    o = boxqp.options_struct(1e-6, 60.0, 200000, 'mixed')
    x_ok, st_ok = engine.solve(*base, o)
    assert boxqp.STATUS_NAMES[st_ok.status] == 'optimal'

    def variant(**change):
        a = [np.array(v, copy=True) for v in base]
        names = ['rowptr', 'col', 'val', 'c', 'lower', 'upper']
        for k, f in change.items():
            f(a[names.index(k)])
        return a

    out_of_range = variant(col=lambda c: c.__setitem__(17, base[0].shape[0] - 1))
    not_finite = variant(val=lambda v: v.__setitem__(123, np.nan))
    zero = variant(val=lambda v: v.__setitem__(slice(None), 0.0))
    for a, exc, match in ((out_of_range, ValueError, 'Invalid Hessian'), (not_finite, ValueError, 'Invalid Hessian'),
                          (zero, boxqp.EngineError, 'Zero-Hessian')):
        with pytest.raises(exc, match=match):
            engine.solve(*a, o)
        for copy in (True, False):
            ident = engine.submit(*a, o, copy=copy)
            with pytest.raises(exc, match=match):
                engine.wait(ident, 60.0)
            engine.release(ident)
    # host checks still come at submission, before the entries
    bad_cost = variant(c=lambda c: c.__setitem__(3, np.inf), col=lambda c: c.__setitem__(17, -5))
    with pytest.raises(ValueError, match='coefficient or bound'):
        engine.submit(*bad_cost, o)
    # infeasible bounds finish at submission: the entries are checked on the host there
    infeasible_bad = variant(lower=lambda l: l.__setitem__(0, 5.0), val=lambda v: v.__setitem__(9, np.inf))
    with pytest.raises(ValueError, match='Invalid Hessian'):
        engine.submit(*infeasible_bad, o)
    infeasible_zero = variant(lower=lambda l: l.__setitem__(0, 5.0), val=lambda v: v.__setitem__(slice(None), 0.0))
    with pytest.raises(boxqp.EngineError, match='Zero-Hessian'):
        engine.submit(*infeasible_zero, o)
    x, st = engine.solve(*base, o)
    assert np.array_equal(x, x_ok) and st.iterations == st_ok.iterations


def test_diagonal_hessian_takes_the_separable_bound(engine):
    """A diagonal Hessian with a positive diagonal (explicit zero off-diagonal entries allowed, as
    check_qp_solution's positive_diagonal test counts nonzero values only) is recognised by the
    admission pass: its dual bound is the separable one, tight at the optimum (relative gap
    ~0), and equal to the oracle checker's."""
    rng = np.random.default_rng(5)
    n = 5000
    d = rng.uniform(0.5, 3.0, n)
    rows = []
    for r in range(n):
        cols, vals = [r], [d[r]]
        if r % 7 == 0 and r + 1 < n:
            cols.append(r + 1)
            vals.append(0.0)  # an explicit zero off the diagonal
        rows.append((np.array(cols), np.array(vals)))
    rowptr, col, val = _rows_to_csr(rows)
    c = rng.standard_normal(n)
    lo, up = -np.ones(n), np.ones(n)
    o = boxqp.options_struct(1e-9, 60.0, 200000, 'fp64')
    x, st = engine.solve(rowptr, col, val, c, lo, up, o)
    assert boxqp.STATUS_NAMES[st.status] == 'optimal'
    hrow = np.arange(n, dtype=np.int64)
    ref = O.check(hrow, hrow, d, c, lo, up, x, tol=1e-9)
    assert st.dual_bound == pytest.approx(ref['dual_bound'], rel=1e-12)
    assert st.relative_gap <= 1e-9


def test_device_name():
    assert 'GB300' in boxqp.cuda_device_name() or len(boxqp.cuda_device_name()) > 0


def _lambda_max(inst, scaled):
    """Largest eigenvalue of Q (or of V Q V, V = diag(Q)^-1/2) by scipy's Lanczos, on the CPU."""
    sp = pytest.importorskip('scipy.sparse')
    la = pytest.importorskip('scipy.sparse.linalg')
    n = inst['n']
    q = sp.csr_matrix((inst['val'], inst['col'], inst['rowptr']), shape=(n, n))
    if scaled:
        v = 1.0 / np.sqrt(q.diagonal())
        q = sp.diags(v) @ q @ sp.diags(v)
    return float(la.eigsh(q, k=1, which='LA', tol=1e-10, return_eigenvectors=False)[0])


@pytest.mark.parametrize('precision', ['fp64', 'fp64_exact', 'mixed'])
def test_power_lipschitz_estimate(engine, precision):
    """BQP_LIPSCHITZ_POWER: the device estimate lies between lambda_max (scipy Lanczos) and the
    Gershgorin bound, the solve verifies with no more iterations than under Gershgorin, and it is
    deterministic."""
    inst = boxqp.planted('graph10k', seed=21)
    a = (inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'])
    og = boxqp.options_struct(1e-7, 60.0, 200000, precision)
    op = boxqp.options_struct(1e-7, 60.0, 200000, precision, lipschitz='power')
    xg, sg = engine.solve(*a, og)
    xp, sp_ = engine.solve(*a, op)
    xp2, _ = engine.solve(*a, op)
    assert boxqp.STATUS_NAMES[sg.status] == 'optimal' and boxqp.STATUS_NAMES[sp_.status] == 'optimal'
    assert np.array_equal(xp, xp2)
    lam = _lambda_max(inst, scaled=precision == 'mixed')
    gersh = boxqp.gershgorin(inst['rowptr'], inst['val'])
    assert lam * (1 - 1e-9) <= sp_.lipschitz <= (gersh if precision != 'mixed' else 2.0 * gersh)
    if precision != 'mixed':
        assert sp_.lipschitz < sg.lipschitz == gersh
        assert sp_.iterations <= sg.iterations
    chk = O.check(*planted_args(boxqp.planted('graph10k', seed=21, lower_triplets=True)), xp, tol=1e-7)
    assert chk['verified']
    assert abs(sp_.objective - sg.objective) <= 1e-9 * max(1.0, abs(sg.objective))


@pytest.mark.parametrize('scaling', [1, 2])
@pytest.mark.parametrize('preset,n,seed', [('graph10k', 0, 5), ('graph1m', 40000, 2), ('tridiagonal', 5000, 1)])
def test_mixed_mode_with_and_without_preconditioned_steps(engine, preset, n, seed, scaling):
    """scaling = 1: per-row steps 1/(L' Q_ii) (the default); 2: the scalar step 1/L.  Both verify
    and land on the planted optimum and active set."""
    inst = boxqp.planted(preset, seed=seed, n=n, lower_triplets=True)
    o = boxqp.options_struct(1e-7, 30.0, 200000, 'mixed', scaling=scaling)
    x, st = engine.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
    assert boxqp.STATUS_NAMES[st.status] == 'optimal', st.as_dict()
    chk = O.check(*planted_args(inst), x, tol=1e-7)
    assert chk['verified'] == 1.0, chk
    assert abs(chk['objective'] - inst['fstar']) / (1 + abs(inst['fstar'])) <= 1e-7
    assert active_set_ok(inst, x)


def test_polish_chains_on_the_tridiagonal_family(engine):
    """The polish's chain preconditioner (Q_FF's tridiagonal part solved along runs of free rows)
    on the reference's tridiagonal family, every variable free: verified by the oracle at 1e-7, on
    the planted optimum, in a handful of CG iterations (Jacobi rows alone need about 78)."""
    inst = boxqp.planted('tridiagonal', seed=3, n=200000, lower_triplets=True)
    o = boxqp.options_struct(1e-7, 30.0, 20000, 'mixed')
    x, st = engine.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
    assert boxqp.STATUS_NAMES[st.status] == 'optimal', st.as_dict()
    chk = O.check(*planted_args(inst), x, tol=1e-7)
    assert chk['verified'] == 1.0, chk
    assert abs(chk['objective'] - inst['fstar']) / (1 + abs(inst['fstar'])) <= 1e-7
    assert 0 < st.polish_iterations <= 12, st.polish_iterations


def test_polish_chains_drop_couplings_that_break_strict_dominance(engine):
    """Rows whose diagonal only equals their off-diagonal sum (weakly dominant: 2 = |-1| + |-1|)
    lose their couplings in the preconditioner, which stays positive definite; the solve still
    verifies against the oracle."""
    inst = boxqp.planted('tridiagonal', seed=5, n=20000, lower_triplets=True)
    rowptr, col, val = inst['rowptr'], inst['col'], inst['val'].copy()
    hrow, hcol, hval = inst['hrow'], inst['hcol'], inst['hval'].copy()
    weak = np.arange(inst['n']) % 3 == 1
    for r in np.nonzero(weak)[0]:
        k = rowptr[r] + np.nonzero(col[rowptr[r]:rowptr[r + 1]] == r)[0][0]
        val[k] = 2.0
    hval[(hrow == hcol) & weak[hrow]] = 2.0
    o = boxqp.options_struct(1e-7, 30.0, 20000, 'mixed')
    x, st = engine.solve(rowptr, col, val, inst['c'], inst['lower'], inst['upper'], o)
    assert boxqp.STATUS_NAMES[st.status] == 'optimal', st.as_dict()
    chk = O.check(hrow, hcol, hval, inst['c'], inst['lower'], inst['upper'], x, tol=1e-7)
    assert chk['verified'] == 1.0, chk


def test_polish_chains_with_marginal_pivots_and_tiny_couplings(engine):
    """The chain preconditioner runs in FP32: couplings below FP32's range (1e-50) end a chain
    where they stand, and rows dominant in FP64 by only 1e-9 (Q_ii = 2 + 1e-9 beside two couplings
    of -1, below the pivot guard's 2^-20 margin in FP32) cut or drop their chain; the solve still
    verifies against the oracle."""
    inst = boxqp.planted('tridiagonal', seed=6, n=20000, lower_triplets=True)
    rowptr, col, val = inst['rowptr'], inst['col'], inst['val'].copy()
    hrow, hcol, hval = inst['hrow'], inst['hcol'], inst['hval'].copy()
    n = inst['n']
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    tiny = np.arange(n) % 5 == 2  # the coupling of row r to row r + 1
    lo_end, hi_end = np.minimum(rows, col), np.maximum(rows, col)
    val[(hi_end == lo_end + 1) & tiny[lo_end]] = -1e-50
    hval[(hrow == hcol + 1) & tiny[hcol]] = -1e-50
    marginal = np.arange(n) % 7 == 3
    val[(rows == col) & marginal[rows]] = 2.0 + 1e-9
    hval[(hrow == hcol) & marginal[hrow]] = 2.0 + 1e-9
    o = boxqp.options_struct(1e-7, 30.0, 20000, 'mixed')
    x, st = engine.solve(rowptr, col, val, inst['c'], inst['lower'], inst['upper'], o)
    assert boxqp.STATUS_NAMES[st.status] == 'optimal', st.as_dict()
    chk = O.check(hrow, hcol, hval, inst['c'], inst['lower'], inst['upper'], x, tol=1e-7)
    assert chk['verified'] == 1.0, chk


def test_nonconvex_hessian_is_reported_before_solving(engine):
    """check_convex_hessian runs first (src/accelerated_qp.cpp:19): an indefinite Q gets
    unsupported_curvature from the C-ABI solve; a PSD but not diagonally dominant Q solves."""
    # [[1, 2], [2, 1]] is indefinite (eigenvalues 3, -1) and not diagonally dominant
    rowptr = np.array([0, 2, 4], np.int32)
    col = np.array([0, 1, 0, 1], np.int32)
    val = np.array([1.0, 2.0, 2.0, 1.0])
    c = np.array([1.0, -1.0])
    lo, up = np.full(2, -1.0), np.full(2, 1.0)
    o = boxqp.options_struct(1e-7, 10.0, 10000, 'fp64')
    x, st = engine.solve(rowptr, col, val, c, lo, up, o)
    assert boxqp.STATUS_NAMES[st.status] == 'unsupported_curvature'
    # [[2, 1.5], [1.5, 2]] is PSD but not diagonally dominant: the LDL^T path accepts it
    val = np.array([2.0, 1.5, 1.5, 2.0])
    for precision in ('fp64', 'mixed'):
        o = boxqp.options_struct(1e-7, 10.0, 10000, precision)
        x, st = engine.solve(rowptr, col, val, c, lo, up, o)
        assert boxqp.STATUS_NAMES[st.status] == 'optimal', precision


@pytest.mark.parametrize('preset,n,seed,precision', [('graph10k', 0, 11, 'mixed'), ('graph1m', 200000, 4, 'mixed'),
                                                     ('tridiagonal', 150000, 2, 'fp64')])
def test_borrowed_submission_and_fetch_paths_agree(engine, preset, n, seed, precision):
    """bqp_submit_borrowed (no host copy) gives the bits of bqp_submit and bqp_solve_sync; a primal
    above 131072 variables is copied at bqp_fetch from device memory, into `out` if given, and a
    second fetch and a fetch after a re-run return the same bits."""
    inst = boxqp.planted(preset, seed=seed, n=n)
    o = boxqp.options_struct(1e-6, 60.0, 200000, precision)
    a = (inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'])
    xs, ss = engine.solve(*a, o)
    i_copy = engine.submit(*a, o)
    i_borrow = engine.submit(*a, o, copy=False)
    assert engine.wait(i_copy, 120.0) and engine.wait(i_borrow, 120.0)
    xc, sc = engine.fetch(i_copy, inst['n'])
    out = np.full(inst['n'], np.nan)
    xb, sb = engine.fetch(i_borrow, inst['n'], out=out)
    assert xb is out
    xb2, _ = engine.fetch(i_borrow, inst['n'])
    engine.resolve([i_borrow])
    assert engine.wait(i_borrow, 120.0)
    xb3, sb3 = engine.fetch(i_borrow, inst['n'])
    engine.release(i_copy)
    engine.release(i_borrow)
    assert boxqp.STATUS_NAMES[ss.status] == 'optimal'
    for x, st in ((xc, sc), (xb, sb), (xb2, sb), (xb3, sb3)):
        assert np.array_equal(x, xs) and st.iterations == ss.iterations and st.objective == ss.objective
    with pytest.raises(ValueError):
        engine.fetch(i_copy, inst['n'], out=np.empty(inst['n'], np.float32))


@pytest.mark.parametrize('precision', ['mixed', 'fp64'])
def test_every_spmv_structure_solves(engine, precision):
    """Each step-kernel group (precision x SpMV structure, forced through kernel_variant) solves
    the same instance to a verified optimum with the same objective."""
    inst = boxqp.planted('graph10k', seed=31, n=3000)
    a = (inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'])
    objs = []
    for variant in (0, 64, 1, 2, 4, 8, 16, 32):
        o = boxqp.options_struct(1e-7, 60.0, 200000, precision, kernel_variant=variant)
        x, st = engine.solve(*a, o)
        assert boxqp.STATUS_NAMES[st.status] == 'optimal', (variant, st.as_dict())
        objs.append(st.objective)
    assert max(objs) - min(objs) <= 1e-9 * max(1.0, abs(objs[0]))


def test_mixed_precisions_and_structures_in_one_batch_equal_solo(engine):
    """A batch holding FP64, FP64_EXACT and mixed solves of several SpMV structures at once (one
    step launch per group, the exact engine's own kernel) gives each solve the bits it gets alone."""
    cases = []
    for k, (preset, n, prec, variant) in enumerate([('graph10k', 2000, 'mixed', -1), ('grid', 64 * 64, 'mixed', -1),
                                                    ('graph10k', 2500, 'fp64', -1), ('tridiagonal', 3000, 'fp64', 2),
                                                    ('graph10k', 1500, 'fp64_exact', -1), ('graph10k', 1800, 'mixed', 8),
                                                    ('grid', 48 * 48, 'fp64', 64), ('graph10k', 2200, 'mixed', 0),
                                                    ('tridiagonal', 3000, 'mixed', -1)]):
        inst = boxqp.planted(preset, seed=40 + k, n=n)
        o = boxqp.options_struct(1e-7, 60.0, 200000, prec, kernel_variant=variant)
        cases.append((inst, o))
    solo = []
    for inst, o in cases:
        x, st = engine.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
        assert boxqp.STATUS_NAMES[st.status] == 'optimal', st.as_dict()
        solo.append((x, st.iterations, st.objective))
    ids = [engine.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
           for inst, o in cases]
    for (inst, _), ident, (xs, its, obj) in zip(cases, ids, solo):
        assert engine.wait(ident, 120.0)
        x, st = engine.fetch(ident, inst['n'])
        engine.release(ident)
        assert np.array_equal(x, xs) and st.iterations == its and st.objective == obj


def test_pinned_host_arrays_give_the_same_bits(engine):
    """Submissions from page-locked arrays (bqp_host_register) upload by DMA and give the bits of
    pageable ones; registering twice is refused, unregistering restores pageable behaviour."""
    inst = boxqp.planted('graph1m', seed=9, n=150000)
    a = (inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'])
    o = boxqp.options_struct(1e-6, 60.0, 200000, 'mixed')
    xs, ss = engine.solve(*a, o)
    with boxqp.pinned(*a):
        with pytest.raises(boxqp.EngineError):
            with boxqp.pinned(a[1]):
                pass
        ids = [engine.submit(*a, o, copy=False) for _ in range(3)]
        xp, sp = engine.solve(*a, o)
        for ident in ids:
            assert engine.wait(ident, 120.0)
            x, st = engine.fetch(ident, inst['n'])
            engine.release(ident)
            assert np.array_equal(x, xs) and st.iterations == ss.iterations
    assert np.array_equal(xp, xs) and sp.objective == ss.objective
    x2, _ = engine.solve(*a, o)
    assert np.array_equal(x2, xs)


@pytest.mark.parametrize('name', ['graph2k_open', 'grid32_open', 'graph2k_fixed'])
@pytest.mark.parametrize('precision', ['mixed', 'fp64'])
def test_one_sided_boxes(engine, golden, name, precision):
    """Infinite lower or upper bounds on a share of the variables, or fixed variables (l = u): the
    FP64 and mixed engines return a point inside the box that verifies at the case's tolerance
    (oracle checker) and reaches the reference's objective."""
    d, _ = golden
    rec = next(c for c in d['cases'] if c['name'] == name)
    p, inst = inputs(rec)
    x, st = solve(engine, inst, precision, rec['tol'])
    assert boxqp.STATUS_NAMES[st.status] == 'optimal', st.as_dict()
    chk = O.check(*args(p), x, tol=rec['tol'])
    assert chk['verified']
    assert np.all(np.isfinite(x))
    assert np.all(x >= p['lower']) and np.all(x <= p['upper'])
    assert st.objective == pytest.approx(rec['objective'], rel=1e-6)


def test_profile_cg_times_the_polish_and_the_solve_reruns_to_the_same_bits(engine):
    """bqp_profile_cg re-runs the polish of a finished mixed solve and times its CG kernels; the
    bytes it reports are the packed Q_FF's, and a re-solve afterwards gives the same answer."""
    inst = boxqp.planted('graph1m', seed=1, n=200000)
    o = boxqp.options_struct(1e-6, 60.0, 200000, 'mixed')
    ident = engine.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
    engine.wait(ident)
    x, st = engine.fetch(ident, inst['n'])
    assert boxqp.STATUS_NAMES[st.status] == 'optimal' and st.polish_iterations > 0
    ms_mv, ms_vec, b_mv, b_vec = engine.profile_cg(ident, 5)
    assert ms_mv > 0 and ms_vec > 0
    free_rows = b_vec / 84.0
    assert 0 < free_rows <= inst['n']
    assert 0 < (b_mv - 52.0 * free_rows) / 12.0 <= inst['nnz']  # packed Q_FF entries
    engine.resolve([ident])
    engine.wait(ident)
    x2, st2 = engine.fetch(ident, inst['n'])
    assert np.array_equal(x, x2) and st2.iterations == st.iterations
    engine.release(ident)


@pytest.mark.parametrize('precision', ['fp64', 'mixed', 'fp64_exact'])
def test_engine_convexity_gate_gives_the_reference_verdicts(engine, precision):
    """The engine decides check_convex_hessian on the device at admission (diagonal dominance and
    the Gershgorin bound in one pass over the uploaded CSR; the host LDL' only where dominance
    fails).  Through the C-ABI, each of the reference's edge cases
    (tests/golden/reference_convexity.json) is solved where the reference calls it convex, with
    the Gershgorin bound of the host helper bit for bit as its L, and finishes
    unsupported_curvature where it does not.  With infeasible bounds, a non-convex Hessian still
    reports unsupported_curvature first, as in the reference."""
    import json
    from pathlib import Path
    cases = json.loads((Path(__file__).resolve().parent / 'golden' / 'reference_convexity.json').read_text())
    for c in cases:
        n = c['n']
        sign = -1.0 if c['maximize'] else 1.0
        rowptr, col, val = boxqp.csr_from_lower(n, np.array(c['hrow'], np.int64), np.array(c['hcol'], np.int64),
                                                np.array(c['hval']), sign)
        o = boxqp.options_struct(1e-7, 30.0, 200000, precision)
        zeros, ones = np.zeros(n), np.ones(n)
        x, st = engine.solve(rowptr, col, val, zeros, zeros, ones, o)
        status = boxqp.STATUS_NAMES[st.status]
        if c['convex']:
            assert status == 'optimal', (c['name'], status)
            assert st.lipschitz == boxqp.gershgorin(rowptr, val), c['name']
        else:
            assert status == 'unsupported_curvature' and st.iterations == 0, (c['name'], status)
        lo = zeros.copy()
        lo[0] = 2.0  # l > u
        x, st = engine.solve(rowptr, col, val, zeros, lo, ones, o)
        want = 'infeasible_bounds' if c['convex'] else 'unsupported_curvature'
        assert boxqp.STATUS_NAMES[st.status] == want, (c['name'], boxqp.STATUS_NAMES[st.status])
