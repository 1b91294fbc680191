"""The reference's solve_qp_admm loop around the device iterations (boxqp/admm.py), without a GPU.

The host side of solve_qp_admm (the scaled set-up, the original-model check with row duals, the
rho adaptation, the 25-iteration cadence and the statuses) is checked against the reference
itself: its set-up against the restatement pinned in tests/test_admm_oracle.py, its checker
against the reference's check_qp_solution on constrained candidates, and the whole loop, driven
by the restated iterations (oracle/admm_pcg.py) in place of the device, against the reference's
own solve_qp_admm answers (tests/golden/reference_admm_solve.npz, made by
tests/golden/make_golden.py from the reference built in oracle/_ref).
"""
import json
import math
import os
from pathlib import Path

import numpy as np
import pytest

import boxqp
from boxqp.admm import (LinearRows, admm_setup, check_solution, merge_rows, solve_diagonal_equalities,
                        solve_qp_admm)
from oracle.admm_pcg import AdmmSystemOracle, admm_iteration, scale_qp_admm

GOLDEN = Path(__file__).resolve().parent / 'golden'
KEYS = ('objective', 'primal_residual', 'stationarity_residual', 'complementarity_residual', 'dual_bound',
        'relative_gap', 'verified')
EXACT = np.finfo(np.longdouble).nmant == 63  # x87 80-bit long double, the reference's on x86


def _cases(file):
    data = np.load(GOLDEN / file)
    names = sorted({k.split('.')[0] for k in data.files})
    return [(name, {k.split('.', 1)[1]: data[k] for k in data.files if k.startswith(name + '.')}) for name in names]


def _problem(p):
    q = boxqp.QuadraticProblem(cost=p['cost'], lower=p['lower'], upper=p['upper'], hessian_row=p['hrow'],
                               hessian_col=p['hcol'], hessian_val=p['hval'],
                               maximize=bool(p['maximize']) if 'maximize' in p else False,
                               offset=float(p['offset']) if 'offset' in p else 0.0)
    rows = LinearRows(p['a_rowptr'], p['a_col'], p['a_val'], p['row_lower'], p['row_upper'])
    return q, rows


class RestatedSystem:
    """The restated ADMM iterations (oracle/admm_pcg.py, bit for bit the reference's) behind the
    device system's interface."""

    def __init__(self, h, a, n):
        self.o = AdmmSystemOracle(h, a, n)
        self.rho_changes = 0

    def set_rho(self, rho, sigma):
        self.rho_changes += 1
        self.o.set_rho(rho, sigma)

    def iterate(self, c, lo, up, x, z, y, first, count):
        total = 0
        for k in range(count):
            x, z, y, inner = admm_iteration(self.o, c, lo, up, x, z, y, first + k)
            total += inner
        return x, z, y, total

    def close(self):
        pass


def _same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b))


def test_setup_equals_the_restated_setup():
    """admm_setup (vectorised) forms the scaled problem of qp_admm.cpp:136-158 with the same bits as
    the loop-by-loop restatement pinned to the reference."""
    for file in ('reference_admm.npz', 'reference_admm_adapt.npz', 'reference_admm_solve.npz',
                 'reference_admm_rows.npz'):
        for name, p in _cases(file):
            scaling = bool(p['scaling']) if 'scaling' in p else True
            q, rows = _problem(p)
            sp = admm_setup(q, rows, scaling)
            ref = scale_qp_admm(int(p['n']), p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'],
                                p['a_rowptr'], p['a_col'], p['a_val'], p['row_lower'], p['row_upper'], scaling,
                                maximize=q.maximize)
            for k in ('c', 'lo', 'up', 'variable', 'x', 'z', 'y', 'rho'):
                assert _same(sp[k], ref[k]), (name, k)
            for k in ('h', 'a'):
                for u, v in zip(sp[k], ref[k]):
                    assert _same(u, v), (name, k)
            assert sp['sigma'] == ref['sigma']


def test_merge_rows_follows_csrmatrix():
    """Rows with unsorted and repeated columns: ascending columns, repeats summed in input order,
    zero sums dropped (CsrMatrix(n, rows), include/sparse_matrix.hpp:10-17)."""
    rowptr = np.array([0, 4, 4, 7])
    col = np.array([3, 1, 3, 0, 2, 2, 5])
    val = np.array([0.1, 2.0, 0.2, -1.0, 1.5, -1.5, 4.0])
    rp, c, v = merge_rows(rowptr, col, val)
    assert rp.tolist() == [0, 3, 3, 4]
    assert c.tolist() == [0, 1, 3, 5]
    assert v.tolist() == [-1.0, 2.0, 0.1 + 0.2, 4.0]


def test_checker_matches_the_reference_on_box_edge_cases():
    """check_solution with no rows returns the reference's check_qp_solution fields on the box
    candidates of tests/golden/reference_checks.json."""
    for c in json.loads((GOLDEN / 'reference_checks.json').read_text()):
        p = {k: np.array([float(v) for v in vs]) for k, vs in c['problem'].items()}
        q = boxqp.QuadraticProblem(cost=p['cost'], lower=p['lower'], upper=p['upper'],
                                   hessian_row=p['hrow'].astype(np.int64), hessian_col=p['hcol'].astype(np.int64),
                                   hessian_val=p['hval'], maximize=c['maximize'], offset=c['offset'])
        rows = LinearRows(np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), np.zeros(0), np.zeros(0))
        got = check_solution(q, rows, np.array([float(v) for v in c['x']]), np.zeros(0), c['tol'])
        for k in KEYS:
            want = float(c['result'][k])
            have = float(got[k])
            if math.isnan(want):
                assert math.isnan(have), (c['name'], k)
            elif EXACT or not math.isfinite(want):
                assert have == want, (c['name'], k, have, want)
            else:
                assert have == pytest.approx(want, rel=1e-15, abs=1e-300), (c['name'], k)


def test_checker_matches_the_reference_with_rows():
    """With linear rows and row duals (the reference's answer, a perturbed primal, zero duals) the
    residuals, complementarity, bound, gap and verdict equal the reference's check_qp_solution."""
    for name, p in _cases('reference_admm_solve.npz'):
        q, rows = _problem(p)
        tol = float(p['tol'])
        for k in range(3):
            got = check_solution(q, rows, p[f'cand{k}_x'], p[f'cand{k}_y'], tol)
            want = dict(zip(KEYS, p[f'cand{k}_stats'].tolist()))
            for key in KEYS:
                if EXACT:
                    assert float(got[key]) == want[key], (name, k, key, got[key], want[key])
                else:
                    assert float(got[key]) == pytest.approx(want[key], rel=1e-14, abs=1e-300), (name, k, key)
        assert bool(dict(zip(KEYS, p['cand0_stats'].tolist()))['verified'])


def test_solve_qp_admm_reproduces_the_reference_answers():
    """The host loop driven by the restated iterations returns the reference's status, iteration
    count, primal, row duals and checker fields (the whole solve_qp_admm, including a rho
    adaptation for the cases that pass iteration 100)."""
    adapted = 0
    for name, p in _cases('reference_admm_solve.npz'):
        q, rows = _problem(p)
        made = []

        def make(h, a, n):
            made.append(RestatedSystem(h, a, n))
            return made[-1]

        r = solve_qp_admm(q, rows, boxqp.QpOptions(tolerance=float(p['tol'])), make_system=make)
        assert r.status == 'optimal' and r.optimality_verified, (name, r.status)
        assert r.iterations == int(p['iterations']), (name, r.iterations, int(p['iterations']))
        assert r.algorithm == 'scaled_admm_pcg'
        if EXACT:
            assert _same(r.primal, p['x']) and _same(r.row_dual, p['row_dual']), name
        else:
            assert np.max(np.abs(r.primal - p['x'])) <= 1e-10, name
        want = dict(zip(KEYS, p['stats'].tolist()))
        assert r.objective == pytest.approx(want['objective'], rel=1e-13), name
        adapted += made[0].rho_changes > 1
    assert adapted >= 1


def test_solve_qp_admm_row_handling_matches_the_reference():
    """Rows with columns out of order, repeated columns, a repeat that cancels, an empty row,
    one-sided rows (an infinite lower or upper bound) and equality rows, a maximisation with an
    offset, and a QP with no linear rows (the ADMM over the bound rows alone): after 20 iterations (tolerance 1e-12, nothing verifies) and over the whole solve at
    1e-5 the loop returns the reference's primal and row duals (bit for bit where long double is
    the reference's type), and the maximisation its objective in the maximisation sense."""
    for name, p in _cases('reference_admm_rows.npz'):
        q, rows = _problem(p)

        def make(h, a, n):
            return RestatedSystem(h, a, n)

        if 'x20' in p:
            r = solve_qp_admm(q, rows, boxqp.QpOptions(tolerance=1e-12, iteration_limit=20), make_system=make)
            assert r.status == 'iteration_limit' and r.iterations == 20
            assert _same(r.primal, p['x20']) and _same(r.row_dual, p['y20']), name
        r = solve_qp_admm(q, rows, boxqp.QpOptions(tolerance=1e-5), make_system=make)
        assert r.objective == pytest.approx(float(p['stats'][0]), rel=1e-13), name
        assert r.status == str(p['status']) and r.iterations == int(p['iterations']), (name, r.status, r.iterations)
        if EXACT:
            assert _same(r.primal, p['x']) and _same(r.row_dual, p['row_dual']), name
        else:
            assert np.max(np.abs(r.primal - p['x'])) <= 1e-10, name


def test_solve_qp_admm_statuses_and_option_checks():
    """Invalid options and integer variables raise as the reference does; lower > upper gives
    infeasible_bounds, a non-convex Hessian unsupported_curvature, an iteration limit of 0 the
    status iteration_limit with the checked starting point."""
    name, p = _cases('reference_admm_solve.npz')[0]
    q, rows = _problem(p)

    def make(h, a, n):
        return RestatedSystem(h, a, n)

    for bad in (dict(tolerance=0.0), dict(tolerance=math.nan), dict(time_limit=-1.0), dict(threads=0)):
        with pytest.raises(ValueError, match='Invalid QP options'):
            solve_qp_admm(q, rows, boxqp.QpOptions(**bad), make_system=make)
    # validate_linear_problem (src/mps.cpp:47-60)
    bad_cost = np.array(q.cost, dtype=float)
    bad_cost[2] = np.nan
    qc = boxqp.QuadraticProblem(cost=bad_cost, lower=q.lower, upper=q.upper, hessian_row=q.hessian_row,
                                hessian_col=q.hessian_col, hessian_val=q.hessian_val)
    with pytest.raises(ValueError, match='Invalid variable coefficient or bound'):
        solve_qp_admm(qc, rows, make_system=make)
    qo = boxqp.QuadraticProblem(cost=q.cost, lower=q.lower, upper=q.upper, hessian_row=q.hessian_row,
                                hessian_col=q.hessian_col, hessian_val=q.hessian_val, offset=math.inf)
    with pytest.raises(ValueError, match='dimensions or offset'):
        solve_qp_admm(qo, rows, make_system=make)
    rb = LinearRows(rows.rowptr, rows.col, rows.val, np.full(rows.m, np.inf), rows.upper)
    with pytest.raises(ValueError, match='Invalid row bound'):
        solve_qp_admm(q, rb, make_system=make)
    bad_col = np.array(rows.col)
    bad_col[0] = q.n
    with pytest.raises(ValueError, match='Invalid sparse row entry'):
        solve_qp_admm(q, LinearRows(rows.rowptr, bad_col, rows.val, rows.lower, rows.upper), make_system=make)
    # malformed row pointers: not starting at 0, decreasing, not ending at the entry count
    for fix in (lambda r: r + 1, lambda r: np.concatenate([r[:1], r[2:2], r[1:]])[::-1].copy(),
                lambda r: np.concatenate([r[:-1], r[-1:] - 1])):
        bad_ptr = fix(np.array(rows.rowptr, dtype=np.int32))
        if bad_ptr.shape != np.asarray(rows.rowptr).shape:
            continue
        with pytest.raises(ValueError, match='Invalid sparse row entry'):
            solve_qp_admm(q, LinearRows(bad_ptr, rows.col, rows.val, rows.lower, rows.upper), make_system=make)
    qi = boxqp.QuadraticProblem(cost=q.cost, lower=q.lower, upper=q.upper, hessian_row=q.hessian_row,
                                hessian_col=q.hessian_col, hessian_val=q.hessian_val,
                                integer=np.arange(q.n) == 0)
    with pytest.raises(ValueError, match='Continuous QP required'):
        solve_qp_admm(qi, rows, make_system=make)
    lo = np.array(q.lower, dtype=float)
    lo[3] = 2.0
    qb = boxqp.QuadraticProblem(cost=q.cost, lower=lo, upper=q.upper, hessian_row=q.hessian_row,
                                hessian_col=q.hessian_col, hessian_val=q.hessian_val)
    assert solve_qp_admm(qb, rows, make_system=make).status == 'infeasible_bounds'
    rl = np.array(rows.lower, dtype=float)
    rl[0] = rows.upper[0] + 1
    rb = LinearRows(rows.rowptr, rows.col, rows.val, rl, rows.upper)
    assert solve_qp_admm(q, rb, make_system=make).status == 'infeasible_bounds'
    hv = np.array(q.hessian_val, dtype=float)
    hv[q.hessian_row == q.hessian_col] *= -1
    qn = boxqp.QuadraticProblem(cost=q.cost, lower=q.lower, upper=q.upper, hessian_row=q.hessian_row,
                                hessian_col=q.hessian_col, hessian_val=hv)
    assert solve_qp_admm(qn, rows, make_system=make).status == 'unsupported_curvature'
    r = solve_qp_admm(q, rows, boxqp.QpOptions(iteration_limit=0), make_system=make)
    assert r.status == 'iteration_limit' and r.iterations == 0 and not r.optimality_verified
    assert np.all(r.primal == 0) and np.all(r.row_dual == 0)
    # a zero time limit ends the solve at the first check, after the verification and the
    # non-finite test (qp_admm.cpp:247-249)
    r = solve_qp_admm(q, rows, boxqp.QpOptions(time_limit=0.0), make_system=make)
    assert r.status == 'time_limit' and r.iterations == 0


def test_solve_qp_admm_kkt_polish_reproduces_the_reference():
    """Diagonal-Hessian QPs whose ADMM does not verify by iteration 250: the loop's KKT polish
    (polish_diagonal) verifies there and returns the reference's primal and row duals
    (tests/golden/reference_admm_polish.npz; bit for bit where long double is the reference's)."""
    for name, p in _cases('reference_admm_polish.npz'):
        q, rows = _problem(p)
        r = solve_qp_admm(q, rows, boxqp.QpOptions(tolerance=float(p['tol'])),
                          make_system=lambda h, a, n: RestatedSystem(h, a, n))
        assert r.status == 'optimal' and r.iterations == 250 == int(p['iterations']), (name, r.status, r.iterations)
        assert r.algorithm == 'scaled_admm_pcg_kkt_polish' and r.optimality_verified
        if EXACT:
            assert _same(r.primal, p['x']) and _same(r.row_dual, p['row_dual']), name
        else:
            assert np.max(np.abs(r.primal - p['x'])) <= 1e-10, name
        assert r.objective == pytest.approx(float(p['stats'][0]), rel=1e-13), name


def test_planted_kkt_tests_of_the_reference_scripts_with_rows():
    """Cases 15-29 of the reference's planted KKT tests (scripts/test_qp.py:30-56: n = 5, dense
    PSD Hessian, three inequality rows active at the planted optimum; tests/golden/
    reference_kkt_rows.json): the loop passes the script's own criteria -- status optimal,
    objective within 1e-6 relative of the planted one, projected-gradient residual of
    H x + c + A'y at most 2e-7, x inside [-3, 3], rows satisfied to 1e-6.  The reference reaches
    14 of them through its KKT polish at iteration 250 (its general, sparse-LU form: the
    Hessians are dense); the loop's polish_kkt verifies the same 14 at iteration 250 with the
    reference's objective to 1e-12 and primal to 1e-9 (another LU rounds differently), and the one
    verified by ADMM alone (case 18, iteration 225) the loop reproduces bit for bit."""
    recs = json.loads((GOLDEN / 'reference_kkt_rows.json').read_text())
    assert len(recs) == 15
    for rec in recs:
        n = 5
        q = boxqp.QuadraticProblem(cost=np.array(rec['cost']), lower=np.full(n, -3.0), upper=np.full(n, 3.0),
                                   hessian_row=np.array(rec['hrow']), hessian_col=np.array(rec['hcol']),
                                   hessian_val=np.array(rec['hval']))
        a_val = np.array(rec['a_val'])
        rows = LinearRows(np.array(rec['a_rowptr']), np.array(rec['a_col']), a_val, np.full(3, -np.inf),
                          np.array(rec['row_upper']))
        r = solve_qp_admm(q, rows, boxqp.QpOptions(), make_system=lambda h, a, n: RestatedSystem(h, a, n))
        expected = rec['expected_objective']
        assert r.status == 'optimal', rec['case']
        assert abs(r.objective - expected) / (1 + abs(expected)) <= 1e-6, rec['case']
        h = np.zeros((n, n))
        h[np.array(rec['hrow']), np.array(rec['hcol'])] = rec['hval']
        h = h + np.tril(h, -1).T
        a = a_val.reshape(3, n)
        g = h @ r.primal + np.array(rec['cost']) + a.T @ r.row_dual
        assert np.max(np.abs(r.primal - np.clip(r.primal - g, -3, 3)) / (1 + np.abs(r.primal))) <= 2e-7, rec['case']
        assert np.all(np.abs(r.primal) <= 3) and np.all(a @ r.primal <= np.array(rec['row_upper']) + 1e-6)
        assert r.iterations == rec['iterations'], (rec['case'], r.iterations, rec['iterations'])
        if rec['iterations'] < 250:
            if EXACT:
                assert _same(r.primal, rec['x']) and _same(r.row_dual, rec['row_dual']), rec['case']
        else:
            assert r.algorithm == 'scaled_admm_pcg_kkt_polish', rec['case']
            assert r.objective == pytest.approx(rec['objective'], rel=1e-12, abs=1e-12), rec['case']
            assert np.max(np.abs(r.primal - np.array(rec['x']))) <= 1e-9, rec['case']


def test_diagonal_equality_presolver_reproduces_the_reference():
    """Positive diagonal Hessian, only equality rows: solve_qp_admm returns its pre-solver's answer
    (solve_diagonal_equalities, the reference's dual Newton) with the reference's status,
    iteration count, primal and row duals (tests/golden/reference_dual_newton.npz), scaled and
    unscaled; a run capped at 3 iterations with an unreachable tolerance stops where the
    reference's does."""
    for name, p in _cases('reference_dual_newton.npz'):
        q, rows = _problem(p)
        tol, limit = float(p['tol']), int(p['limit'])
        o = boxqp.QpOptions(tolerance=tol, iteration_limit=limit, scaling=bool(p['scaling']), time_limit=600.0)
        if str(p['status']) == 'optimal':
            r = solve_qp_admm(q, rows, o, make_system=lambda h, a, n: pytest.fail('the ADMM must not run'))
            assert r.algorithm == 'diagonal_qp_dual_newton', name
        else:
            r = solve_diagonal_equalities(q, rows, o)
        assert r.status == str(p['status']) and r.iterations == int(p['iterations']), (name, r.status, r.iterations)
        if EXACT:
            assert _same(r.primal, p['x']) and _same(r.row_dual, p['row_dual']), name
        else:
            assert np.max(np.abs(r.primal - p['x'])) <= 1e-10, name
    # other structures are declined at once
    name, p = _cases('reference_admm_solve.npz')[0]
    q, rows = _problem(p)
    assert solve_diagonal_equalities(q, rows, boxqp.QpOptions()).status == 'unsupported_structure'


@pytest.mark.skipif(not os.environ.get('BOXQP_REFERENCE_DIR'), reason='set BOXQP_REFERENCE_DIR to the reference solver')
def test_solve_qp_admm_on_qplib_9002():
    """QPLIB 9002 (2,890 variables, diagonal Hessian, 1,649 equality rows), read by
    read_qplib_rows: the pre-solver answers within its 10 s share of the default time limit with
    the reference's status, iteration count (180), primal and row duals; no ADMM runs."""
    from boxqp.qplib import read_qplib_rows
    path = Path(os.environ['BOXQP_REFERENCE_DIR']) / 'datasets' / 'qplib' / '9002.qplib'
    q, rows = read_qplib_rows(path.read_text())
    r = solve_qp_admm(q, rows, boxqp.QpOptions(tolerance=1e-7),
                      make_system=lambda h, a, n: pytest.fail('the ADMM must not run'))
    assert r.status == 'optimal' and r.algorithm == 'diagonal_qp_dual_newton' and r.iterations == 180
    assert r.objective == pytest.approx(5698097498.5664835, rel=1e-15)


def test_qplib_model_with_rows_end_to_end():
    """A QCL model in QPLIB text (rows listed out of order, one-sided and equality rows): read by
    read_qplib_rows and solved by the loop (restated iterations in place of the device), it gets
    the reference's answer -- the reference's own reader and solve_qp_admm on the same file."""
    from oracle import oracle as O
    from test_qplib_cli import constrained_qplib_text
    from boxqp.qplib import read_qplib_rows
    if not O.ref_available():
        pytest.skip('oracle/_ref not built on this host')
    text = constrained_qplib_text(seed=11)
    q, rows = read_qplib_rows(text)
    r = solve_qp_admm(q, rows, boxqp.QpOptions(tolerance=1e-6), make_system=lambda h, a, n: RestatedSystem(h, a, n))
    status, x, st = O.ref_solve_qp_admm(q.hessian_row, q.hessian_col, q.hessian_val, q.cost, q.lower, q.upper,
                                        rows.rowptr, rows.col, rows.val, rows.lower, rows.upper, tol=1e-6,
                                        offset=q.offset)
    assert r.status == status and r.iterations == int(st['iterations']), (r.status, r.iterations, status, st)
    if r.algorithm == 'scaled_admm_pcg_kkt_polish':
        assert np.max(np.abs(r.primal - x)) <= 1e-9
    elif EXACT:
        assert _same(r.primal, x) and _same(r.row_dual, st['row_dual'])
    assert r.objective == pytest.approx(st['objective'], rel=1e-12)
