"""The CPU restatement of the reference's diagonal-Hessian equality solver (oracle/dual_newton.py)
and its row-aware checker, against the reference's own answers (no GPU).

solve_qp_admm tries solve_diagonal_equalities (src/qp_dual_newton.cpp:9-66) first on QPs with a
positive diagonal Hessian and only equality rows.  tests/golden/reference_dual_newton.npz holds the
reference's answers on four such QPs (tests/golden/make_golden.py, from the reference built in
oracle/_ref); the restatement must reproduce status, iteration count, primal and row duals bit for
bit where long double is the reference's 80-bit type (x86), to 1e-12 elsewhere.
"""
import os
from pathlib import Path

import numpy as np
import pytest

from oracle.dual_newton import check_rows, solve_diagonal_equalities_restated

GOLDEN = Path(__file__).resolve().parent / 'golden'
EXACT = np.finfo(np.longdouble).nmant == 63
KEYS = ('objective', 'primal_residual', 'stationarity_residual', 'complementarity_residual', 'dual_bound',
        'relative_gap', 'verified')


def _cases(file):
    data = np.load(GOLDEN / file)
    names = sorted({k.split('.')[0] for k in data.files})
    return [(name, {k.split('.', 1)[1]: data[k] for k in data.files if k.startswith(name + '.')}) for name in names]


def _rows(p):
    rp, col, val = p['a_rowptr'], p['a_col'], p['a_val']
    return [[(int(col[k]), float(val[k])) for k in range(rp[i], rp[i + 1])] for i in range(len(rp) - 1)]


def _close(a, b):
    return np.array_equal(a, b) if EXACT else np.max(np.abs(np.asarray(a) - np.asarray(b))) <= 1e-12


def test_restated_dual_newton_reproduces_the_reference():
    for name, p in _cases('reference_dual_newton.npz'):
        status, iterations, x, y, chk = solve_diagonal_equalities_restated(
            p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], _rows(p), p['row_lower'],
            p['row_upper'], float(p['tol']), int(p['limit']), bool(p['scaling']))
        assert status == str(p['status']) and iterations == int(p['iterations']), (name, status, iterations)
        assert _close(x, p['x']) and _close(y, p['row_dual']), name
        if EXACT:
            assert chk['objective'] == float(p['stats'][0]), name


def test_restated_row_checker_reproduces_the_reference_checker():
    """check_rows (plain loops) on the reference's constrained candidates: every field equal."""
    for name, p in _cases('reference_admm_solve.npz'):
        for k in range(3):
            got = check_rows(p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], _rows(p),
                             p['row_lower'], p['row_upper'], p[f'cand{k}_x'], p[f'cand{k}_y'], float(p['tol']))
            want = dict(zip(KEYS, p[f'cand{k}_stats'].tolist()))
            for key in KEYS:
                if EXACT:
                    assert float(got[key]) == want[key], (name, k, key)
                else:
                    assert float(got[key]) == pytest.approx(want[key], rel=1e-14, abs=1e-300), (name, k, key)


def test_structures_the_dual_newton_declines():
    """No rows, an inequality row, or a coupled Hessian: unsupported_structure
    (qp_dual_newton.cpp:13-17), so solve_qp_admm goes on to its ADMM."""
    name, p = _cases('reference_dual_newton.npz')[0]
    args = (p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'])
    assert solve_diagonal_equalities_restated(*args, [], [], [])[0] == 'unsupported_structure'
    up = np.array(p['row_upper'], dtype=float)
    up[0] += 1
    assert solve_diagonal_equalities_restated(*args, _rows(p), p['row_lower'], up)[0] == 'unsupported_structure'
    coupled = (np.append(p['hrow'], 1), np.append(p['hcol'], 0), np.append(p['hval'], 0.1))
    assert solve_diagonal_equalities_restated(*coupled, p['cost'], p['lower'], p['upper'], _rows(p), p['row_lower'],
                                              p['row_upper'])[0] == 'unsupported_structure'


@pytest.mark.skipif(not os.environ.get('BOXQP_REFERENCE_DIR'), reason='set BOXQP_REFERENCE_DIR to the reference solver')
def test_restated_dual_newton_on_qplib_9002():
    """QPLIB 9002 (diagonal Hessian, 1,649 equality rows): the reference solves it with this method
    in 180 iterations to objective 5698097498.5664835; the restatement gives the same bits (about
    a minute here)."""
    from boxqp.qplib import read_qplib_rows
    from oracle import oracle as O
    path = Path(os.environ['BOXQP_REFERENCE_DIR']) / 'datasets' / 'qplib' / '9002.qplib'
    q, rows = read_qplib_rows(path.read_text())
    rl = [[(int(rows.col[k]), float(rows.val[k])) for k in range(rows.rowptr[i], rows.rowptr[i + 1])]
          for i in range(rows.m)]
    status, iterations, x, y, chk = solve_diagonal_equalities_restated(
        q.hessian_row, q.hessian_col, q.hessian_val, q.cost, q.lower, q.upper, rl, rows.lower, rows.upper, 1e-7)
    assert status == 'optimal' and iterations == 180
    assert chk['objective'] == pytest.approx(5698097498.5664835, rel=1e-15)
    if O.ref_available():
        st, rx, s = O.ref_solve_diagonal_equalities(q.hessian_row, q.hessian_col, q.hessian_val, q.cost, q.lower,
                                                    q.upper, rows.rowptr, rows.col, rows.val, rows.lower, rows.upper,
                                                    tol=1e-7)
        assert _close(x, rx) and _close(y, s['row_dual'])
