"""solve_qp_admm with its iterations on the GPU (needs a GPU).

The host loop (boxqp/admm.py) is pinned to the reference's solve_qp_admm bit for bit on the CPU
(tests/test_admm_solver.py, with the restated iterations in place of the device).  On the GPU the
iterations round differently (FMA, double instead of long double inner products), so the loop
takes its own path to the same answer: on the reference's constrained QPs solved at 1e-4 and
1e-5 it must return a primal and row duals that the reference's checker (restated bit for bit by
check_solution) verifies at that tolerance, with the reference's objective to 1e-5 relative.
"""
from pathlib import Path

import numpy as np
import pytest

import boxqp
from boxqp.admm import LinearRows, check_solution, solve_qp_admm

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / 'golden'


def _cases():
    data = np.load(GOLDEN / 'reference_admm_solve.npz')
    names = sorted({k.split('.')[0] for k in data.files})
    return [(name, {k.split('.', 1)[1]: data[k] for k in data.files if k.startswith(name + '.')}) for name in names]


def test_solve_qp_admm_on_the_gpu_verifies_the_reference_answers():
    ran = 0
    for name, p in _cases():
        tol = float(p['tol'])
        if tol < 1e-5:
            continue
        q = boxqp.QuadraticProblem(cost=p['cost'], lower=p['lower'], upper=p['upper'], hessian_row=p['hrow'],
                                   hessian_col=p['hcol'], hessian_val=p['hval'])
        rows = LinearRows(p['a_rowptr'], p['a_col'], p['a_val'], p['row_lower'], p['row_upper'])
        r = solve_qp_admm(q, rows, boxqp.QpOptions(tolerance=tol, iteration_limit=5000, time_limit=60.0))
        assert r.status == 'optimal' and r.optimality_verified, (name, r.status, r.iterations)
        assert r.engine['inner_iterations'] > 0
        chk = check_solution(q, rows, r.primal, r.row_dual, tol)
        assert chk['verified'], name
        ref_objective = float(p['stats'][0])
        assert abs(r.objective - ref_objective) / (1 + abs(ref_objective)) <= 1e-5, name
        assert np.max(np.abs(r.primal - p['x'])) <= 1e-3, name
        ran += 1
    assert ran == 3
