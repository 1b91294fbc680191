"""Parity at the benchmarked sizes, and the reference's public box instances (needs a GPU).

The engine's results at the full sizes of the workloads are checked on the host by the oracle
(check_qp_solution restated and pinned to the reference bit for bit) and against the planted
optimum.  Tolerances:
  * KKT: verified by the oracle's FP64 checker at the requested tolerance (stationarity and
    primal residual <= tol).
  * objective: |f - f*| <= 1e-7 (1 + |f*|), f* the planted optimum in long double.
  * active set: no variable off the planted active set where the planted margin exceeds 1e-6
    (the planted margins are >= 0.1 at active bounds, so none is allowed).
  * QPLIB 8792 / 8991 (the reference's box instances, staged from its datasets by
    oracle/ref.mk): read by the product's QPLIB reader, the bit-exact FP64 engine gives the
    reference's status, iteration count and objective (to 1e-12); the plain FP64 and the mixed
    engines verify at 1e-7 with the objective to 1e-7 relative.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import boxqp
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def solve(engine, inst, precision, tol, iteration_limit=200000):
    o = boxqp.options_struct(tol, 120.0, iteration_limit, precision)
    return engine.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)


def verify(inst, x, st, tol):
    chk = O.check(inst['hrow'], inst['hcol'], inst['hval'], inst['c'], inst['lower'], inst['upper'], x, tol=tol)
    assert boxqp.STATUS_NAMES[st.status] == 'optimal', st.as_dict()
    assert chk['verified'] == 1.0, chk
    assert chk['stationarity_residual'] <= tol and chk['primal_residual'] <= tol
    fstar = inst['fstar']
    assert abs(chk['objective'] - fstar) <= 1e-7 * (1 + abs(fstar))
    assert st.objective == pytest.approx(chk['objective'], rel=1e-12, abs=1e-12)
    assert O.active_set_mismatches(x, inst) == 0
    return chk


@pytest.fixture(scope='module')
def graph1m():
    return boxqp.planted('graph1m', seed=1, lower_triplets=True)


@pytest.fixture(scope='module')
def grid1024():
    return boxqp.planted('grid', seed=2, lower_triplets=True)


@pytest.mark.parametrize('precision', ['mixed', 'fp64'])
def test_random_graph_1m_at_full_size(engine, graph1m, precision):
    """n = 1,000,000, 7 edges per vertex (~15M nonzeros), bounds [-1, 1], KKT <= 1e-6."""
    assert graph1m['n'] == 1000000 and graph1m['nnz'] > 14_000_000
    x, st = solve(engine, graph1m, precision, 1e-6)
    verify(graph1m, x, st, 1e-6)


@pytest.mark.parametrize('precision,tol', [('mixed', 1e-6), ('fp64', 1e-6), ('mixed', 1e-8), ('fp64', 1e-8)])
def test_grid_1024_squared_at_full_size(engine, grid1024, precision, tol):
    """1024 x 1024 five-point Laplacian + 1e-3 I (n = 1,048,576), random boxes, KKT <= 1e-6 and 1e-8."""
    assert grid1024['n'] == 1024 * 1024
    x, st = solve(engine, grid1024, precision, tol)
    verify(grid1024, x, st, tol)


@pytest.mark.parametrize('precision', ['mixed', 'fp64'])
def test_graph10k_over_seeds_0_to_31(engine, precision):
    """n = 10,000, 5 edges per vertex, bounds [0, 1], seeds 0..31, KKT <= 1e-6."""
    for seed in range(32):
        inst = boxqp.planted('graph10k', seed=seed, lower_triplets=True)
        x, st = solve(engine, inst, precision, 1e-6)
        verify(inst, x, st, 1e-6)


def _qplib_records():
    d = json.loads((ROOT / 'tests' / 'golden' / 'reference_cases.json').read_text())
    return {r['name']: r for r in d['qplib']}


@pytest.mark.parametrize('name', ['8792', '8991'])
def test_qplib_box_instances_on_the_product_path(engine, name):
    """QPLIB 8792 and 8991 (the reference's published box instances: objectives
    3593.5162939294105 and -0.0016678673619609664) read by boxqp.qplib and solved on the GPU."""
    path = O.REF_QPLIB / f'{name}.qplib'
    if not path.exists():
        pytest.skip('the reference QPLIB files are not staged (make -f oracle/ref.mk stage)')
    rec = _qplib_records()[name]
    data = path.read_bytes()
    assert hashlib.sha256(data).hexdigest() == rec['sha256']
    from boxqp.qplib import read_qplib
    q, rows = read_qplib(data.decode())
    assert rows == 0 and q.n == rec['n']
    r = boxqp.solve_accelerated_box(q, boxqp.QpOptions(tolerance=1e-7, precision='fp64_exact', time_limit=600),
                                    engine=engine)
    assert r.status == rec['status'] and r.optimality_verified
    assert r.iterations == rec['iterations']
    assert r.objective == pytest.approx(rec['objective'], rel=1e-12, abs=1e-15)
    for precision in ('fp64', 'mixed'):
        r = boxqp.solve_accelerated_box(q, boxqp.QpOptions(tolerance=1e-7, precision=precision, time_limit=600),
                                        engine=engine)
        assert r.status == 'optimal' and r.optimality_verified, (precision, r.status)
        assert abs(r.objective - rec['objective']) <= 1e-7 * (1 + abs(rec['objective'])), (precision, r.objective)
