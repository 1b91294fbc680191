"""The CPU oracle (oracle/boxqp_oracle.c) against the reference's own results.

The golden fixtures were produced by the reference engine itself (tests/golden/make_golden.py);
the oracle must reproduce its statuses and iteration counts exactly and its primal vectors bit
for bit (both round every product and sum separately, in the same order).
"""
import hashlib
import json
import math
import os
import platform
from pathlib import Path

import numpy as np
import pytest

import boxqp
from oracle import oracle as O
from golden_cases import args, inputs

EXACT_HOST = platform.machine() in ('x86_64', 'AMD64')


def digest(x):
    return hashlib.sha256(np.ascontiguousarray(x, np.float64).tobytes()).hexdigest()


def test_fixture_covers_reference_known_answers(golden):
    d, _ = golden
    names = {c['name'] for c in d['cases']}
    assert {'tridiagonal_1000', 'tridiagonal_10000', 'v2_psd_300', 'two_var', 'graph2k_limit60'} <= names
    by = {c['name']: c for c in d['cases']}
    # solver_scale's published known objective for n = 10,000 (-947.124889445...) and 1700 iterations
    assert abs(by['tridiagonal_10000']['objective'] - (-947.124889445)) < 1e-8
    assert by['tridiagonal_10000']['iterations'] == 1700
    # test_solver.cpp:85-90 objective -5; test_v2.cpp:18-25 verified optimal
    assert abs(by['two_var']['objective'] + 5) < 1e-7
    assert by['v2_psd_300']['status'] == 'optimal' and by['v2_psd_300']['verified']
    # QPLIB box instances, objectives published with the reference's CPU benchmark record
    q = {r['name']: r for r in d['qplib']}
    assert q['8792']['objective'] == pytest.approx(3593.5162939294105, rel=1e-12)
    assert q['8991']['objective'] == pytest.approx(-0.0016678673619609664, rel=1e-9)
    assert d['convex'] == {'v2_psd_300': 1, 'v2_indefinite_300': 0}


def test_edge_case_fixtures_have_their_analytic_answers(golden):
    """One variable (min x^2 - 3x on [0, 1]: x = 1, objective -2) and variables with no Hessian
    entries (linear only: at the lower bound where the cost is positive, at the upper where it is
    negative) in the reference's own answers."""
    d, xs = golden
    by = {c['name']: c for c in d['cases']}
    assert by['single_var']['status'] == 'optimal'
    assert xs['single_var'].tolist() == [1.0] and by['single_var']['objective'] == pytest.approx(-2.0, abs=1e-12)
    rec = by['graph2k_zero_rows']
    p, _ = inputs(rec)
    x = xs['graph2k_zero_rows']
    linear = np.arange(len(x)) % rec['generator']['zero_rows_every'] == 0
    assert not np.isin(np.flatnonzero(linear), np.concatenate([p['hrow'], p['hcol']])).any()
    assert rec['status'] == 'optimal'
    assert np.array_equal(x[linear & (p['cost'] > 0)], p['lower'][linear & (p['cost'] > 0)])
    assert np.array_equal(x[linear & (p['cost'] < 0)], p['upper'][linear & (p['cost'] < 0)])


CASE_NAMES = [c['name'] for c in json.loads((Path(__file__).resolve().parent / 'golden' /
                                              'reference_cases.json').read_text())['cases']]


def test_planted_kkt_cases_of_the_reference_scripts(golden):
    """The 15 box cases of the reference's planted KKT tests (scripts/test_qp.py:30-56, n = 5, dense
    PSD Hessian R'R + I, interior planted optimum): the reference's answers pass that script's own
    criteria (status optimal, objective within 1e-6 relative of the planted one, projected-gradient
    residual <= 2e-7, x inside [-3, 3])."""
    d, xs = golden
    recs = [c for c in d['cases'] if c['name'].startswith('kkt5_')]
    assert len(recs) == 15
    for rec in recs:
        p, _ = inputs(rec)
        x = xs[rec['name']]
        n = len(x)
        h = np.zeros((n, n))
        h[p['hrow'], p['hcol']] = p['hval']
        h = h + np.tril(h, -1).T
        expected = rec['expected_objective']
        assert rec['status'] == 'optimal'
        assert abs(rec['objective'] - expected) / (1 + abs(expected)) <= 1e-6
        g = h @ x + p['cost']
        assert np.max(np.abs(x - np.clip(x - g, -3, 3)) / (1 + np.abs(x))) <= 2e-7
        assert np.all((x >= -3) & (x <= 3))
        assert np.max(np.abs(x - np.array(rec['planted_x']))) <= 1e-5


@pytest.mark.parametrize('name', CASE_NAMES)
def test_oracle_matches_reference(golden, name):
    d, xs = golden
    rec = next(c for c in d['cases'] if c['name'] == name)
    p, inst = inputs(rec)
    status, x, st = O.solve_box(*args(p), tol=rec['tol'], iteration_limit=rec['iteration_limit'], time_limit=600,
                                threads=1, maximize=rec['maximize'], offset=rec['offset'])
    assert status == rec['status']
    assert int(st['iterations']) == rec['iterations']
    if EXACT_HOST:
        assert digest(x) == rec['x_sha256']
        assert st['objective'] == rec['objective']
    else:
        assert st['objective'] == pytest.approx(rec['objective'], rel=1e-13, abs=1e-13)
    if rec['name'] in xs:
        ref_x = xs[rec['name']]
        assert np.max(np.abs(x - ref_x)) <= (0 if EXACT_HOST else 1e-12)


def test_oracle_multithreaded_equals_single(golden):
    """OpenMP row partitioning changes no rounding: threads give the same bits."""
    d, _ = golden
    rec = next(c for c in d['cases'] if c['name'] == 'graph10k_s0')
    p, _ = inputs(rec)
    s1, x1, _ = O.solve_box(*args(p), tol=1e-6, threads=1)
    s4, x4, _ = O.solve_box(*args(p), tol=1e-6, threads=4)
    assert s1 == s4 and np.array_equal(x1, x4)


def test_tridiagonal_family_known_objectives():
    """The seeded tridiagonal family of the reference's scale harness (src/scale_benchmark.cpp:
    LCG seed 26119, H = tridiag(-1, 2.02, -1), box [0, 3], known objective in long double) at the
    sizes with published known objectives: n = 10,000 (-947.124889445...), 50,000
    (-4710.360537563), 100,000 (-9446.3140183450014) and 1,000,000 (-94123.887220104109, the
    benchmark size)."""
    assert boxqp.planted('tridiagonal', n=10000)['fstar'] == pytest.approx(-947.124889445, abs=1e-9)
    assert boxqp.planted('tridiagonal', n=50000)['fstar'] == pytest.approx(-4710.360537563, abs=1e-9)
    assert boxqp.planted('tridiagonal', n=100000)['fstar'] == float('-9446.3140183450014')
    assert boxqp.planted('tridiagonal', n=1000000)['fstar'] == float('-94123.887220104109')


def test_oracle_passes_the_scale_harness_at_50k():
    """The scale harness's pass criteria (src/scale_benchmark.cpp:21-23) at n = 50,000: status
    optimal and verified, objective within 1e-8 relative of the known objective, max |x - x*| <
    1e-4 (the reference's own run took 1700 iterations at 10,000, as here)."""
    inst = boxqp.planted('tridiagonal', n=50000, lower_triplets=True)
    status, x, st = O.solve_box(inst['hrow'], inst['hcol'], inst['hval'], inst['c'], inst['lower'], inst['upper'],
                                tol=1e-7, iteration_limit=20000, threads=4)
    assert status == 'optimal' and st['verified'] == 1.0
    assert abs(st['objective'] - inst['fstar']) / (1 + abs(inst['fstar'])) <= 1e-8
    assert np.max(np.abs(x - inst['xstar'])) < 1e-4


def test_planted_optimum_is_verified_by_oracle():
    inst = boxqp.planted('graph10k', seed=5, n=3000, lower_triplets=True)
    p = {'hrow': inst['hrow'], 'hcol': inst['hcol'], 'hval': inst['hval'], 'cost': inst['c'],
         'lower': inst['lower'], 'upper': inst['upper']}
    st = O.check(*args(p), inst['xstar'], tol=1e-12)
    assert st['verified'] == 1.0
    assert st['objective'] == pytest.approx(inst['fstar'], rel=1e-13)


def test_checker_adversarial_cases():
    """The checker trusts nothing: NaN, out-of-box and non-stationary candidates fail."""
    inst = boxqp.planted('graph10k', seed=6, n=500, lower_triplets=True)
    p = {'hrow': inst['hrow'], 'hcol': inst['hcol'], 'hval': inst['hval'], 'cost': inst['c'],
         'lower': inst['lower'], 'upper': inst['upper']}
    x = inst['xstar'].copy()
    x[3] = np.nan
    st = O.check(*args(p), x)
    assert st['verified'] == 0 and math.isnan(st['objective'])
    x = inst['xstar'].copy()
    x[0] = inst['upper'][0] + 0.5
    st = O.check(*args(p), x)
    assert st['primal_residual'] > 0.1 and st['verified'] == 0
    x = inst['xstar'].copy()
    free = np.flatnonzero((x > inst['lower']) & (x < inst['upper']))
    x[free[0]] += 1e-3
    st = O.check(*args(p), x, tol=1e-6)
    assert st['stationarity_residual'] > 1e-6 and st['verified'] == 0


def test_oracle_checker_agrees_with_reference_checker():
    if not O.ref_available():
        pytest.skip('oracle/_ref not built on this host')
    inst = boxqp.planted('grid', seed=9, n=400, lower_triplets=True)
    p = {'hrow': inst['hrow'], 'hcol': inst['hcol'], 'hval': inst['hval'], 'cost': inst['c'],
         'lower': inst['lower'], 'upper': inst['upper']}
    rng = np.random.default_rng(0)
    for scale in (0.0, 1e-8, 1e-4, 1e-1):
        x = np.clip(inst['xstar'] + scale * rng.standard_normal(inst['n']), inst['lower'] - scale, inst['upper'])
        a = O.check(*args(p), x, tol=1e-6)
        b = O.ref_check(*args(p), x, tol=1e-6)
        for k in ('objective', 'primal_residual', 'stationarity_residual', 'dual_bound', 'relative_gap', 'verified'):
            assert a[k] == pytest.approx(b[k], rel=1e-15, abs=1e-300), k


def _dec(v):
    return float(v)


def test_oracle_checker_reproduces_reference_edge_cases():
    """The reference's check_qp_solution on candidates that probe the checker's edges
    (tests/golden/reference_checks.json: tiny curvature on a huge box, out-of-box, NaN and infinite
    candidates, maximisation with an offset, a coupled Hessian with infinite bounds, variables
    without curvature, one-sided and fixed bounds): the oracle's checker returns every residual,
    bound, gap and verdict the reference returned (bit for bit on x86, where long double is the
    same 80-bit type; to 1e-15 elsewhere)."""
    cases = json.loads((Path(__file__).resolve().parent / 'golden' / 'reference_checks.json').read_text())
    assert len(cases) >= 12
    for c in cases:
        p = {k: np.array([_dec(v) for v in vs]) for k, vs in c['problem'].items()}
        p['hrow'] = p['hrow'].astype(np.int64)
        p['hcol'] = p['hcol'].astype(np.int64)
        x = np.array([_dec(v) for v in c['x']])
        st = O.check(*args(p), x, tol=c['tol'], maximize=c['maximize'], offset=c['offset'])
        for k, v in c['result'].items():
            want = _dec(v)
            if math.isnan(want):
                assert math.isnan(st[k]), (c['name'], k)
            elif EXACT_HOST or not math.isfinite(want):
                assert st[k] == want, (c['name'], k, st[k], want)
            else:
                assert st[k] == pytest.approx(want, rel=1e-15, abs=1e-300), (c['name'], k)
    by = {c['name']: c['result'] for c in cases}
    assert by['tiny_curvature_huge_box']['verified'] == 0 and by['tiny_curvature_huge_box']['stationarity_residual'] < 1e-7
    assert by['maximize_optimum']['verified'] == 1 and by['maximize_optimum']['objective'] == 5.0


def test_convexity_gate_matches_the_reference_on_edge_cases():
    """The reference's check_convex_hessian verdicts (tests/golden/reference_convexity.json) on a
    diagonally dominant matrix, a zero diagonal with a coupling, an empty row, a negative
    diagonal, concave and convex maximisations, a singular PSD Gram matrix (its LDL' path), the
    same shifted slightly indefinite, and repeated diagonal terms: the oracle's and the product's
    gate (bqp_check_convex) give the same verdict on each."""
    cases = json.loads((Path(__file__).resolve().parent / 'golden' / 'reference_convexity.json').read_text())
    assert {c['convex'] for c in cases} == {0, 1}
    for c in cases:
        hr, hc, hv = np.array(c['hrow'], np.int64), np.array(c['hcol'], np.int64), np.array(c['hval'])
        assert O.check_convex(c['n'], hr, hc, hv, maximize=c['maximize']) == c['convex'], c['name']
        q = boxqp.QuadraticProblem(cost=np.zeros(c['n']), lower=np.zeros(c['n']), upper=np.ones(c['n']),
                                   hessian_row=hr, hessian_col=hc, hessian_val=hv, maximize=c['maximize'])
        assert boxqp.check_convex_hessian(q) == bool(c['convex']), c['name']


def test_oracle_convexity_matches_reference(golden):
    d, _ = golden
    p, _ = inputs(next(c for c in d['cases'] if c['name'] == 'v2_psd_300'))
    assert O.check_convex(300, p['hrow'], p['hcol'], p['hval']) == d['convex']['v2_psd_300']
    bad = p['hval'].copy()
    bad[0] = -1.0
    assert O.check_convex(300, p['hrow'], p['hcol'], bad) == d['convex']['v2_indefinite_300']


@pytest.mark.skipif(not os.environ.get('BOXQP_REFERENCE_DIR'), reason='set BOXQP_REFERENCE_DIR to the reference solver')
def test_oracle_on_qplib_box_instances(golden):
    """QPLIB 8792 / 8991 read by the reference's reader, solved by the oracle."""
    d, _ = golden
    if not O.ref_available():
        pytest.skip('oracle/_ref not built')
    data = Path(os.environ['BOXQP_REFERENCE_DIR']) / 'datasets' / 'qplib'
    for rec in d['qplib']:
        q = O.ref_read_qplib(data / f"{rec['name']}.qplib")
        status, x, st = O.solve_box(q['hrow'], q['hcol'], q['hval'], q['cost'], q['lower'], q['upper'], tol=1e-7,
                                    time_limit=600, maximize=q['maximize'], offset=q['offset'])
        assert status == rec['status'] and int(st['iterations']) == rec['iterations']
        assert st['objective'] == pytest.approx(rec['objective'], rel=1e-12)
