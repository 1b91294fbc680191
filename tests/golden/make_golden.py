"""Generates the golden fixtures of the box-QP path from the reference itself.

Run from the repository root where the reference checkout exists:
    python tests/golden/make_golden.py [--reference /root/reference/02-software/solver]

It builds oracle/_ref (the reference's unmodified solver sources + oracle/ref_shim.cpp, see
oracle/ref.mk), runs the reference's own CPU engine solve_accelerated_box(q, opt, false) and
checker on each case below, and writes
    tests/golden/reference_cases.json   statuses, iterations, objectives, residuals, x digests
    tests/golden/reference_x.npz        primal vectors of the cases with n <= 2000
The cases are the reference's known answers for this path (its tests and published harness)
plus planted instances of the synthetic families.  tests/golden/reference_admm.npz holds the
reference's ADMM (solve_qp_admm) after a few iterations on small constrained QPs and
reference_admm_adapt.npz after 120-230 iterations, across its rho adaptation (--only admm
regenerates just those two files).  QPLIB instances are read from the
reference's datasets folder by the reference's own reader; only scalar results and the input
file's SHA-256 are stored.
"""
import argparse
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / 'hypergrey-sih-26_gb300'))

import boxqp  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def digest(x):
    return hashlib.sha256(np.ascontiguousarray(x, np.float64).tobytes()).hexdigest()


def v2_psd_case():
    """src/tests/test_v2.cpp:18-25: n=300, PSD, not diagonally dominant."""
    n = 300
    hr, hc, hv = [], [], []
    for j in range(n):
        hr.append(j); hc.append(j); hv.append(5.0 if j % 2 else 1.0)
        if j % 2:
            hr.append(j); hc.append(j - 1); hv.append(2.0)
    return dict(hrow=np.array(hr), hcol=np.array(hc), hval=np.array(hv), cost=-np.ones(n), lower=np.zeros(n),
                upper=np.full(n, 10.0))


def two_var_case():
    """src/tests/test_solver.cpp:85-90: objective -5."""
    return dict(hrow=np.array([0, 1]), hcol=np.array([0, 1]), hval=np.array([2.0, 2.0]), cost=np.array([-2.0, -4.0]),
                lower=np.array([-10.0, -10.0]), upper=np.array([10.0, 10.0]))


def cases():
    out = []
    for seed in range(4):
        inst = boxqp.planted('graph10k', seed=seed, lower_triplets=True)
        out.append((f'graph10k_s{seed}', inst, dict(tol=1e-6), {'preset': 'graph10k', 'seed': seed}))
    for seed in range(6):
        inst = boxqp.planted('graph10k', seed=100 + seed, n=2000, lower_triplets=True)
        out.append((f'graph2k_s{100 + seed}', inst, dict(tol=1e-6), {'preset': 'graph10k', 'seed': 100 + seed, 'n': 2000}))
    inst = boxqp.planted('graph10k', seed=7, n=2000, lower_triplets=True)
    out.append(('graph2k_tol1e-8', inst, dict(tol=1e-8), {'preset': 'graph10k', 'seed': 7, 'n': 2000}))
    out.append(('graph2k_limit60', inst, dict(tol=1e-9, iteration_limit=60), {'preset': 'graph10k', 'seed': 7, 'n': 2000}))
    out.append(('graph2k_limit0', inst, dict(tol=1e-9, iteration_limit=0), {'preset': 'graph10k', 'seed': 7, 'n': 2000}))
    for n in (1000, 10000):
        inst = boxqp.planted('tridiagonal', n=n, lower_triplets=True)
        # solver_scale's options: iteration_limit 20000, tolerance 1e-7 (src/scale_benchmark.cpp:19)
        out.append((f'tridiagonal_{n}', inst, dict(tol=1e-7, iteration_limit=20000), {'preset': 'tridiagonal', 'n': n}))
    for tol in (1e-6, 1e-8):
        inst = boxqp.planted('grid', seed=2, n=32 * 32, lower_triplets=True)
        out.append((f'grid32_tol{tol:g}', inst, dict(tol=tol), {'preset': 'grid', 'seed': 2, 'n': 1024}))
    for seed in range(3):
        inst = boxqp.planted('batch', seed=3, index=seed, lower_triplets=True)
        out.append((f'batch_i{seed}', inst, dict(tol=1e-6), {'preset': 'batch', 'seed': 3, 'index': seed}))
    return out


def run_case(name, p, opts, maximize=False, offset=0.0):
    args = (p['hrow'], p['hcol'], p['hval'], p['cost'] if 'cost' in p else p['c'], p['lower'], p['upper'])
    status, x, st = O.ref_solve_box(*args, tol=opts.get('tol', 1e-7), iteration_limit=opts.get('iteration_limit', 200000),
                                    time_limit=600.0, threads=1, maximize=maximize, offset=offset)
    rec = {'name': name, 'status': status, 'iterations': int(st['iterations']), 'objective': st['objective'],
           'stationarity_residual': st['stationarity_residual'], 'primal_residual': st['primal_residual'],
           'relative_gap': st['relative_gap'], 'dual_bound': st['dual_bound'], 'verified': bool(st['verified']),
           'x_sha256': digest(x), 'n': int(len(x)), 'tol': opts.get('tol', 1e-7),
           'iteration_limit': opts.get('iteration_limit', 200000), 'maximize': maximize, 'offset': offset}
    return rec, x


def admm_case(seed, n, m, equality_rows):
    """A constrained QP for the reference's ADMM: lower-triangle Hessian (diagonal U[2,4] plus 3n/2
    off-diagonal terms U[-0.5,0.5]), bounds [-1, 1], m rows of 4 normal entries with bounds
    [-U[0.1,0.5], U[0.1,0.5]] (the first `equality_rows` of them equalities at 0.1)."""
    rng = np.random.default_rng(seed)
    hrow, hcol, hval = [], [], []
    for i in range(n):
        hrow.append(i)
        hcol.append(i)
        hval.append(float(rng.uniform(2, 4)))
    for _ in range(3 * n // 2):
        i, j = sorted(rng.choice(n, 2, replace=False).tolist())[::-1]
        hrow.append(i)
        hcol.append(j)
        hval.append(float(rng.uniform(-0.5, 0.5)))
    rowptr, col, val = [0], [], []
    for _ in range(m):
        cs = np.sort(rng.choice(n, 4, replace=False))
        col += cs.tolist()
        val += rng.normal(size=4).tolist()
        rowptr.append(len(col))
    row_lower = -rng.uniform(0.1, 0.5, m)
    row_upper = rng.uniform(0.1, 0.5, m)
    row_lower[:equality_rows] = 0.1
    row_upper[:equality_rows] = 0.1
    return {'n': n, 'hrow': np.array(hrow, np.int64), 'hcol': np.array(hcol, np.int64), 'hval': np.array(hval),
            'cost': rng.normal(size=n), 'lower': -np.ones(n), 'upper': np.ones(n),
            'a_rowptr': np.array(rowptr, np.int32), 'a_col': np.array(col, np.int32), 'a_val': np.array(val),
            'row_lower': row_lower, 'row_upper': row_upper}


def make_admm_golden():
    """The reference's solve_qp_admm (src/qp_admm.cpp:118-280) after a few ADMM iterations (below its
    first rho adaptation and polish) on small constrained QPs: tests/golden/reference_admm.npz;
    and after 120-230 iterations (across the rho adaptation): reference_admm_adapt.npz."""
    out = {}
    for name, (seed, n, m, eq, its, scaling) in {'admm_a': (7, 40, 25, 0, 20, True),
                                                  'admm_b': (8, 120, 60, 10, 12, True),
                                                  'admm_c': (9, 80, 50, 5, 8, False),
                                                  'admm_d': (10, 300, 150, 30, 15, True),
                                                  'admm_e': (11, 200, 120, 0, 30, True)}.items():
        p = admm_case(seed, n, m, eq)
        status, x, st = O.ref_solve_qp_admm(p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'],
                                            p['a_rowptr'], p['a_col'], p['a_val'], p['row_lower'], p['row_upper'],
                                            tol=1e-12, iteration_limit=its, scaling=scaling)
        assert status == 'iteration_limit' and int(st['iterations']) == its, (name, status, st)
        for k, v in p.items():
            out[f'{name}.{k}'] = np.asarray(v)
        out[f'{name}.iterations'] = np.array(its)
        out[f'{name}.scaling'] = np.array(1 if scaling else 0)
        out[f'{name}.x'] = x
        print(name, status, its, float(np.max(np.abs(x))), flush=True)
    np.savez_compressed(OUT / 'reference_admm.npz', **out)
    # longer runs that cross the rho adaptation at iterations 100 and 200 (src/qp_admm.cpp:265-271),
    # still below the first polish (250): tests/golden/reference_admm_adapt.npz
    out = {}
    for name, (seed, n, m, eq, its, scaling) in {'admm_f': (12, 60, 40, 0, 150, True),
                                                  'admm_g': (13, 100, 70, 8, 230, True),
                                                  'admm_h': (14, 50, 30, 4, 120, False),
                                                  'admm_i': (15, 150, 90, 0, 210, True)}.items():
        p = admm_case(seed, n, m, eq)
        status, x, st = O.ref_solve_qp_admm(p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'],
                                            p['a_rowptr'], p['a_col'], p['a_val'], p['row_lower'], p['row_upper'],
                                            tol=1e-12, iteration_limit=its, scaling=scaling)
        assert status == 'iteration_limit' and int(st['iterations']) == its, (name, status, st)
        out.update({f'{name}.{k}': np.asarray(v) for k, v in p.items()})
        out[f'{name}.iterations'] = np.array(its)
        out[f'{name}.scaling'] = np.array(1 if scaling else 0)
        out[f'{name}.x'] = x
        print(name, status, its, float(np.max(np.abs(x))), flush=True)
    np.savez_compressed(OUT / 'reference_admm_adapt.npz', **out)
    make_admm_solve_golden()


def admm_rows_case(seed, n=40, m=30):
    """A constrained QP whose rows exercise the reference's row handling: columns out of order,
    repeated columns (summed), a pair that cancels to zero (dropped), an empty row, rows with an
    infinite lower or upper bound, and three equality rows; Hessian and box as admm_case."""
    p = admm_case(seed, n, 0, 0)
    rng = np.random.default_rng(seed + 1000)
    rowptr, col, val = [0], [], []
    for i in range(m):
        if i == 5:
            rowptr.append(len(col))  # empty row
            continue
        cs = rng.choice(n, int(rng.integers(3, 6)), replace=False).tolist()
        vs = rng.normal(size=len(cs)).tolist()
        if i % 4 == 1:  # a repeated column
            cs.append(cs[0])
            vs.append(float(rng.normal()))
        if i == 7:  # a repeated column that cancels
            cs += [cs[1]]
            vs += [-vs[1]]
        col += cs
        val += vs
        rowptr.append(len(col))
    lo = -rng.uniform(0.1, 0.5, m)
    up = rng.uniform(0.1, 0.5, m)
    lo[1::6] = -np.inf
    up[2::6] = np.inf
    lo[3:6], up[3:6] = 0.05, 0.05
    lo[5], up[5] = -1.0, 1.0  # the empty row
    p.update({'a_rowptr': np.array(rowptr, np.int32), 'a_col': np.array(col, np.int32), 'a_val': np.array(val),
              'row_lower': lo, 'row_upper': up})
    return p


def diagonal_equality_case(seed, n=80, m=30):
    """A QP with a positive diagonal Hessian (U[1, 3]) and m equality rows of 4 normal entries,
    right-hand sides A x0 for an x0 inside the box [-1, 1]: the structure solve_qp_admm hands to
    its dual Newton solver first."""
    rng = np.random.default_rng(seed)
    rowptr, col, val = [0], [], []
    for _ in range(m):
        cs = np.sort(rng.choice(n, 4, replace=False))
        col += cs.tolist()
        val += rng.normal(size=4).tolist()
        rowptr.append(len(col))
    hval = rng.uniform(1, 3, n)
    rowptr, col, val = np.array(rowptr, np.int32), np.array(col, np.int32), np.array(val)
    x0 = rng.uniform(-0.5, 0.5, n)
    b = np.array([float(np.dot(val[rowptr[i]:rowptr[i + 1]], x0[col[rowptr[i]:rowptr[i + 1]]])) for i in range(m)])
    return {'n': n, 'hrow': np.arange(n, dtype=np.int64), 'hcol': np.arange(n, dtype=np.int64), 'hval': hval,
            'cost': 3 * rng.normal(size=n), 'lower': -np.ones(n), 'upper': np.ones(n), 'a_rowptr': rowptr,
            'a_col': col, 'a_val': val, 'row_lower': b, 'row_upper': b.copy()}


def make_dual_newton_golden():
    """The reference's solve_diagonal_equalities (src/qp_dual_newton.cpp:9-66) on diagonal-Hessian
    equality QPs: verified solves (scaled and unscaled) and a run stopped after 3 iterations with an
    unreachable tolerance: tests/golden/reference_dual_newton.npz."""
    out = {}
    for name, (seed, tol, limit, scaling) in {'dn_a': (50, 1e-7, 200000, True), 'dn_b': (51, 1e-8, 200000, False),
                                              'dn_c': (52, 1e-300, 3, True), 'dn_d': (53, 1e-7, 200000, True)}.items():
        p = diagonal_equality_case(seed)
        a = (p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], p['a_rowptr'], p['a_col'],
             p['a_val'], p['row_lower'], p['row_upper'])
        status, x, st = O.ref_solve_diagonal_equalities(*a, tol=tol, iteration_limit=limit, scaling=scaling)
        out.update({f'{name}.{k}': np.asarray(v) for k, v in p.items()})
        out[f'{name}.tol'] = np.array(tol)
        out[f'{name}.limit'] = np.array(limit)
        out[f'{name}.scaling'] = np.array(1 if scaling else 0)
        out[f'{name}.status'] = np.array(status)
        out[f'{name}.iterations'] = np.array(int(st['iterations']))
        out[f'{name}.x'] = x
        out[f'{name}.row_dual'] = st['row_dual']
        out[f'{name}.stats'] = np.array([st[k] for k in CHECK_KEYS])
        print(name, status, int(st['iterations']), st['objective'], flush=True)
    np.savez_compressed(OUT / 'reference_dual_newton.npz', **out)


ADMM_SOLVE_CASES = {'solve_20': (20, 60, 40, 0, 1e-6), 'solve_21': (21, 100, 70, 8, 1e-6),
                    'solve_22': (22, 50, 30, 4, 1e-5), 'solve_23': (23, 150, 90, 0, 1e-5),
                    'solve_26': (26, 50, 30, 4, 1e-4), 'solve_29': (29, 100, 70, 8, 1e-6)}


def make_admm_solve_golden():
    """The reference's whole solve_qp_admm (src/qp_admm.cpp:118-280, scaled, default limits) on
    constrained QPs that it verifies before its first polish: status, iterations, primal, row
    duals and the checker's fields; and its check_qp_solution on candidates around each answer
    (the answer, a perturbed primal, zero row duals): tests/golden/reference_admm_solve.npz."""
    out = {}
    for name, (seed, n, m, eq, tol) in ADMM_SOLVE_CASES.items():
        p = admm_case(seed, n, m, eq)
        a = (p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], p['a_rowptr'], p['a_col'],
             p['a_val'], p['row_lower'], p['row_upper'])
        status, x, st = O.ref_solve_qp_admm(*a, tol=tol, iteration_limit=200000, time_limit=600.0, scaling=True)
        assert status == 'optimal' and st['iterations'] < 250, (name, status, st)
        out.update({f'{name}.{k}': np.asarray(v) for k, v in p.items()})
        out[f'{name}.tol'] = np.array(tol)
        out[f'{name}.iterations'] = np.array(int(st['iterations']))
        out[f'{name}.x'] = x
        out[f'{name}.row_dual'] = st['row_dual']
        out[f'{name}.stats'] = np.array([st[k] for k in CHECK_KEYS])
        rng = np.random.default_rng(seed)
        cands = [(x, st['row_dual']), (x + 1e-3 * rng.standard_normal(n), st['row_dual']), (x, np.zeros(m))]
        for k, (cx, cy) in enumerate(cands):
            chk = O.ref_check_rows(*a, cx, cy, tol=tol)
            out[f'{name}.cand{k}_x'] = cx
            out[f'{name}.cand{k}_y'] = cy
            out[f'{name}.cand{k}_stats'] = np.array([chk[k2] for k2 in CHECK_KEYS])
        print(name, status, int(st['iterations']), st['objective'], flush=True)
    np.savez_compressed(OUT / 'reference_admm_solve.npz', **out)
    # row handling: the reference's primal after 20 iterations and its whole solve
    out = {}
    for name, seed in (('rows_a', 40), ('rows_b', 41)):
        p = admm_rows_case(seed)
        a = (p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], p['a_rowptr'], p['a_col'],
             p['a_val'], p['row_lower'], p['row_upper'])
        out.update({f'{name}.{k}': np.asarray(v) for k, v in p.items()})
        status, x, st = O.ref_solve_qp_admm(*a, tol=1e-12, iteration_limit=20, time_limit=600.0)
        assert status == 'iteration_limit', (name, status)
        out[f'{name}.x20'] = x
        out[f'{name}.y20'] = st['row_dual']
        status, x, st = O.ref_solve_qp_admm(*a, tol=1e-5, iteration_limit=200000, time_limit=600.0)
        out[f'{name}.status'] = np.array(status)
        out[f'{name}.iterations'] = np.array(int(st['iterations']))
        out[f'{name}.x'] = x
        out[f'{name}.row_dual'] = st['row_dual']
        out[f'{name}.stats'] = np.array([st[k] for k in CHECK_KEYS])
        print(name, status, int(st['iterations']), st['objective'], flush=True)
    # a maximisation (concave objective: the Hessian and cost of admm_case negated) with an offset
    p = admm_case(24, 60, 40, 4)
    p['hval'] = -p['hval']
    p['cost'] = -p['cost']
    a = (p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], p['a_rowptr'], p['a_col'], p['a_val'],
         p['row_lower'], p['row_upper'])
    status, x, st = O.ref_solve_qp_admm(*a, tol=1e-5, iteration_limit=200000, time_limit=600.0, maximize=True,
                                        offset=1.5)
    out.update({f'max_a.{k}': np.asarray(v) for k, v in p.items()})
    out['max_a.maximize'] = np.array(1)
    out['max_a.offset'] = np.array(1.5)
    out['max_a.status'] = np.array(status)
    out['max_a.iterations'] = np.array(int(st['iterations']))
    out['max_a.x'] = x
    out['max_a.row_dual'] = st['row_dual']
    out['max_a.stats'] = np.array([st[k] for k in CHECK_KEYS])
    print('max_a', status, int(st['iterations']), st['objective'], flush=True)
    # no linear rows: the ADMM over the bound rows alone
    p = admm_case(25, 50, 0, 0)
    a = (p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], p['a_rowptr'], p['a_col'], p['a_val'],
         p['row_lower'], p['row_upper'])
    status, x, st = O.ref_solve_qp_admm(*a, tol=1e-6, iteration_limit=200000, time_limit=600.0)
    out.update({f'box_a.{k}': np.asarray(v) for k, v in p.items()})
    out['box_a.status'] = np.array(status)
    out['box_a.iterations'] = np.array(int(st['iterations']))
    out['box_a.x'] = x
    out['box_a.row_dual'] = st['row_dual']
    out['box_a.stats'] = np.array([st[k] for k in CHECK_KEYS])
    print('box_a', status, int(st['iterations']), st['objective'], flush=True)
    np.savez_compressed(OUT / 'reference_admm_rows.npz', **out)


OPEN_CASES = [('graph2k_open', {'preset': 'graph10k', 'seed': 300, 'n': 2000, 'open_bounds': 3}, dict(tol=1e-6)),
              ('grid32_open', {'preset': 'grid', 'seed': 4, 'n': 1024, 'open_bounds': 2}, dict(tol=1e-7)),
              ('graph2k_fixed', {'preset': 'graph10k', 'seed': 301, 'n': 2000, 'fixed_every': 5}, dict(tol=1e-6)),
              ('graph2k_zero_rows', {'preset': 'graph10k', 'seed': 302, 'n': 2000, 'zero_rows_every': 7},
               dict(tol=1e-6))]


def update_open_cases():
    """One-sided boxes (infinite lower or upper bounds on a share of the variables), fixed
    variables (l = u), variables with no Hessian entries, a one-variable problem and the planted
    KKT box cases of the reference's scripts (planted_kkt_cases), run by the reference and merged
    into reference_cases.json / reference_x.npz."""
    sys.path.insert(0, str(OUT.parent))
    from golden_cases import inputs
    d = json.loads((OUT / 'reference_cases.json').read_text())
    xs = dict(np.load(OUT / 'reference_x.npz'))
    for name, gen, opts in OPEN_CASES:
        p, inst = inputs({'generator': gen})
        rec, x = run_case(name, p, opts)
        rec['generator'] = gen
        rec['fstar'] = None
        d['cases'] = [c for c in d['cases'] if c['name'] != name] + [rec]
        xs[name] = x
        print(name, rec['status'], rec['iterations'], rec['objective'], flush=True)
    # one variable: min x^2 - 3x on [0, 1] (the unconstrained minimiser 1.5 is clipped to 1)
    single = {'hrow': np.array([0], np.int64), 'hcol': np.array([0], np.int64), 'hval': np.array([2.0]),
              'cost': np.array([-3.0]), 'lower': np.array([0.0]), 'upper': np.array([1.0])}
    rec, x = run_case('single_var', single, dict(tol=1e-9))
    rec['problem'] = {k: np.asarray(v).tolist() for k, v in single.items()}
    d['cases'] = [c for c in d['cases'] if c['name'] != 'single_var'] + [rec]
    xs['single_var'] = x
    print('single_var', rec['status'], rec['iterations'], rec['objective'], x, flush=True)
    for rec, x in planted_kkt_cases():
        d['cases'] = [c for c in d['cases'] if c['name'] != rec['name']] + [rec]
        xs[rec['name']] = x
    (OUT / 'reference_cases.json').write_text(json.dumps(d, indent=1) + '\n')
    np.savez_compressed(OUT / 'reference_x.npz', **xs)


CHECK_KEYS = ('objective', 'primal_residual', 'stationarity_residual', 'complementarity_residual', 'dual_bound',
              'relative_gap', 'verified')


def check_cases():
    """Candidates that probe the checker's edges (after the adversarial tests of the reference's
    independent certificate, scripts/test_qp_certificate.py:17-49, restated for a box QP): each is
    (name, problem, candidate x, maximize, offset, tol)."""
    inf = float('inf')
    nan = float('nan')

    def prob(terms, c, lo, up):
        return {'hrow': [t[0] for t in terms], 'hcol': [t[1] for t in terms], 'hval': [t[2] for t in terms],
                'cost': c, 'lower': lo, 'upper': up}
    diag2 = prob([(0, 0, 2.0), (1, 1, 2.0)], [-1.0, -1.0], [-1.0, -1.0], [1.0, 1.0])
    concave = prob([(0, 0, -2.0), (1, 1, -2.0)], [2.0, 2.0], [-5.0, -5.0], [5.0, 5.0])
    coupled = prob([(0, 0, 2.0), (1, 0, 1.0), (1, 1, 2.0)], [1.0, 1.0], [-inf, -inf], [inf, inf])
    return [
        # tiny curvature, huge box: the projected gradient is small, the separable dual bound is not
        ('tiny_curvature_huge_box', prob([(0, 0, 1e-16), (1, 1, 1.0)], [0.0, 0.0], [-1e12, -1.0], [1e12, 1.0]),
         [1e8, 0.0], False, 0.0, 1e-7),
        ('diagonal_optimum', diag2, [0.5, 0.5], False, 0.0, 1e-7),
        ('out_of_box', diag2, [2.0, 0.0], False, 0.0, 1e-7),
        ('non_finite', diag2, [nan, 0.0], False, 0.0, 1e-7),
        ('infinite_candidate', diag2, [inf, 0.0], False, 0.0, 1e-7),
        # maximisation with an offset: the bound is reported in the minimisation sense
        ('maximize_optimum', concave, [1.0, 1.0], True, 3.0, 1e-7),
        ('maximize_nonstationary', concave, [0.5, 1.5], True, 3.0, 1e-7),
        # coupled Hessian, free variables: tangent bound toward an infinite bound
        ('coupled_free_near', coupled, [-1 / 3 + 1e-3, -1 / 3], False, 0.0, 1e-7),
        ('coupled_free_optimum', coupled, [-1 / 3, -1 / 3], False, 0.0, 1e-7),
        # a variable without curvature (no positive diagonal): verified by stationarity alone
        ('linear_variable', prob([(1, 1, 1.0)], [1.0, -1.0], [0.0, 0.0], [1.0, 1.0]), [0.0, 1.0], False, 0.0, 1e-7),
        ('one_sided_bounds', prob([(0, 0, 1.0), (1, 1, 1.0)], [1.0, -3.0], [0.0, -inf], [inf, 2.0]), [0.0, 2.0],
         False, 0.0, 1e-7),
        ('fixed_variable', prob([(0, 0, 1.0), (1, 0, 0.5), (1, 1, 1.0)], [0.0, -1.0], [0.25, -2.0], [0.25, 2.0]),
         [0.25, 0.875], False, 0.0, 1e-7),
    ]


def convexity_cases():
    """Hessians (lower-triangle triplets) at the edges of the reference's convexity gate
    (src/qp_admm.cpp:30-62): (name, n, terms, maximize)."""
    rng = np.random.default_rng(77)
    n = 30
    r = rng.normal(size=(8, n))
    gram = r.T @ r  # rank 8: PSD, singular, not diagonally dominant
    low = [(i, j, float(gram[i, j])) for i in range(n) for j in range(i + 1) if gram[i, j] != 0]
    shifted = [(i, j, v - (1e-3 if i == j else 0.0)) for i, j, v in low]  # slightly indefinite
    return [
        ('dominant', 3, [(0, 0, 2.0), (1, 0, -1.0), (1, 1, 2.0), (2, 1, -1.0), (2, 2, 2.0)], False),
        ('zero_diagonal_coupled', 2, [(0, 0, 0.0), (1, 0, 0.5), (1, 1, 1.0)], False),
        ('zero_row', 3, [(1, 1, 1.0), (2, 2, 1.0)], False),
        ('negative_diagonal', 2, [(0, 0, -1.0), (1, 1, 1.0)], False),
        ('concave_maximised', 2, [(0, 0, -2.0), (1, 0, 0.5), (1, 1, -2.0)], True),
        ('convex_maximised', 2, [(0, 0, 2.0), (1, 1, 2.0)], True),
        ('psd_singular_gram', n, low, False),
        ('indefinite_gram_shift', n, shifted, False),
        ('repeated_diagonal_terms', 2, [(0, 0, 1.0), (0, 0, 1.0), (1, 0, -1.9), (1, 1, 2.0)], False),
    ]


def make_check_golden():
    """The reference's check_qp_solution (src/qp_admm.cpp:63-117) on check_cases():
    tests/golden/reference_checks.json (non-finite numbers as the strings 'nan', 'inf', '-inf')."""
    def enc(v):
        return v if np.isfinite(v) else ('nan' if np.isnan(v) else ('inf' if v > 0 else '-inf'))
    out = []
    for name, p, x, maximize, offset, tol in check_cases():
        st = O.ref_check(p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], np.array(x), tol=tol,
                         maximize=maximize, offset=offset)
        out.append({'name': name, 'problem': {k: [enc(v) for v in vs] for k, vs in p.items()},
                    'x': [enc(v) for v in x], 'maximize': maximize, 'offset': offset, 'tol': tol,
                    'result': {k: enc(st[k]) for k in CHECK_KEYS}})
        print(name, {k: st[k] for k in CHECK_KEYS}, flush=True)
    (OUT / 'reference_checks.json').write_text(json.dumps(out, indent=1) + '\n')
    conv = []
    for name, n, terms, maximize in convexity_cases():
        hr = np.array([t[0] for t in terms], np.int64)
        hc = np.array([t[1] for t in terms], np.int64)
        hv = np.array([t[2] for t in terms])
        verdict = O.ref_check_convex(n, hr, hc, hv, maximize=maximize)
        conv.append({'name': name, 'n': n, 'hrow': hr.tolist(), 'hcol': hc.tolist(), 'hval': hv.tolist(),
                     'maximize': maximize, 'convex': int(verdict)})
        print('convex', name, verdict, flush=True)
    (OUT / 'reference_convexity.json').write_text(json.dumps(conv, indent=1) + '\n')


def _planted_kkt_draws():
    """The 30 problems of the reference's planted KKT tests (scripts/test_qp.py:30-44), drawn from
    one random.Random(26121) stream in the script's order: n = 5, H = R'R + I, x* uniform in
    [-1, 1], and for cases 15-29 three rows a (uniform in [-1, 1]) with duals y in [0.2, 2]
    active at x* (a x <= b, b = a x*), c = -H x* - A'y; box [-3, 3]."""
    import random
    rng = random.Random(26121)
    out = []
    for case in range(30):
        n = 5
        m = 3 if case >= 15 else 0
        r = [[rng.uniform(-1, 1) for _ in range(n)] for _ in range(n)]
        h = [[sum(r[k][i] * r[k][j] for k in range(n)) + (1 if i == j else 0) for j in range(n)] for i in range(n)]
        optimum = [rng.uniform(-1, 1) for _ in range(n)]
        a = [[rng.uniform(-1, 1) for _ in range(n)] for _ in range(m)]
        y = [rng.uniform(.2, 2) for _ in range(m)]
        b = [sum(v * x for v, x in zip(row, optimum)) for row in a]
        c = [-sum(h[i][j] * optimum[j] for j in range(n)) - sum(a[k][i] * y[k] for k in range(m)) for i in range(n)]
        expected = sum(c[i] * optimum[i] + .5 * sum(h[i][j] * optimum[i] * optimum[j] for j in range(n))
                       for i in range(n))
        out.append((case, n, h, optimum, a, b, c, expected))
    return out


def diagonal_inequality_case(seed, n=40, m=25, eq=3):
    """A QP with a positive diagonal Hessian (U[2, 4]) and m rows of 4 normal entries, bounds
    [-U[0.1, 0.5], U[0.1, 0.5]], the first `eq` equalities at 0.1; box [-1, 1].  Its rows are not all
    equalities, so solve_qp_admm skips its dual Newton pre-solver and polishes in the
    diagonal-Hessian form."""
    rng = np.random.default_rng(seed)
    rowptr, col, val = [0], [], []
    for _ in range(m):
        cs = np.sort(rng.choice(n, 4, replace=False))
        col += cs.tolist()
        val += rng.normal(size=4).tolist()
        rowptr.append(len(col))
    lo = -rng.uniform(0.1, 0.5, m)
    up = rng.uniform(0.1, 0.5, m)
    lo[:eq] = 0.1
    up[:eq] = 0.1
    return {'n': n, 'hrow': np.arange(n, dtype=np.int64), 'hcol': np.arange(n, dtype=np.int64),
            'hval': rng.uniform(2, 4, n), 'cost': 2 * rng.normal(size=n), 'lower': -np.ones(n), 'upper': np.ones(n),
            'a_rowptr': np.array(rowptr, np.int32), 'a_col': np.array(col, np.int32), 'a_val': np.array(val),
            'row_lower': lo, 'row_upper': up}


def make_polish_golden():
    """The reference's solve_qp_admm on diagonal-Hessian QPs with inequality rows at tolerances its
    ADMM does not reach by iteration 250, where its KKT polish (diagonal-Hessian form) verifies:
    tests/golden/reference_admm_polish.npz."""
    out = {}
    for name, (seed, tol) in {'pol_a': (60, 1e-9), 'pol_b': (62, 1e-10), 'pol_c': (65, 1e-9)}.items():
        p = diagonal_inequality_case(seed)
        a = (p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper'], p['a_rowptr'], p['a_col'],
             p['a_val'], p['row_lower'], p['row_upper'])
        status, x, st = O.ref_solve_qp_admm(*a, tol=tol, time_limit=600.0)
        out.update({f'{name}.{k}': np.asarray(v) for k, v in p.items()})
        out[f'{name}.tol'] = np.array(tol)
        out[f'{name}.status'] = np.array(status)
        out[f'{name}.iterations'] = np.array(int(st['iterations']))
        out[f'{name}.x'] = x
        out[f'{name}.row_dual'] = st['row_dual']
        out[f'{name}.stats'] = np.array([st[k] for k in CHECK_KEYS])
        print(name, status, int(st['iterations']), st['objective'], flush=True)
    np.savez_compressed(OUT / 'reference_admm_polish.npz', **out)


def make_kkt_rows_golden():
    """Cases 15-29 of the reference's planted KKT tests (three inequality rows each) through the
    reference's solve_qp_admm with default options: tests/golden/reference_kkt_rows.json (the
    problems, the script's expected objectives and the reference's answers)."""
    recs = []
    for case, n, h, optimum, a, b, c, expected in _planted_kkt_draws()[15:]:
        terms = [(i, j, h[i][j]) for i in range(n) for j in range(i + 1) if h[i][j] != 0]
        m = len(a)
        rowptr = [n * i for i in range(m + 1)]
        col = [j for _ in range(m) for j in range(n)]
        val = [v for row in a for v in row]
        status, x, st = O.ref_solve_qp_admm(np.array([t[0] for t in terms]), np.array([t[1] for t in terms]),
                                            np.array([t[2] for t in terms]), np.array(c), np.full(n, -3.0),
                                            np.full(n, 3.0), np.array(rowptr, np.int32), np.array(col, np.int32),
                                            np.array(val), np.full(m, -np.inf), np.array(b), tol=1e-7,
                                            time_limit=600.0)
        recs.append({'case': case, 'hrow': [t[0] for t in terms], 'hcol': [t[1] for t in terms],
                     'hval': [t[2] for t in terms], 'cost': c, 'a_rowptr': rowptr, 'a_col': col, 'a_val': val,
                     'row_upper': b, 'expected_objective': expected, 'planted_x': optimum, 'status': status,
                     'iterations': int(st['iterations']), 'objective': st['objective'], 'x': x.tolist(),
                     'row_dual': st['row_dual'].tolist()})
        print('kkt_rows', case, status, int(st['iterations']), st['objective'], expected, flush=True)
    (OUT / 'reference_kkt_rows.json').write_text(json.dumps(recs, indent=1) + '\n')


def planted_kkt_cases():
    """The box cases 0-14 of the reference's planted KKT tests (scripts/test_qp.py:30-56): n = 5,
    H = R'R + I with R uniform in [-1, 1], x* uniform in [-1, 1], c = -H x*, box [-3, 3] (x* is
    interior, so the expected objective is c'x* + x*'H x*/2), drawn from one random.Random(26121)
    stream in the order the script draws them.  The script writes each as a QPLIB file for the
    reference's CLI, which sends a box QP to solve_accelerated_box with the default options
    (tolerance 1e-7); here the same lower-triangle terms go to it directly.  Each record keeps
    the script's expected objective."""
    out = []
    for case, n, h, optimum, _, _, c, expected in _planted_kkt_draws()[:15]:
        terms = [(i, j, h[i][j]) for i in range(n) for j in range(i + 1) if h[i][j] != 0]
        prob = {'hrow': np.array([t[0] for t in terms], np.int64), 'hcol': np.array([t[1] for t in terms], np.int64),
                'hval': np.array([t[2] for t in terms]), 'cost': np.array(c), 'lower': np.full(n, -3.0),
                'upper': np.full(n, 3.0)}
        name = f'kkt5_{case:02d}'
        rec, x = run_case(name, prob, dict(tol=1e-7))
        rec['problem'] = {k: np.asarray(v).tolist() for k, v in prob.items()}
        rec['expected_objective'] = expected
        rec['planted_x'] = optimum
        out.append((rec, x))
        print(name, rec['status'], rec['iterations'], rec['objective'], expected, flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default='/root/reference/02-software/solver')
    ap.add_argument('--only', choices=['admm', 'open'], default=None,
                    help='regenerate only the constrained-QP fixtures (ADMM, dual Newton, checker, KKT rows), '
                         'or those plus the added box cases merged in place')
    a = ap.parse_args()
    if not O.build_reference(a.reference):
        raise SystemExit('cannot build oracle/_ref from ' + a.reference)
    make_admm_golden()
    make_dual_newton_golden()
    make_kkt_rows_golden()
    make_polish_golden()
    make_check_golden()
    if a.only == 'admm':
        return
    if a.only == 'open':
        update_open_cases()
        return
    records, vectors = [], {}
    for name, inst, opts, gen in cases():
        rec, x = run_case(name, inst, opts)
        rec['generator'] = gen
        rec['fstar'] = inst['fstar']
        records.append(rec)
        if len(x) <= 2000:
            vectors[name] = x
        print(name, rec['status'], rec['iterations'], rec['objective'], flush=True)
    explicit = [('v2_psd_300', v2_psd_case(), dict(tol=1e-7), False, 0.0),
                ('two_var', two_var_case(), dict(tol=1e-7), False, 0.0),
                ('two_var_maximize', {**two_var_case(), 'hval': -two_var_case()['hval'],
                                      'cost': -two_var_case()['cost']}, dict(tol=1e-7), True, 3.0)]
    for name, p, opts, mx, off in explicit:
        rec, x = run_case(name, p, opts, mx, off)
        rec['problem'] = {k: np.asarray(v).tolist() for k, v in p.items()}
        records.append(rec)
        vectors[name] = x
        print(name, rec['status'], rec['iterations'], rec['objective'], flush=True)
    # convexity verdicts of the reference (src/qp_admm.cpp:30-62)
    p = v2_psd_case()
    bad = p['hval'].copy(); bad[0] = -1.0
    convex = {'v2_psd_300': O.ref_check_convex(300, p['hrow'], p['hcol'], p['hval']),
              'v2_indefinite_300': O.ref_check_convex(300, p['hrow'], p['hcol'], bad)}
    # public QPLIB box instances (scalar results only)
    qplib = []
    data = Path(a.reference) / 'datasets' / 'qplib'
    for name in ('8792', '8991'):
        path = data / f'{name}.qplib'
        if not path.exists():
            continue
        q = O.ref_read_qplib(path)
        status, x, st = O.ref_solve_box(q['hrow'], q['hcol'], q['hval'], q['cost'], q['lower'], q['upper'], tol=1e-7,
                                        time_limit=600.0, threads=1, maximize=q['maximize'], offset=q['offset'])
        qplib.append({'name': name, 'sha256': hashlib.sha256(path.read_bytes()).hexdigest(), 'n': q['n'],
                      'hessian_entries': int(len(q['hrow'])), 'status': status, 'iterations': int(st['iterations']),
                      'objective': st['objective'], 'stationarity_residual': st['stationarity_residual']})
        print('qplib', name, status, st['iterations'], st['objective'], flush=True)
    meta = {'generated_by': 'tests/golden/make_golden.py', 'engine': 'reference solve_accelerated_box(cuda=false), 1 thread',
            'build': 'oracle/ref.mk (g++ -O3 -fopenmp -ffp-contract=off)'}
    (OUT / 'reference_cases.json').write_text(json.dumps({'meta': meta, 'cases': records, 'convex': convex,
                                                           'qplib': qplib}, indent=1) + '\n')
    np.savez_compressed(OUT / 'reference_x.npz', **vectors)


if __name__ == '__main__':
    main()
