"""QPLIB reader and the CLI drop-in (CPU parts; the solve itself is in the GPU test below)."""
import json
import math
import os
from pathlib import Path

import numpy as np
import pytest

import boxqp
from boxqp import cli
from boxqp.qplib import read_qplib, read_qplib_rows, write_qplib
from oracle import oracle as O


def planted_problem(n=200, seed=5):
    inst = boxqp.planted('graph10k', seed=seed, n=n, lower_triplets=True)
    return inst, boxqp.problem_from_planted(inst)


def test_writer_reader_roundtrip(tmp_path):
    inst, q = planted_problem()
    q.offset = 2.5
    path = tmp_path / 'm.qplib'
    write_qplib(path, q)
    r, rows = read_qplib(path.read_text())
    assert rows == 0 and r.n == q.n and r.offset == 2.5
    assert np.array_equal(r.hessian_row, q.hessian_row) and np.array_equal(r.hessian_col, q.hessian_col)
    assert np.array_equal(r.hessian_val, q.hessian_val)
    assert np.array_equal(r.cost, q.cost) and np.array_equal(r.lower, q.lower) and np.array_equal(r.upper, q.upper)


@pytest.mark.parametrize('text,msg', [
    ('x QCB minimize 0\n', 'Empty'),
    ('x QIB minimize 2\n', 'unsupported_qplib_type'),
    ('x QCB upward 2\n', 'sense'),
    ('x QCB minimize 200000\n', 'oversized'),
    ('x QCB minimize 2 1 1 2 1.0\n', 'Hessian'),
    ('x QCB minimize 2 0 0 0 0', 'Truncated'),
    ('x QCB minimize 1 1 1 1 1e400\n', 'Hessian'),  # finite as a long double, infinite as a double
    ('x QCL minimize 1 1 0 0 0 0 1 1 1 1e400\n', 'matrix'),
])
def test_reader_rejects_like_the_reference(text, msg):
    with pytest.raises(ValueError, match=msg):
        read_qplib(text)


def constrained_qplib_text(seed=3, n=30, m=12):
    """A QCL model (linear rows) in QPLIB layout: lower-triangle Hessian, sparse cost, row entries
    listed in shuffled order, row bounds with the 1e20 infinity marker (one-sided and equality
    rows), variable bounds."""
    rng = np.random.default_rng(seed)
    lines = ['GEN', 'QCL', 'minimize', str(n), str(m)]
    h = [(j, j, 2.0 + rng.random()) for j in range(n)] + [(j + 1, j, -0.5 * rng.random()) for j in range(n - 1)]
    lines += [str(len(h))] + [f'{i + 1} {j + 1} {v:.17g}' for i, j, v in h]
    cost = rng.normal(size=n)
    lines += ['0', str(n)] + [f'{j + 1} {cost[j]:.17g}' for j in range(n)] + ['0.5']
    entries = [(i, j, rng.normal()) for i in range(m) for j in sorted(rng.choice(n, 3, replace=False))]
    entries = [entries[k] for k in rng.permutation(len(entries))]
    lines += [str(len(entries))] + [f'{i + 1} {j + 1} {v:.17g}' for i, j, v in entries]
    lines += ['1e20']
    lo = [-1e20 if i % 4 == 0 else -0.5 for i in range(m)]
    up = [1e20 if i % 4 == 1 else (-0.5 if i % 4 == 2 else 0.5) for i in range(m)]
    for vec in (lo, up):
        lines += ['0', str(m)] + [f'{i + 1} {v:.17g}' for i, v in enumerate(vec)]
    lines += ['-1', '0', '1', '0']  # variable bounds [-1, 1]
    lines += ['0', '0', '0', '0', '0', '0', '0', '0']  # start vectors, names
    return '\n'.join(lines) + '\n'


def test_reader_rows_match_the_reference_reader(tmp_path):
    """read_qplib_rows gives the reference reader's rows (row by row, each in file order), row
    bounds (the infinity marker mapped to infinity) and the same problem as read_qplib."""
    if not O.ref_available():
        pytest.skip('oracle/_ref not built on this host')
    path = tmp_path / 'c.qplib'
    path.write_text(constrained_qplib_text())
    ref = O.ref_read_qplib(path)
    q, rows = read_qplib_rows(path.read_text())
    q0, m = read_qplib(path.read_text())
    assert m == rows.m == ref['rows'] == 12 and q.n == q0.n == ref['n']
    for k in ('a_rowptr', 'a_col', 'a_val', 'row_lower', 'row_upper'):
        mine = {'a_rowptr': rows.rowptr, 'a_col': rows.col, 'a_val': rows.val, 'row_lower': rows.lower,
                'row_upper': rows.upper}[k]
        assert np.array_equal(mine, ref[k]), k
    assert np.isinf(rows.lower[0]) and np.isinf(rows.upper[1]) and rows.lower[2] == rows.upper[2] == -0.5
    for a, b in ((q.hessian_val, ref['hval']), (q.cost, ref['cost']), (q.lower, ref['lower']), (q.upper, ref['upper'])):
        assert np.array_equal(a, b)
    assert q.offset == ref['offset'] == 0.5
    _, none = read_qplib_rows('x QCB minimize 1 1 1 1 2.0 0 0 0 1e20 0 0 1 0 0 0 0 0 0 0\n')
    assert none.m == 0 and none.rowptr.tolist() == [0]


@pytest.mark.skipif(not os.environ.get('BOXQP_REFERENCE_DIR'), reason='set BOXQP_REFERENCE_DIR to the reference solver')
def test_reader_matches_reference_reader_on_qplib_box_instances():
    if not O.build_reference(os.environ['BOXQP_REFERENCE_DIR']):
        pytest.skip('oracle/_ref not built')
    data = Path(os.environ['BOXQP_REFERENCE_DIR']) / 'datasets' / 'qplib'
    for name in ('8792', '8991'):
        ref = O.ref_read_qplib(data / f'{name}.qplib')
        q, rows = read_qplib((data / f'{name}.qplib').read_text())
        assert rows == 0 and q.n == ref['n'] and q.maximize == ref['maximize'] and q.offset == ref['offset']
        for a, b in ((q.hessian_row, ref['hrow']), (q.hessian_col, ref['hcol'])):
            assert np.array_equal(a, b)
        for a, b in ((q.hessian_val, ref['hval']), (q.cost, ref['cost']), (q.lower, ref['lower']), (q.upper, ref['upper'])):
            assert np.allclose(a, b, rtol=1e-15, atol=0)


def test_cli_option_errors_exit_2(tmp_path, capsys):
    _, q = planted_problem(20)
    path = tmp_path / 'm.qplib'
    write_qplib(path, q)
    assert cli.main([str(path), '--backend', 'gpu']) == 2
    assert cli.main([str(path), '--threads', '0', '--backend', 'cuda']) == 2
    assert cli.main([str(path), '--backend', 'cuda', '--bogus']) == 2
    assert cli.main([str(path), '--backend', 'cpu']) == 2
    assert cli.main([str(tmp_path / 'missing.qplib'), '--backend', 'cuda']) == 2


@pytest.mark.gpu
def test_cli_json_record_matches_the_reference_fields(tmp_path, capsys, golden):
    d, _ = golden
    rec = next(c for c in d['cases'] if c['name'] == 'two_var')
    q = boxqp.QuadraticProblem(cost=np.array(rec['problem']['cost']), lower=np.array(rec['problem']['lower']),
                               upper=np.array(rec['problem']['upper']), hessian_row=np.array(rec['problem']['hrow']),
                               hessian_col=np.array(rec['problem']['hcol']), hessian_val=np.array(rec['problem']['hval']))
    path = tmp_path / 'two.qplib'
    write_qplib(path, q)
    assert cli.main([str(path), '--json', '--backend', 'cuda', '--precision', 'fp64_exact']) == 0
    out = json.loads(capsys.readouterr().out)
    for key in ('status', 'algorithm', 'threads', 'optimality_verified', 'iterations', 'total_seconds', 'rows', 'columns',
                'objective', 'primal_residual', 'stationarity_residual', 'complementarity_residual',
                'dual_bound_minimization_sense', 'relative_gap', 'primal', 'row_dual'):
        assert key in out
    assert out['status'] == 'optimal' and out['iterations'] == rec['iterations']
    assert math.isclose(out['objective'], rec['objective'], rel_tol=1e-12)
