"""QPLIB reader and the CLI drop-in (CPU parts; the solve itself is in the GPU test below)."""
import json
import math
import os
from pathlib import Path

import numpy as np
import pytest

import boxqp
from boxqp import cli
from boxqp.qplib import read_qplib, write_qplib
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
])
def test_reader_rejects_like_the_reference(text, msg):
    with pytest.raises(ValueError, match=msg):
        read_qplib(text)


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
