"""C-ABI library and host logic, without a GPU: symbols, generator, CSR builder, convexity gate,
validation and error behaviour of the reference-facing API."""
import re
from pathlib import Path

import numpy as np
import pytest

import boxqp
from boxqp import _native as N
from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    names = set()
    for h in (ROOT / 'include').glob('*.h'):
        text = re.sub(r'/\*.*?\*/', '', h.read_text(), flags=re.S)
        for m in re.finditer(r'\b(bqp_[a-z0-9_]+)\s*\(', text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = boxqp.lib()
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_the_header():
    assert set(header_functions()) <= set(N.PROTOTYPES)


def test_options_defaults_mirror_qpoptions():
    o = N.Options()
    boxqp.lib().bqp_options_default(o)
    # check_interval 0 and polish_switch 0 select the engine defaults (25 = the reference's cadence
    # for the FP64 engines)
    assert (o.tolerance, o.time_limit, o.iteration_limit, o.check_interval) == (1e-7, 30.0, 200000, 0)
    assert o.polish_switch == 0
    assert o.precision == 0 and o.diagonal_gate == -1


def test_planted_generator_is_deterministic_and_planted():
    a = boxqp.planted('graph10k', seed=11, n=4000)
    b = boxqp.planted('graph10k', seed=11, n=4000)
    c = boxqp.planted('graph10k', seed=12, n=4000)
    for k in ('rowptr', 'col', 'val', 'c', 'lower', 'upper', 'xstar', 'z'):
        assert np.array_equal(a[k], b[k]), k
    assert not np.array_equal(a['val'], c['val'])
    n, rp, col, val = a['n'], a['rowptr'], a['col'], a['val']
    # symmetric, sorted rows, diagonally dominant with positive diagonal
    rows = np.repeat(np.arange(n), np.diff(rp))
    dense_pairs = dict(zip(zip(rows.tolist(), col.tolist()), val.tolist()))
    for (i, j), v in list(dense_pairs.items())[:5000]:
        assert dense_pairs[(j, i)] == v
    for i in range(0, n, 97):
        seg = col[rp[i]:rp[i + 1]]
        assert np.all(np.diff(seg) > 0)
        d = val[rp[i]:rp[i + 1]][seg == i][0]
        off = np.abs(val[rp[i]:rp[i + 1]][seg != i]).sum()
        assert d >= off + 0.5 - 1e-12
    # planted KKT: Q x* + c = z, z >= 0.1 at lower, <= -0.1 at upper, 0 inside
    qx = np.zeros(n)
    np.add.at(qx, rows, val * a['xstar'][col])
    g = qx + a['c']
    assert np.allclose(g, a['z'], atol=1e-12)
    lo, up = a['xstar'] == a['lower'], a['xstar'] == a['upper']
    assert np.all(a['z'][lo] >= 0.1) and np.all(a['z'][up] <= -0.1) and np.all(a['z'][~(lo | up)] == 0)
    assert 0.25 < lo.mean() < 0.35 and 0.25 < up.mean() < 0.35


def test_presets_match_the_workload_shapes():
    s = boxqp.planted_spec('graph1m')
    assert (s.n, s.edges_per_vertex, s.lower, s.upper, s.frac_lower, s.frac_upper) == (1000000, 7, -1, 1, .25, .25)
    s = boxqp.planted_spec('grid')
    assert (s.grid_side, s.shift, s.bounds_mode, s.frac_lower) == (1024, 1e-3, 1, .2)
    sizes = [boxqp.planted_spec('batch', seed=3, index=i).n for i in range(400)]
    assert min(sizes) >= 64 and max(sizes) < 16384
    assert 1500 < np.mean(sizes) < 4500  # log-uniform [64, 16384] has mean ~2943
    epv = {boxqp.planted_spec('batch', seed=3, index=i).edges_per_vertex for i in range(200)}
    assert epv == {2, 3, 4, 5, 6}
    sizes = [boxqp.planted_spec('serve', seed=4, index=i).n for i in range(400)]
    assert min(sizes) >= 1000 and max(sizes) < 200000


def test_grid_family_structure():
    g = boxqp.planted('grid', seed=2, n=16 * 16)
    assert g['n'] == 256 and g['nnz'] == 5 * 256 - 4 * 16
    assert np.all(g['lower'] <= -0.5) and np.all(g['upper'] >= 0.5)
    d = g['val'][g['col'] == np.repeat(np.arange(256), np.diff(g['rowptr']))]
    assert np.allclose(d, 4.001)


@pytest.mark.parametrize('seed', range(4))
def test_csr_builder_matches_reference_assembly(seed):
    """bqp_csr_from_lower == mirroring + std::map merge (oracle restatement), incl. duplicates and zeros."""
    rng = np.random.default_rng(seed)
    n = 200
    k = 1500
    r = rng.integers(0, n, k)
    c = rng.integers(0, n, k)
    hr, hc = np.maximum(r, c), np.minimum(r, c)
    hv = rng.choice([-1.5, 0.0, 0.25, 1.0, 2.0], size=k)
    # an exact cancellation pair
    hr = np.append(hr, [5, 5]); hc = np.append(hc, [3, 3]); hv = np.append(hv, [1.25, -1.25])
    for sign in (1.0, -1.0):
        a = boxqp.csr_from_lower(n, hr, hc, hv, sign)
        b = O.build_csr(n, hr, hc, hv, sign)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_parallel_csr_builder_keeps_input_order_across_chunks():
    """Enough triplets for the multi-threaded path (several chunks, several row blocks): repeated
    entries of one row spread over all chunks must still be summed in input order."""
    rng = np.random.default_rng(7)
    n = 3000
    k = 900000
    r = rng.integers(0, n, k)
    c = rng.integers(0, n, k)
    hr, hc = np.maximum(r, c), np.minimum(r, c)
    hv = rng.standard_normal(k) * 10.0 ** rng.integers(-8, 8, k)  # sums whose value depends on order
    hv[rng.random(k) < 0.05] = 0.0
    a = boxqp.csr_from_lower(n, hr, hc, hv, 1.0)
    b = O.build_csr(n, hr, hc, hv, 1.0)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_gershgorin_matches_oracle():
    g = boxqp.planted('graph10k', seed=3, n=2000)
    assert boxqp.gershgorin(g['rowptr'], g['val']) == O.max_abs_row_sum(g['rowptr'], g['val'])


def test_convexity_gate_matches_reference(golden):
    d, _ = golden
    n = 300
    hr, hc, hv = [], [], []
    for j in range(n):
        hr.append(j); hc.append(j); hv.append(5.0 if j % 2 else 1.0)
        if j % 2:
            hr.append(j); hc.append(j - 1); hv.append(2.0)
    q = boxqp.QuadraticProblem(cost=-np.ones(n), lower=np.zeros(n), upper=np.full(n, 10.0), hessian_row=np.array(hr),
                               hessian_col=np.array(hc), hessian_val=np.array(hv))
    assert boxqp.check_convex_hessian(q) == bool(d['convex']['v2_psd_300'])
    q.hessian_val = q.hessian_val.copy()
    q.hessian_val[0] = -1.0
    assert boxqp.check_convex_hessian(q) == bool(d['convex']['v2_indefinite_300'])
    rng = np.random.default_rng(1)
    for trial in range(20):
        m = 30
        a = rng.standard_normal((m, m)) * (rng.random((m, m)) < 0.15)
        h = a @ a.T + (0.0 if trial % 2 else -0.3) * np.eye(m)
        rr, cc = np.tril_indices(m)
        keep = h[rr, cc] != 0
        prob = boxqp.QuadraticProblem(cost=np.zeros(m), lower=np.zeros(m), upper=np.ones(m), hessian_row=rr[keep],
                                      hessian_col=cc[keep], hessian_val=h[rr, cc][keep])
        assert int(boxqp.check_convex_hessian(prob)) == O.check_convex(m, rr[keep], cc[keep], h[rr, cc][keep])


def small_problem():
    return boxqp.QuadraticProblem(cost=np.array([-2.0, -4.0]), lower=np.array([-10.0, -10.0]),
                                  upper=np.array([10.0, 10.0]), hessian_row=np.array([0, 1]),
                                  hessian_col=np.array([0, 1]), hessian_val=np.array([2.0, 2.0]))


def test_reference_argument_errors_raise_value_error():
    """std::invalid_argument cases of src/accelerated_qp.cpp:14-17 and src/mps.cpp:47-60."""
    for bad in (dict(tolerance=0.0), dict(tolerance=float('nan')), dict(time_limit=-1.0), dict(threads=0)):
        with pytest.raises(ValueError):
            boxqp.solve_accelerated_box(small_problem(), boxqp.QpOptions(**bad))
    q = small_problem()
    q.rows = 1
    with pytest.raises(ValueError, match='box constraints only'):
        boxqp.solve_accelerated_box(q)
    q = small_problem()
    q.integer = np.array([True, False])
    with pytest.raises(ValueError, match='continuous'):
        boxqp.solve_accelerated_box(q)
    q = small_problem()
    q.cost = np.array([np.nan, 1.0])
    with pytest.raises(ValueError):
        boxqp.solve_accelerated_box(q)
    with pytest.raises(ValueError):
        boxqp.solve_accelerated_box(small_problem(), cuda=False)


def test_statuses_decided_before_the_device():
    q = small_problem()
    q.hessian_val = np.array([2.0, -2.0])
    assert boxqp.solve_accelerated_box(q).status == 'unsupported_curvature'
    q = small_problem()
    q.hessian_val = np.array([0.0, 0.0])
    with pytest.raises(ValueError, match='Zero-Hessian'):
        boxqp.solve_accelerated_box(q)
    q = small_problem()
    q.lower = np.array([1.0, -10.0])
    q.upper = np.array([0.0, 10.0])
    assert boxqp.solve_accelerated_box(q).status == 'infeasible_bounds'


def test_engine_reports_missing_device_without_a_gpu():
    import subprocess
    import sys
    code = ('import sys; sys.path[:0]=[{!r},{!r}]\n'
            'import boxqp\n'
            'h = boxqp.lib().bqp_create(0, 0)\n'
            'print("CTX", bool(h), boxqp.lib().bqp_last_error(None).decode())\n').format(
        str(ROOT), str(ROOT / 'hypergrey-sih-26_gb300'))
    out = subprocess.run([sys.executable, '-c', code], capture_output=True, text=True, timeout=120,
                         env={'CUDA_VISIBLE_DEVICES': '', 'PATH': '/usr/bin:/bin'})
    assert 'CTX False' in out.stdout and 'No CUDA device' in out.stdout


def test_splitmix64_reference_values():
    # splitmix64 from state 0: first outputs of the published generator
    out, state = boxqp.splitmix64(0)
    assert out == 0xE220A8397B1DCDAF
    out2, _ = boxqp.splitmix64(state)
    assert out2 == 0x6E789E6AA1B965F4


def test_level_a_plugin_links_into_the_reference():
    """The reference's own scale harness, linked with the GB300 plugin in place of its CUDA file
    and with the engine route, reaches the GB300 code: without a GPU both report the reference's
    message and exit code 2, and the engine route's cpu backend still runs the reference's own
    solver (its harness passes)."""
    import json
    import subprocess
    out_dir = O.build_level_a()
    if out_dir is None:
        pytest.skip('the reference sources are not staged on this host')
    env = {'CUDA_VISIBLE_DEVICES': '', 'PATH': '/usr/bin:/bin'}
    for name in ('solver_scale_gb300', 'solver_scale_gb300_engine'):
        out = subprocess.run([str(out_dir / name), '1000', 'cuda', '1', '30'], capture_output=True, text=True,
                             timeout=120, env=env)
        assert out.returncode == 2 and 'No CUDA device available' in out.stderr, (name, out.stderr)
    out = subprocess.run([str(out_dir / 'solver_scale_gb300_engine'), '1000', 'cpu', '1', '30'], capture_output=True,
                         text=True, timeout=120, env=env)
    assert out.returncode == 0 and json.loads(out.stdout)['passed'] is True


def test_csr_builder_from_several_threads_at_once():
    """Callers on several threads share the host worker pool (their tasks queue and the workers
    help each in turn); each gets exactly the single-caller result."""
    import threading
    rng = np.random.default_rng(11)
    n = 2500
    jobs = []
    for t in range(4):
        k = 400000 + 50000 * t
        r = rng.integers(0, n, k)
        c = rng.integers(0, n, k)
        jobs.append((np.maximum(r, c), np.minimum(r, c), rng.standard_normal(k)))
    expected = [boxqp.csr_from_lower(n, *j, 1.0) for j in jobs]
    results = [None] * len(jobs)

    def run(i):
        for _ in range(3):
            results[i] = boxqp.csr_from_lower(n, *jobs[i], 1.0)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(len(jobs))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for got, want in zip(results, expected):
        for x, y in zip(got, want):
            assert np.array_equal(x, y)


def test_gpu_entry_points_fail_loudly_without_a_gpu():
    """No CPU fallback: with no device visible, page-locking and the ADMM system report a CUDA
    error instead of running anything on the host."""
    import subprocess
    import sys
    code = ('import sys; sys.path[:0]=[{!r},{!r}]\n'
            'import numpy as np, boxqp\n'
            'from boxqp.admm import AdmmSystem\n'
            'a = np.zeros(1000)\n'
            'try:\n'
            '    with boxqp.pinned(a):\n'
            '        print("PINNED")\n'
            'except boxqp.EngineError as e:\n'
            '    print("PIN-ERROR", e)\n'
            'h = (np.array([0, 1], np.int32), np.array([0], np.int32), np.array([2.0]))\n'
            'try:\n'
            '    AdmmSystem(*h, np.array([0], np.int32), np.zeros(0, np.int32), np.zeros(0), 1)\n'
            '    print("ADMM-CREATED")\n'
            'except ValueError as e:\n'
            '    print("ADMM-ERROR", e)\n').format(str(ROOT), str(ROOT / 'hypergrey-sih-26_gb300'))
    out = subprocess.run([sys.executable, '-c', code], capture_output=True, text=True, timeout=120,
                         env={'CUDA_VISIBLE_DEVICES': '', 'PATH': '/usr/bin:/bin'})
    assert 'PIN-ERROR' in out.stdout and 'ADMM-ERROR' in out.stdout, out.stdout + out.stderr
