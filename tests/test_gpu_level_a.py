"""The reference's own CLI and scale harness on the GB300 (needs a GPU).

oracle/ref.mk links the reference's unmodified solver objects and its src/main.cpp and
src/scale_benchmark.cpp two ways:
  * *_gb300: with SOVEREIGN_CUDA defined and the GB300 plugin (plugin/cuda_box_gb300.cpp) in
    place of src/cuda_box.cu: the reference's loop steps the device through make_cuda_box /
    BoxIteration, one fused FISTA kernel per iteration, and checks on the host every 25;
  * *_gb300_engine: the same objects linked with -Wl,--wrap for solve_accelerated_box, which
    sends cuda = true to the device-resident engine (plugin/engine_route.cpp, bqp_solve_sync).
Each binary runs as the reference's users run it, and its own JSON output is checked:
  * plugin: the cuda backend gives the cpu backend's status, iteration count and objective bit
    for bit (the plugin's step reproduces the CPU loop's arithmetic);
  * engine route: the harness's own pass criteria at its published size (n = 1,000,000: status
    optimal and verified, relative objective error <= 1e-8, max error < 1e-4), and on the QPLIB
    box instances the published objectives to 1e-7 relative, verified at the CLI's tolerance.
"""
import json
import subprocess

import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

REF = O.HERE / '_ref'


def binary(name):
    path = REF / name
    if not path.exists():
        pytest.skip(f'{name} is not built (needs the staged reference sources: make -f oracle/ref.mk stage)')
    return path


def run_json(cmd, timeout=600):
    proc = subprocess.run([str(c) for c in cmd], capture_output=True, text=True, timeout=timeout)
    lines = [ln for ln in proc.stdout.splitlines() if ln.startswith('{')]
    assert lines, f'no JSON from {cmd}: rc {proc.returncode}\n{proc.stdout[-2000:]}\n{proc.stderr[-2000:]}'
    return proc.returncode, json.loads(lines[-1])


def test_scale_harness_plugin_backend_equals_cpu_backend():
    exe = binary('solver_scale_gb300')
    rc_cpu, cpu = run_json([exe, 10000, 'cpu', 1, 60])
    rc_gpu, gpu = run_json([exe, 10000, 'cuda', 1, 60])
    assert rc_cpu == 0 and cpu['passed'] is True
    assert rc_gpu == 0 and gpu['passed'] is True, gpu
    assert gpu['status'] == cpu['status'] == 'optimal'
    assert gpu['iterations'] == cpu['iterations']
    assert gpu['objective'] == cpu['objective']


def test_scale_harness_on_engine_route_at_published_size():
    """The reference's published family at n = 1,000,000 (known objective -94123.887220104109)."""
    exe = binary('solver_scale_gb300_engine')
    rc, out = run_json([exe, 1000000, 'cuda', 1, 120])
    assert rc == 0 and out['passed'] is True, out
    assert out['status'] == 'optimal' and out['columns'] == 1000000
    assert out['relative_objective_error'] <= 1e-8 and out['max_solution_error'] < 1e-4
    assert out['objective'] == pytest.approx(-94123.887220104109, rel=1e-8)


@pytest.mark.parametrize('name', ['8792', '8991'])
def test_cli_plugin_backend_equals_cpu_backend_on_qplib(name):
    exe = binary('solver_cli_gb300')
    model = O.REF_QPLIB / f'{name}.qplib'
    if not model.exists():
        pytest.skip('QPLIB files not staged')
    rc_cpu, cpu = run_json([exe, model, '--json', '--backend', 'cpu'])
    rc_gpu, gpu = run_json([exe, model, '--json', '--backend', 'cuda'])
    assert rc_cpu == 0 and rc_gpu == 0
    assert gpu['status'] == cpu['status'] == 'optimal' and gpu['optimality_verified']
    assert gpu['iterations'] == cpu['iterations']
    assert gpu['objective'] == cpu['objective']
    assert gpu['primal'] == cpu['primal']


@pytest.mark.parametrize('name,objective', [('8792', 3593.5162939294105), ('8991', -0.0016678673619609664)])
def test_cli_engine_route_on_qplib(name, objective):
    exe = binary('solver_cli_gb300_engine')
    model = O.REF_QPLIB / f'{name}.qplib'
    if not model.exists():
        pytest.skip('QPLIB files not staged')
    rc, out = run_json([exe, model, '--json', '--backend', 'cuda'])
    assert rc == 0 and out['status'] == 'optimal' and out['optimality_verified'] is True, out
    assert out['algorithm'] == 'cuda_fista_box'
    assert abs(out['objective'] - objective) <= 1e-7 * (1 + abs(objective))
    assert out['stationarity_residual'] <= 1e-7
