#!/usr/bin/env python
"""Benchmark of the GB300 box-QP engine; prints ONE JSON line (rank 0).

Default workload: the planted random-graph box QP with n = 1,000,000 variables, 7 edges per
vertex (~15M nonzeros), bounds [-1, 1], solved in mixed precision to KKT <= 1e-6 and verified
in FP64.  A step is one complete solve of that instance.

  value   solves/s with the problem resident in HBM: K re-solves (x0 = clip(0), no upload),
          timed with CUDA events on the engine stream (graph launches + re-arm kernels)
  e2e     solves/s through the public C-ABI call bqp_solve_sync with host buffers: upload of
          the CSR and vectors, admission, solve and the copy of x back, timed per call
  roofline  the FISTA step kernel (dominant kernel) timed alone with CUDA events on the same
          instance; algorithmic bytes per launch nnz*(4+4) + 4(n+1) + 7*4n
  cpu_baseline  the FP64 reference FISTA (CPU oracle port, all host cores) on one full solve

--impl reference times the reference algorithm's CPU implementation (the oracle port of
src/accelerated_qp.cpp, OpenMP on all host cores) on the same workload and metric.
Multi-GPU (--gpus N under torchrun): independent replicas, one per GPU (no data exchange).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path[:0] = [str(ROOT), str(ROOT / 'hypergrey-sih-26_gb300')]

METRIC = 'box-QP solves/s & HBM GB/s at KKT≤1e-6, mixed vs FP64; serve p50/p99 ms'
L2_BYTES = 129e6


def load_peaks():
    p = ROOT / 'MEASURED_PEAKS.json'
    if p.exists():
        d = json.loads(p.read_text())
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.device), f'--query-gpu={self.FIELDS}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in self.lines:
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith('active'):
                    reasons.add(name)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': mx or None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def make_workload(name, rank):
    import boxqp
    if name == 'graph1m':
        inst = boxqp.planted('graph1m', seed=1 + rank, lower_triplets=True)
        desc = ('planted random-graph Laplacian box QP, n=1,000,000, 7 edges/vertex, bounds [-1,1], '
                '25/25/50 planted pattern')
    elif name == 'grid':
        inst = boxqp.planted('grid', seed=2 + rank, lower_triplets=True)
        desc = '1024x1024 5-point grid Laplacian + 1e-3 I, random bounds, 20/20/60 planted pattern'
    elif name == 'graph10k':
        inst = boxqp.planted('graph10k', seed=rank, lower_triplets=True)
        desc = 'planted random-graph Laplacian box QP, n=10,000, 5 edges/vertex, bounds [0,1]'
    else:
        raise SystemExit(f'unknown workload {name}')
    return inst, desc


def oracle_args(inst):
    return inst['hrow'], inst['hcol'], inst['hval'], inst['c'], inst['lower'], inst['upper']


def cpu_reference_solve(inst, tol, time_limit=60.0):
    """One FP64 reference-FISTA solve on all host cores (oracle port); returns (seconds, info)."""
    from oracle import oracle as O
    threads = O.max_threads()
    t0 = time.perf_counter()
    status, x, st = O.solve_box(*oracle_args(inst), tol=tol, threads=threads, time_limit=time_limit)
    dt = time.perf_counter() - t0
    return dt, {'status': status, 'iterations': int(st['iterations']), 'threads': threads}


def dist_setup(args):
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault('MASTER_ADDR', '127.0.0.1')
        dist.init_process_group('gloo', rank=rank, world_size=world)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg:
        pg.barrier()


def allreduce_max(pg, value):
    if not pg:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(pg, value):
    if not pg:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def run_reference(args, world, rank, pg):
    """The reference arm: the reference algorithm on the host cores (rank 0 only)."""
    if rank != 0:
        return
    inst, desc = make_workload(args.workload, 0)
    for _ in range(args.warmup):
        cpu_reference_solve(inst, args.tol)
    times, info = [], {}
    for _ in range(args.steps):
        dt, info = cpu_reference_solve(inst, args.tol)
        times.append(dt)
    total = sum(times)
    value = args.steps / total
    line = {'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': 'solves/s', 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * total / args.steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': desc, 'n': inst['n'], 'nnz': inst['nnz'], 'tolerance': args.tol,
                       'engine': 'reference FISTA (src/accelerated_qp.cpp), CPU oracle port, OpenMP'},
            'cpu_baseline': {'value': value, 'unit': 'solves/s', 'cores': info.get('threads'), 'kind': 'port',
                             'sample': f'{args.steps} full FP64 solves of the workload at KKT<={args.tol:g} '
                                       f'({info.get("iterations")} iterations each)'},
            'e2e': {'value': value, 'unit': 'solves/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local, pg):
    import numpy as np
    import boxqp
    from boxqp import options_struct

    peak, peak_kind = load_peaks()
    inst, desc = make_workload(args.workload, rank)
    n, nnz = inst['n'], inst['nnz']
    eng = boxqp.Engine(local)
    opts = options_struct(args.tol, 60.0, 200000, args.precision)
    ident = eng.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], opts)
    eng.wait(ident)
    x, st = eng.fetch(ident, n)
    # warm-up re-solves
    for _ in range(max(args.warmup - 1, 0)):
        eng.resolve([ident])
        eng.wait(ident)
    # ---- timed region: K resident re-solves ---------------------------------------------------
    barrier(pg)
    eng.timer(reset=True)
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        iters, bytes_total = [], 0.0
        for _ in range(args.steps):
            eng.resolve([ident])
            eng.wait(ident)
            x, st = eng.fetch(ident, n)
            iters.append(int(st.iterations))
            bytes_total += st.bytes
        wall = time.perf_counter() - t0
    dev_ms, kernels, launches = eng.timer()
    barrier(pg)
    dev_s = allreduce_max(pg, dev_ms / 1e3)
    total_solves = allreduce_sum(pg, args.steps)
    value = total_solves / dev_s
    status = boxqp.STATUS_NAMES[st.status]
    result = {'status': status, 'iterations': iters[-1], 'polish_iterations': int(st.polish_iterations),
              'checks': int(st.checks), 'kkt_stationarity': st.stationarity_residual,
              'primal_residual': st.primal_residual,
              'objective_rel_err': abs(st.objective - inst['fstar']) / (1 + abs(inst['fstar']))}
    # ---- roofline of the dominant kernel (step kernel alone, CUDA events) ----------------------
    step_ms, step_bytes = eng.profile_step(ident, 100)
    achieved = step_bytes / (step_ms * 1e-3) / 1e9
    traffic = None
    tp = ROOT / 'profiles' / 'roofline_traffic.json'
    if tp.exists():
        traffic = json.loads(tp.read_text()).get(f'{args.workload}_{args.precision}')
    roofline = {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
                'traffic': traffic, 'peak_kind': peak_kind, 'kernel': f'step_kernel<{args.precision}>',
                'ms_per_launch': step_ms, 'algorithmic_bytes_per_launch': step_bytes}
    eng.resolve([ident])  # restore a valid iterate
    eng.wait(ident)
    x, st = eng.fetch(ident, n)
    # ---- FP64 plain engine on the same instance (the mixed-vs-FP64 half of the metric) --------
    fp64 = None
    if args.precision == 'mixed' and not args.quick:
        o64 = options_struct(args.tol, 60.0, 200000, 'fp64')
        id64 = eng.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o64)
        eng.wait(id64)
        eng.resolve([id64])
        eng.wait(id64)
        eng.timer(reset=True)
        reps = max(1, min(3, args.steps))
        for _ in range(reps):
            eng.resolve([id64])
            eng.wait(id64)
        ms64, _, _ = eng.timer()
        x64, s64 = eng.fetch(id64, n)
        ms64_step, b64 = eng.profile_step(id64, 50)
        eng.release(id64)
        fp64 = {'solves_per_s': reps / (ms64 / 1e3), 'hbm_gbs': s64.bytes / (ms64 / 1e3 / reps) / 1e9,
                'iterations': int(s64.iterations), 'status': boxqp.STATUS_NAMES[s64.status],
                'step_kernel_gbs': b64 / (ms64_step * 1e-3) / 1e9}
    # ---- e2e through the public C-ABI with host buffers -----------------------------------------
    e2e = None
    if not args.quick:
        h2d = (inst['rowptr'].nbytes + inst['col'].nbytes + inst['val'].nbytes + inst['c'].nbytes +
               inst['lower'].nbytes + inst['upper'].nbytes)
        d2h = n * 8
        e2e_steps = max(1, min(args.steps, 5))
        eng.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], opts)
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            xe, se = eng.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'],
                               opts)
        e2e_s = allreduce_max(pg, time.perf_counter() - t0)
        e2e = {'value': allreduce_sum(pg, e2e_steps) / e2e_s, 'unit': 'solves/s', 'h2d_bytes_per_step': int(h2d),
               'd2h_bytes_per_step': int(d2h), 'api': 'bqp_solve_sync (pageable host buffers)',
               'status': boxqp.STATUS_NAMES[se.status]}
    # ---- CPU baseline (rank 0, N = 1) -----------------------------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.quick:
        dt, info = cpu_reference_solve(inst, args.tol)
        cpu = {'value': 1.0 / dt, 'unit': 'solves/s', 'cores': info['threads'], 'kind': 'port',
               'sample': f'one full FP64 reference-FISTA solve of the workload at KKT<={args.tol:g} '
                         f'({info["iterations"]} iterations, status {info["status"]})'}
    eng.release(ident)
    eng.close()
    if rank != 0:
        return
    line = {'metric': METRIC, 'value': value, 'unit': 'solves/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': 1e3 * dev_s / args.steps, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32+f64' if args.precision == 'mixed' else 'f64',
            'data': 'synthetic',
            'config': {'workload': desc, 'n': n, 'nnz': nnz, 'precision': args.precision, 'tolerance': args.tol,
                       'l2': f'inputs larger than L2: one iteration streams '
                             f'{step_bytes / 1e6:.0f} MB > {L2_BYTES / 1e6:.0f} MB L2',
                       'parallelism': f'replicas x{world}'},
            'hbm_gbs': bytes_total / args.steps / (dev_s / args.steps) / 1e9,
            'wall_ms_per_step': 1e3 * wall / args.steps,
            'solve': result, 'fp64_engine': fp64, 'roofline': roofline, 'cpu_baseline': cpu, 'e2e': e2e,
            'gpu_launches': int(kernels), 'graph_launches': int(launches),
            'clocks': clocks.summary()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', choices=['ours', 'reference'], default='ours')
    ap.add_argument('--workload', default='graph1m', choices=['graph1m', 'grid', 'graph10k'])
    ap.add_argument('--precision', default='mixed', choices=['mixed', 'fp64'])
    ap.add_argument('--tol', type=float, default=1e-6)
    ap.add_argument('--quick', action='store_true', help='skip e2e, FP64 and CPU legs')
    args = ap.parse_args()
    world, rank, local, pg = dist_setup(args)
    if args.impl == 'reference':
        run_reference(args, world, rank, pg)
    else:
        run_ours(args, world, rank, local, pg)
    if pg:
        pg.destroy_process_group()


if __name__ == '__main__':
    main()
