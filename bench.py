#!/usr/bin/env python
"""Benchmark of the GB300 box-QP engine; prints ONE JSON line (rank 0).

Default workload: the planted random-graph box QP with n = 1,000,000 variables, 7 edges per
vertex (~15M nonzeros), bounds [-1, 1], solved in mixed precision to KKT <= 1e-6 and verified
in FP64.  A step is one complete solve of that instance.

  value   solves/s with the problem resident in HBM: K re-solves (x0 = clip(0), no upload),
          timed with CUDA events on the engine stream (graph launches + re-arm kernels)
  e2e     solves/s through the public C-ABI with host buffers: every solve submits its CSR and
          vectors (scan, upload, admission), solves, and copies x back; asynchronous submissions
          with three in flight through bqp_submit_borrowed (e2e.copy: bqp_submit, which copies
          the inputs at submission; e2e.sync: bqp_solve_sync one call at a time)
  roofline  the FISTA step kernel (dominant kernel) timed alone with CUDA events on the same
          instance; algorithmic bytes per launch nnz*(4+4) + 4(n+1) + 7*4n
  roofline_cg  the polish CG product kernel of the same solve (bqp_profile_cg), bytes per launch
          12 nnz_FF + 48 n_F on the packed free-free block
  solve.oracle_check  the timed solve's primal checked on the host by the oracle
          (check_qp_solution restated) and against the planted active set
  cpu_baseline  one full FP64 solve by the reference's own solve_accelerated_box, built from its
          sources on this host (all cores; the oracle port where no staged copy exists)

Other workloads (--workload): grid, graph10k, tridiagonal (the reference's published family),
batch (4,096 uneven instances in one launch), serve (Poisson arrivals into the continuous-batching
request loop) and admm (the constrained-QP ADMM inner solve, CG iterations/s).

--impl reference times the reference's own CPU solve_accelerated_box (src/accelerated_qp.cpp,
OpenMP on all host cores) on the same workload and metric, on an instance made by the oracle
library's copy of the generator, so that process never loads the engine library.
--case solve|step: small runs for kernel profilers (one solve; the step kernel alone).
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
                                          '--format=csv,noheader,nounits', '-lms', '100'],
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


WORKLOADS = {
    'graph1m': dict(preset='graph1m', seed=1, n=0,
                    desc='planted random-graph Laplacian box QP, n=1,000,000, 7 edges/vertex, bounds [-1,1], '
                         '25/25/50 planted pattern'),
    'grid': dict(preset='grid', seed=2, n=0,
                 desc='1024x1024 5-point grid Laplacian + 1e-3 I, random bounds, 20/20/60 planted pattern'),
    'graph10k': dict(preset='graph10k', seed=0, n=0,
                     desc='planted random-graph Laplacian box QP, n=10,000, 5 edges/vertex, bounds [0,1]'),
    'tridiagonal': dict(preset='tridiagonal', seed=1, n=1000000,
                        desc="the reference's published scale family (src/scale_benchmark.cpp:13-19): tridiagonal "
                             '2.02/-1, n=1,000,000, bounds [0,3], tolerance 1e-7, iteration limit 20000'),
}


def make_workload(name, rank, oracle_side=False):
    """The workload's planted instance (seed shifted by the rank).  oracle_side: generated by the
    generator linked into the oracle library, so the reference arm never loads the engine library
    (the arrays are the same bits)."""
    if name not in WORKLOADS:
        raise SystemExit(f'unknown workload {name}')
    w = WORKLOADS[name]
    seed = w['seed'] + (rank if name != 'tridiagonal' else 0)
    if oracle_side:
        from oracle import oracle as O
        inst = O.planted(w['preset'], seed=seed, n=w['n'], lower_triplets=True)
    else:
        import boxqp
        inst = boxqp.planted(w['preset'], seed=seed, n=w['n'], lower_triplets=True)
    return inst, w['desc']


def oracle_args(inst):
    return inst['hrow'], inst['hcol'], inst['hval'], inst['c'], inst['lower'], inst['upper']


def cpu_reference_solve(inst, tol, time_limit=600.0, prefer_reference=True, threads=0):
    """One FP64 CPU solve on `threads` host cores (0: all of them, QpOptions::threads): the
    reference's own solve_accelerated_box(q, opt, false) (oracle/_ref, built from its sources on
    this host) when available, else the oracle port of it.  Returns (seconds of the solve call,
    info)."""
    from oracle import oracle as O
    threads = threads or O.max_threads()
    if prefer_reference and O.ref_available():
        status, x, st = O.ref_solve_box(*oracle_args(inst), tol=tol, threads=threads, time_limit=time_limit)
        return st['seconds'], {'status': status, 'iterations': int(st['iterations']), 'threads': threads,
                               'kind': 'reference',
                               'engine': 'the reference build (oracle/_ref: src/accelerated_qp.cpp and its library, '
                                         'compiled from the reference sources on this host, -O3 -fopenmp)'}
    t0 = time.perf_counter()
    status, x, st = O.solve_box(*oracle_args(inst), tol=tol, threads=threads, time_limit=time_limit)
    dt = time.perf_counter() - t0
    return dt, {'status': status, 'iterations': int(st['iterations']), 'threads': threads, 'kind': 'port',
                'engine': 'the CPU oracle port of src/accelerated_qp.cpp (oracle/boxqp_oracle.c, OpenMP)'}


def oracle_check(inst, x, tol):
    """The oracle's check_qp_solution (restated, pinned to the reference) of a primal on the host,
    plus the active-set comparison with the planted optimum."""
    from oracle import oracle as O
    chk = O.check(*oracle_args(inst), x, tol=tol)
    fstar = inst['fstar']
    return {'verified': bool(chk['verified']), 'stationarity': chk['stationarity_residual'],
            'primal_residual': chk['primal_residual'],
            'objective_rel_err': abs(chk['objective'] - fstar) / (1 + abs(fstar)),
            'active_set_mismatches': O.active_set_mismatches(x, inst)}


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
    """The reference arm: the reference's own CPU solve_accelerated_box on the host cores (rank 0
    only), on the same instance, tolerance and metric.  The instance comes from the oracle
    library's copy of the generator: nothing of the engine is loaded in this process.  Each step
    is one full solve; the run is bounded to about a minute of solves (at least one), and `steps`
    reports how many were timed."""
    if rank != 0:
        return
    inst, desc = make_workload(args.workload, 0, oracle_side=True)
    for _ in range(min(args.warmup, 1)):
        cpu_reference_solve(inst, args.tol, threads=args.cpu_threads)
    times, info = [], {}
    budget = 60.0
    while len(times) < args.steps and (not times or sum(times) < budget):
        dt, info = cpu_reference_solve(inst, args.tol, threads=args.cpu_threads)
        times.append(dt)
    total = sum(times)
    value = len(times) / total
    line = {'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': 'solves/s', 'n_gpus': args.gpus,
            'steps': len(times), 'warmup': min(args.warmup, 1), 'ms_per_step': 1e3 * total / len(times),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': desc, 'n': inst['n'], 'nnz': inst['nnz'], 'tolerance': args.tol,
                       'engine': info.get('engine')},
            'cpu_baseline': {'value': value, 'unit': 'solves/s', 'cores': info.get('threads'), 'kind': info.get('kind'),
                             'sample': f'{len(times)} full FP64 solves of the workload at KKT<={args.tol:g} '
                                       f'({info.get("iterations")} iterations each, status {info.get("status")}), '
                                       f'timed around the solve_accelerated_box call; at most {args.steps} solves '
                                       f'or about {budget:g} s'},
            'e2e': {'value': value, 'unit': 'solves/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    gpu = reference_gpu_row(inst, args.tol)
    if gpu:
        line['reference_gpu'] = gpu
    print(json.dumps(line), flush=True)


def reference_gpu_row(inst, tol):
    """The reference's own CUDA plugin on this GPU: its kernels (src/cuda_box.cu, compiled unmodified
    for sm_103a into oracle/_ref) under its host loop with the host check every 25 iterations.
    Reported beside the reference arm's CPU value (which stays the arm's `value`); one solve."""
    from oracle import oracle as O
    if not O.REF_CUBIN.exists():
        return {'unavailable': 'the reference CUDA module was not built (no reference checkout where build() ran)'}
    if not O.build_ref_cuda():
        return {'unavailable': 'the driver-API harness did not compile'}
    try:
        status, st, x, (solve_s, loop_s) = O.ref_cuda_solve(
            inst['rowptr'], inst['col'], inst['val'], *oracle_args(inst), tol=tol, time_limit=120.0)
    except Exception as exc:
        return {'unavailable': str(exc)[:200]}
    return {'value': 1.0 / solve_s, 'unit': 'solves/s', 'status': status, 'iterations': int(st['iterations']),
            'seconds_per_solve': solve_s, 'loop_seconds': loop_s,
            'kind': 'reference CUDA plugin kernels (src/cuda_box.cu, unmodified, sm_103a) under the reference host '
                    'loop (src/accelerated_qp.cpp:36-57): 2 launches per iteration, host check every 25'}


def run_ours(args, world, rank, local, pg):
    import numpy as np
    import boxqp
    from boxqp import options_struct

    peak, peak_kind = load_peaks()
    inst, desc = make_workload(args.workload, rank)
    n, nnz = inst['n'], inst['nnz']
    eng = boxqp.Engine(local)
    iteration_limit = 20000 if args.workload == 'tridiagonal' else 200000
    opts = options_struct(args.tol, 60.0, iteration_limit, args.precision)
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
    # the last timed solve's primal checked on the host by the oracle (check_qp_solution restated
    # and pinned to the reference) and against the planted active set
    result['oracle_check'] = oracle_check(inst, x, args.tol)
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
    # second roofline entry: the polish CG of this solve (mixed precision), its product kernel
    # (the one that dominates the polish) and its vector kernel, on the packed Q_FF
    roofline_cg = None
    if args.precision == 'mixed':
        eng.resolve([ident])
        eng.wait(ident)
        try:
            ms_mv, ms_vec, b_mv, b_vec = eng.profile_cg(ident, 10)
            roofline_cg = {'bound': 'hbm', 'kernel': 'cg_matvec_kernel', 'achieved': b_mv / (ms_mv * 1e-3) / 1e9,
                           'peak': peak, 'unit': 'GB/s', 'frac': b_mv / (ms_mv * 1e-3) / 1e9 / peak,
                           'peak_kind': peak_kind, 'ms_per_launch': ms_mv, 'algorithmic_bytes_per_launch': b_mv,
                           'vector_kernel': {'kernel': 'cg_vector_kernel', 'ms_per_launch': ms_vec,
                                             'algorithmic_bytes_per_launch': b_vec,
                                             'achieved': b_vec / (ms_vec * 1e-3) / 1e9}}
        except Exception as exc:  # the solve ended without a polish: no CG to time
            roofline_cg = {'unavailable': str(exc)[:200]}
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
                'step_kernel_gbs': b64 / (ms64_step * 1e-3) / 1e9, 'oracle_check': oracle_check(inst, x64, args.tol)}
    # ---- e2e through the public C-ABI with host buffers -----------------------------------------
    e2e = None
    if not args.quick:
        h2d = (inst['rowptr'].nbytes + inst['col'].nbytes + inst['val'].nbytes + inst['c'].nbytes +
               inst['lower'].nbytes + inst['upper'].nbytes)
        d2h = n * 8
        args_host = (inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'])
        e2e_steps = max(1, min(args.steps, 5))
        eng.solve(*args_host, opts)
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            xe, se = eng.solve(*args_host, opts)
        sync_s = allreduce_max(pg, time.perf_counter() - t0)
        # the asynchronous API with three solves in flight: the host work of one submission (input
        # scan) overlaps the device work of the previous ones; every solve still uploads its inputs
        # from host memory and copies its primal back.  Headline: bqp_submit_borrowed (no host
        # copy of the inputs, the caller keeps them unchanged until the solve finishes); also
        # timed: bqp_submit, which copies the inputs first.
        def pipelined(copy, depth=3):
            steps = max(6, min(args.steps, 20))
            inflight, statuses = [], set()
            out = [np.empty(n, dtype=np.float64) for _ in range(depth)]

            def finish(k):
                i = inflight.pop(0)
                eng.wait(i)
                _, st = eng.fetch(i, n, out=out[k % depth])
                eng.release(i)
                statuses.add(boxqp.STATUS_NAMES[st.status])

            barrier(pg)
            t0 = time.perf_counter()
            for k in range(steps):
                inflight.append(eng.submit(*args_host, opts, copy=copy))
                if len(inflight) >= depth:
                    finish(k)
            while inflight:
                finish(0)
            return allreduce_sum(pg, steps) / allreduce_max(pg, time.perf_counter() - t0), statuses

        pipelined(False)  # host buffers, pool threads warm
        borrowed, st_b = pipelined(False)
        copied, st_c = pipelined(True)
        # the same with the caller's arrays page-locked once (bqp_host_register): the uploads
        # become DMA from the arrays themselves, with no staging copy on the host
        with boxqp.pinned(*args_host):
            pipelined(False)
            pinned_rate, st_p = pipelined(False)
        e2e = {'value': borrowed, 'unit': 'solves/s', 'h2d_bytes_per_step': int(h2d),
               'd2h_bytes_per_step': int(d2h),
               'api': 'bqp_submit_borrowed (3 in flight) + bqp_wait + bqp_fetch + bqp_release, pageable host buffers',
               'status': ','.join(sorted(st_b)),
               'copy': {'value': copied, 'api': 'bqp_submit (3 in flight, inputs copied at submission)',
                        'status': ','.join(sorted(st_c))},
               'pinned': {'value': pinned_rate, 'api': 'bqp_submit_borrowed (3 in flight) from page-locked host '
                          'arrays (bqp_host_register once)', 'status': ','.join(sorted(st_p))},
               'sync': {'value': allreduce_sum(pg, e2e_steps) / sync_s, 'api': 'bqp_solve_sync, one at a time',
                        'status': boxqp.STATUS_NAMES[se.status]}}
    # ---- CPU baseline (rank 0, N = 1) -----------------------------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.quick:
        dt, info = cpu_reference_solve(inst, args.tol, threads=args.cpu_threads)
        cpu = {'value': 1.0 / dt, 'unit': 'solves/s', 'cores': info['threads'], 'kind': info['kind'],
               'sample': f'one full FP64 solve of the workload at KKT<={args.tol:g} by {info["engine"]} '
                         f'({info["iterations"]} iterations, status {info["status"]})'}
    eng.release(ident)
    eng.close()
    if rank != 0:
        return
    # the reference publishes solve seconds only for its tridiagonal family: n = 1M on a Tesla T4,
    # median of 3, 3.501 s (README.md:94-101; reports/kaggle-gpu-03/REPORT.md:17-23)
    vs = value / (1.0 / 3.501) if args.workload == 'tridiagonal' else None
    line = {'metric': METRIC, 'value': value, 'unit': 'solves/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': 1e3 * dev_s / args.steps, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': vs, 'dtype': 'f32+f64' if args.precision == 'mixed' else 'f64',
            'data': 'synthetic',
            'config': {'workload': desc, 'n': n, 'nnz': nnz, 'precision': args.precision, 'tolerance': args.tol,
                       'l2': (f'inputs larger than L2: one iteration streams {step_bytes / 1e6:.0f} MB > '
                              f'{L2_BYTES / 1e6:.0f} MB L2') if step_bytes > L2_BYTES else
                             (f'one iteration streams {step_bytes / 1e6:.0f} MB, which fits the {L2_BYTES / 1e6:.0f} MB '
                              'L2: iterations after the first read mostly from L2, so the HBM roofline fraction '
                              'of the step kernel overstates HBM use for this workload'),
                       'parallelism': f'replicas x{world}'},
            'hbm_gbs': bytes_total / args.steps / (dev_s / args.steps) / 1e9,
            'wall_ms_per_step': 1e3 * wall / args.steps,
            'solve': result, 'fp64_engine': fp64, 'roofline': roofline, 'roofline_cg': roofline_cg,
            'cpu_baseline': cpu, 'e2e': e2e,
            'gpu_launches': int(kernels), 'graph_launches': int(launches),
            'clocks': clocks.summary()}
    print(json.dumps(line), flush=True)


def run_batch(args, world, rank, local, pg):
    """4,096 planted box QPs of uneven size (n log-uniform [64, 16384], 2..6 edges/vertex) solved in
    one running batch (mixed precision, each to its own KKT <= 1e-6), against a loop of single-instance
    solves of the plain FP64 engine and against the CPU reference algorithm."""
    import numpy as np
    import boxqp
    from boxqp import options_struct
    count = args.instances
    t0 = time.perf_counter()
    insts = [boxqp.planted('batch', seed=3 + 1000 * rank, index=i) for i in range(count)]
    gen_s = time.perf_counter() - t0
    n_tot = sum(p['n'] for p in insts)
    nnz_tot = sum(p['nnz'] for p in insts)
    eng = boxqp.Engine(local)
    opts = options_struct(args.tol, 60.0, 200000, 'mixed')
    ids = [eng.submit(p['rowptr'], p['col'], p['val'], p['c'], p['lower'], p['upper'], opts) for p in insts]
    for i in ids:
        eng.wait(i)
    for _ in range(args.warmup):
        eng.resolve(ids)
        for i in ids:
            eng.wait(i)
    barrier(pg)
    eng.timer(reset=True)
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            eng.resolve(ids)
            for i in ids:
                eng.wait(i)
        wall = time.perf_counter() - t0
    dev_ms, kernels, launches = eng.timer()
    dev_s = allreduce_max(pg, dev_ms / 1e3)
    solves = allreduce_sum(pg, args.steps * count)
    value = solves / dev_s
    statuses, iters, bytes_total, worst_kkt, worst_obj = {}, [], 0.0, 0.0, 0.0
    for p, i in zip(insts, ids):
        x, st = eng.fetch(i, p['n'])
        name = boxqp.STATUS_NAMES[st.status]
        statuses[name] = statuses.get(name, 0) + 1
        iters.append(int(st.iterations))
        bytes_total += st.bytes
        worst_kkt = max(worst_kkt, st.stationarity_residual)
        worst_obj = max(worst_obj, abs(st.objective - p['fstar']) / (1 + abs(p['fstar'])))
    # plain FP64 engine, one instance at a time
    o64 = options_struct(args.tol, 60.0, 200000, 'fp64')
    sample = list(range(0, count, args.fp64_stride))
    eng.timer(reset=True)
    t0 = time.perf_counter()
    for k in sample:
        p = insts[k]
        eng.solve(p['rowptr'], p['col'], p['val'], p['c'], p['lower'], p['upper'], o64)
    fp64_wall = time.perf_counter() - t0
    fp64_dev, _, _ = eng.timer()
    fp64 = {'solves_per_s': len(sample) / (fp64_dev / 1e3), 'wall_solves_per_s': len(sample) / fp64_wall,
            'sample': f'every {args.fp64_stride}th instance ({len(sample)} solves), one at a time through bqp_solve_sync'}
    # e2e: submit every instance from host buffers, collect every primal
    h2d = sum(p['rowptr'].nbytes + p['col'].nbytes + p['val'].nbytes + 3 * p['c'].nbytes for p in insts)
    d2h = 8 * n_tot
    for i in ids:
        eng.release(i)
    t0 = time.perf_counter()
    ids2 = [eng.submit(p['rowptr'], p['col'], p['val'], p['c'], p['lower'], p['upper'], opts) for p in insts]
    for p, i in zip(insts, ids2):
        eng.wait(i)
        eng.fetch(i, p['n'])
    e2e_s = allreduce_max(pg, time.perf_counter() - t0)
    for i in ids2:
        eng.release(i)
    e2e = {'value': allreduce_sum(pg, count) / e2e_s, 'unit': 'solves/s', 'h2d_bytes_per_step': int(h2d),
           'd2h_bytes_per_step': int(d2h), 'api': 'bqp_submit x4096 + bqp_wait + bqp_fetch (pageable host buffers)'}
    cpu = None
    if rank == 0 and world == 1 and not args.quick:
        from oracle import oracle as O
        cs = list(range(0, count, args.cpu_stride))
        t0 = time.perf_counter()
        for k in cs:
            p = boxqp.planted('batch', seed=3, index=k, lower_triplets=True)
            O.solve_box(p['hrow'], p['hcol'], p['hval'], p['c'], p['lower'], p['upper'], tol=args.tol, threads=1)
        cpu_s = time.perf_counter() - t0
        cpu = {'value': len(cs) / cpu_s, 'unit': 'solves/s', 'cores': 1, 'kind': 'port',
               'sample': f'every {args.cpu_stride}th instance ({len(cs)} FP64 reference-FISTA solves, 1 thread each, '
                         'sequential); instances are too small for OpenMP rows'}
    peak, kind = load_peaks()
    achieved = bytes_total / (dev_s / args.steps) / 1e9
    eng.close()
    if rank != 0:
        return
    line = {'metric': METRIC, 'value': value, 'unit': 'solves/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': 1e3 * dev_s / args.steps, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32+f64', 'data': 'synthetic',
            'config': {'workload': f'uneven batch: {count} planted box QPs, n log-uniform [64,16384], 2..6 '
                                   'edges/vertex, l=0, u~U[0.5,2], one running batch, mixed precision',
                       'instances': count, 'sum_n': n_tot, 'sum_nnz': nnz_tot, 'tolerance': args.tol,
                       'generation_s': gen_s,
                       'l2': f'inputs larger than L2: {(8 * nnz_tot + 32 * n_tot) / 1e6:.0f} MB per batch iteration'},
            'batch': {'statuses': statuses, 'iterations_mean': float(np.mean(iters)),
                      'iterations_max': int(np.max(iters)), 'worst_kkt': worst_kkt, 'worst_objective_rel_err': worst_obj},
            'hbm_gbs': achieved, 'wall_ms_per_step': 1e3 * wall / args.steps,
            'fp64_single_instance_loop': fp64, 'speedup_vs_fp64_single_loop': value / fp64['solves_per_s'],
            'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
                         'traffic': None, 'peak_kind': kind, 'scope': 'whole batch solve (algorithmic bytes / device time)'},
            'cpu_baseline': cpu, 'e2e': e2e, 'gpu_launches': int(kernels), 'graph_launches': int(launches),
            'clocks': clocks.summary()}
    print(json.dumps(line), flush=True)


def run_serve(args, world, rank, local, pg):
    """Poisson stream of box-QP requests (n log-uniform [1000, 200000], tolerance 1e-4 or 1e-8 by a
    seeded coin) into the continuous-batching request loop under a 40 GB admission cap."""
    import numpy as np
    import boxqp
    from boxqp.serve import BoxQPServer
    rate, duration = args.rate, args.duration
    st = 4 + 7919 * rank
    arrivals, t, k = [], 0.0, 0
    while True:
        out, st = boxqp.splitmix64(st)
        t += -np.log(1.0 - (out >> 11) * 2.0 ** -53) / rate
        if t >= duration:
            break
        coin, st = boxqp.splitmix64(st)
        arrivals.append((t, k, 1e-4 if coin & 1 else 1e-8))
        k += 1
    # The request bodies are generated before the timed region: a pool of args.pool distinct
    # planted instances (request index k uses instance k mod pool), so that every request is
    # submitted at its scheduled arrival time and a client's latency is measured from it.
    pool_size = min(args.pool, len(arrivals))
    pool = [None] * pool_size
    workers = 8

    def produce(start):
        for i in range(start, pool_size, workers):
            pool[i] = boxqp.planted('serve', seed=4 + rank, index=i)
    producers = [threading.Thread(target=produce, args=(s,), daemon=True) for s in range(workers)]
    for p in producers:
        p.start()
    for p in producers:
        p.join()
    server = BoxQPServer(local, mem_cap_bytes=40 << 30, latency_ms=args.latency_ms)
    # untimed warm-up (with --warmup > 0): every pool instance once, both tolerances, so that the
    # engine's graphs and kernels for all request sizes exist before the first timed arrival
    n_warm = pool_size if args.warmup > 0 else 0
    warm = [server.submit(pool[i]['rowptr'], pool[i]['col'], pool[i]['val'], pool[i]['c'], pool[i]['lower'],
                          pool[i]['upper'], 1e-4 if i & 1 else 1e-8) for i in range(n_warm)]
    for fut in warm:
        fut.result(timeout=300)
    results = []
    lag = []
    barrier(pg)
    t_start = time.perf_counter()
    with ClockSampler(local) as clocks:
        for i, (t_i, idx, tol) in enumerate(arrivals):
            inst = pool[idx % pool_size]
            now = time.perf_counter() - t_start
            if now < t_i:
                time.sleep(t_i - now)
            lag.append(max(0.0, time.perf_counter() - t_start - t_i))
            fut = server.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], tol)
            results.append((inst['n'], inst['fstar'], tol, fut, t_start + t_i))
        done, from_arrival = [], []
        for n, fstar, tol, fut, arrival in results:
            r = fut.result(timeout=300)
            done.append((n, fstar, tol, r))
            # a client's latency: from the request's scheduled arrival (not from its submission,
            # which the generator threads may have delayed) to the result
            from_arrival.append(r.finished - arrival)
        elapsed = time.perf_counter() - t_start
    load = server.load()
    server.close()
    lat = np.array(from_arrival) * 1e3
    service_lat = np.array([r.latency for _, _, _, r in done]) * 1e3
    ok = sum(1 for _, _, _, r in done if r.status == 'optimal')
    worst = {}
    for tol in (1e-4, 1e-8):
        sel = [(n, f, r) for n, f, tt, r in done if tt == tol]
        if sel:
            worst[f'{tol:g}'] = {'requests': len(sel), 'worst_kkt': max(r.stationarity for _, _, r in sel),
                                 'worst_objective_rel_err': max(abs(r.objective - f) / (1 + abs(f)) for _, f, r in sel)}
    thr = allreduce_sum(pg, len(done)) / allreduce_max(pg, elapsed)
    if rank != 0:
        return
    line = {'metric': METRIC, 'value': thr, 'unit': 'solves/s', 'n_gpus': world, 'steps': len(done), 'warmup': n_warm,
            'ms_per_step': float(np.median(lat)), 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f32+f64', 'data': 'synthetic',
            'config': {'workload': f'serving stream: Poisson arrivals {rate:g}/s for {duration:g} s, n log-uniform '
                                   '[1000, 200000], 5 edges/vertex, tolerance 1e-4 or 1e-8, 40 GB admission cap',
                       'request_pool': f'{pool_size} distinct planted instances generated before the timed region; '
                                       'request k carries instance k mod pool',
                       'latency_target_ms': args.latency_ms, 'requests': len(arrivals)},
            'latency_ms': {'p50': float(np.percentile(lat, 50)), 'p99': float(np.percentile(lat, 99)),
                           'p99.9': float(np.percentile(lat, 99.9)), 'max': float(lat.max()), 'mean': float(lat.mean()),
                           'from': 'scheduled arrival'},
            'service_latency_ms': {'p50': float(np.percentile(service_lat, 50)),
                                   'p99': float(np.percentile(service_lat, 99)),
                                   'p99.9': float(np.percentile(service_lat, 99.9)), 'from': 'submission'},
            'arrival_lag_ms_p99': float(np.percentile(np.array(lag) * 1e3, 99)),
            'offered_rate': len(arrivals) / max(arrivals[-1][0], 1e-9) if arrivals else 0.0,
            'optimal': ok, 'peak_resident': load['peak_resident'], 'errors_vs_fp64_checks': worst,
            'e2e': {'value': thr, 'unit': 'solves/s', 'h2d_bytes_per_step': None, 'd2h_bytes_per_step': None,
                    'api': 'BoxQPServer.submit (bqp_submit) from host buffers; latency from each request\'s scheduled '
                           'arrival to its result'},
            'clocks': clocks.summary()}
    print(json.dumps(line), flush=True)


def run_admm(args, world, rank, local, pg):
    """The constrained-QP ADMM inner solve (K = H + sigma I + A' diag(rho) A, Jacobi PCG as
    qp_admm.cpp:262-273) on a 1M-variable system: H the random-graph Hessian (15M nonzeros), A
    500k rows of 8 entries.  A step is one inner solve from x = 0 to the reference's first-
    iteration accuracy 1e-7 (1 + max|rhs|), through bqp_admm_solve (host rhs and x copied in and
    out every step); value = CG iterations per second."""
    import numpy as np
    import boxqp
    from boxqp.admm import AdmmSystem
    n, m, per_row = 1000000, 500000, 8
    inst = boxqp.planted('graph1m', seed=1 + rank)
    rng = np.random.default_rng(11 + rank)
    cols = np.sort(rng.integers(0, n, size=(m, per_row)), axis=1)
    a_rowptr = (np.arange(m + 1) * per_row).astype(np.int32)
    a_col = cols.reshape(-1).astype(np.int32)
    a_val = rng.normal(size=m * per_row)
    rho = np.where(rng.random(m) < 0.1, 10.0, 0.1)
    sigma = 1e-8
    rhs = rng.normal(size=n)
    accuracy = 1e-7 * (1.0 + np.max(np.abs(rhs)))
    max_inner = min(4000, 2 * n + 20)
    sysm = AdmmSystem(inst['rowptr'], inst['col'], inst['val'], a_rowptr, a_col, a_val, n, device=local)
    sysm.set_rho(rho, sigma)
    x0 = np.zeros(n)
    for _ in range(args.warmup):
        sysm.solve(rhs, x0, accuracy, max_inner)
    barrier(pg)
    inner_total, resid = 0, 0.0
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            x, inner, resid = sysm.solve(rhs, x0, accuracy, max_inner)
            inner_total += inner
        wall = allreduce_max(pg, time.perf_counter() - t0)
    nnz_h, nnz_a = int(inst['rowptr'][-1]), m * per_row
    # per CG iteration: H, A and A' (values + columns), rho and t, and eight n-vectors read or written
    it_bytes = 12.0 * nnz_h + 2 * 12.0 * nnz_a + 4.0 * (2 * n + m + 2) + 16.0 * m + 8.0 * 8 * n
    ms_per_it = 1e3 * wall / max(inner_total, 1)
    peak, kind = load_peaks()
    cpu = None
    if rank == 0 and world == 1 and not args.quick:
        # the CPU restatement (pure-Python loops) on a 2,000-variable sample of the same recipe
        from oracle.admm_pcg import AdmmSystemOracle
        sn, sm = 2000, 1000
        small = boxqp.planted('graph10k', seed=3, n=sn)
        srng = np.random.default_rng(5)
        scols = np.sort(srng.choice(sn, size=(sm, per_row)), axis=1)
        sa = ((np.arange(sm + 1) * per_row).astype(np.int32), scols.reshape(-1).astype(np.int32),
              srng.normal(size=sm * per_row))
        o = AdmmSystemOracle((small['rowptr'], small['col'], small['val']), sa, sn)
        o.set_rho(np.where(srng.random(sm) < 0.1, 10.0, 0.1), sigma)
        srhs = srng.normal(size=sn)
        t1 = time.perf_counter()
        _, sinner, _ = o.solve(srhs, np.zeros(sn), 1e-7 * (1 + np.max(np.abs(srhs))), 30)
        cdt = time.perf_counter() - t1
        cpu = {'value': sinner / cdt, 'unit': 'CG iterations/s', 'cores': 1, 'kind': 'port',
               'sample': f'{sinner} inner iterations of the CPU restatement on a {sn}-variable, {sm}-row system'}
    if rank == 0:
        out = {'metric': 'ADMM inner-solve CG iterations/s (K = H + sigma I + A\' diag(rho) A)',
               'value': allreduce_sum(pg, inner_total) / wall, 'unit': 'CG iterations/s', 'n_gpus': world,
               'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * wall / args.steps,
               'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
               'data': 'synthetic',
               'config': {'workload': f'ADMM x-update system: H random-graph Hessian n={n} ({nnz_h} nonzeros), '
                                      f'A {m} rows x {per_row} entries, sigma 1e-8, rho 0.1 (10 on 10 % of rows)',
                          'accuracy': accuracy, 'max_inner': max_inner, 'parallelism': f'replicas x{world}',
                          'l2': 'inputs larger than L2: one iteration streams ~330 MB'},
               'inner_per_step': inner_total / args.steps, 'final_max_residual': resid,
               'roofline': {'bound': 'hbm', 'achieved': it_bytes / (ms_per_it * 1e-3) / 1e9, 'peak': peak,
                            'unit': 'GB/s', 'frac': it_bytes / (ms_per_it * 1e-3) / 1e9 / peak, 'traffic': None,
                            'peak_kind': kind, 'scope': 'one CG iteration (4 kernels), algorithmic bytes / wall time'},
               'cpu_baseline': cpu,
               'e2e': {'value': allreduce_sum(pg, inner_total) / wall, 'unit': 'CG iterations/s',
                       'h2d_bytes_per_step': 16 * n, 'd2h_bytes_per_step': 8 * n,
                       'api': 'bqp_admm_solve (rhs and x from host memory, x back)'},
               'gpu_launches': int(inner_total * 4 + args.steps * 2), 'clocks': clocks.summary()}
        print(json.dumps(out))
    sysm.close()


def run_case(args):
    """Small runs for kernel profilers (ncu): `--case solve` one solve of the workload (with
    BOXQP_LAUNCH=stream its kernels run as plain launches, which per-kernel profilers can see;
    inside the conditional graph they cannot), `--case step` the FISTA step kernel alone, launched
    1 + --steps times on the uploaded instance.  Prints a line of text, not the bench JSON."""
    import boxqp
    inst, _ = make_workload(args.workload, 0)
    eng = boxqp.Engine(0)
    try:
        if args.case == 'solve':
            o = boxqp.options_struct(args.tol, 60.0, 200000, args.precision)
            x, st = eng.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
            print({k: v for k, v in st.as_dict().items() if k in ('status_name', 'iterations', 'polish_iterations',
                                                                 'checks', 'device_seconds', 'bytes')})
        else:
            o = boxqp.options_struct(args.tol, 60.0, 0, args.precision)
            ident = eng.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
            eng.wait(ident)
            ms, nbytes = eng.profile_step(ident, args.steps)
            print(f'step kernel: {ms * 1e3:.1f} us per launch, {nbytes / 1e6:.1f} MB algorithmic, '
                  f'{nbytes / ms / 1e6:.0f} GB/s')
            eng.release(ident)
    finally:
        eng.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=None,
                    help='timed steps (default: 100 single solves, 3 batch solves, ignored for serve)')
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', choices=['ours', 'reference'], default='ours')
    ap.add_argument('--workload', default='graph1m',
                    choices=['graph1m', 'grid', 'graph10k', 'tridiagonal', 'batch', 'serve', 'admm'])
    ap.add_argument('--instances', type=int, default=4096, help='batch: number of instances')
    ap.add_argument('--fp64-stride', type=int, default=1, help='batch: FP64 single-solve loop over every k-th')
    ap.add_argument('--cpu-stride', type=int, default=32, help='batch: CPU baseline over every k-th instance')
    ap.add_argument('--rate', type=float, default=200.0, help='serve: arrivals per second')
    ap.add_argument('--duration', type=float, default=60.0, help='serve: seconds of arrivals')
    ap.add_argument('--latency-ms', type=float, default=2.0, help='serve: device launch length target')
    ap.add_argument('--pool', type=int, default=512, help='serve: distinct request instances generated up front')
    ap.add_argument('--precision', default='mixed', choices=['mixed', 'fp64'])
    ap.add_argument('--tol', type=float, default=None, help='KKT tolerance (default 1e-6; 1e-7 for tridiagonal)')
    ap.add_argument('--quick', action='store_true', help='skip e2e, FP64 and CPU legs')
    ap.add_argument('--cpu-threads', type=int, default=0,
                    help='host threads of the reference CPU solve (cpu_baseline and --impl reference; 0: all cores)')
    ap.add_argument('--case', choices=['solve', 'step'], default=None,
                    help='profiling run instead of the benchmark: one solve, or the step kernel alone --steps times')
    args = ap.parse_args()
    if args.tol is None:
        args.tol = 1e-7 if args.workload == 'tridiagonal' else 1e-6
    if args.case:
        args.steps = 3 if args.steps is None else args.steps
        run_case(args)
        return
    if args.steps is None:
        args.steps = 3 if args.workload in ('batch', 'admm') else (10 if args.impl == 'reference' else 100)
    world, rank, local, pg = dist_setup(args)
    if args.impl == 'reference' and args.workload == 'admm':
        if rank == 0:
            print(json.dumps({'impl': 'reference', 'unavailable': 'the reference runs this inner solve only inside '
                              'its ADMM loop (qp_admm.cpp:262-273); the CPU restatement is timed as cpu_baseline'}))
    elif args.impl == 'reference':
        run_reference(args, world, rank, pg)
    elif args.workload == 'batch':
        run_batch(args, world, rank, local, pg)
    elif args.workload == 'serve':
        run_serve(args, world, rank, local, pg)
    elif args.workload == 'admm':
        run_admm(args, world, rank, local, pg)
    else:
        run_ours(args, world, rank, local, pg)
    if pg:
        pg.destroy_process_group()


if __name__ == '__main__':
    main()
