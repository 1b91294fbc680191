"""Command-line drop-in for the box-QP branch of the reference CLI on the GB300 engine.

    python -m boxqp.cli MODEL.qplib --json [--backend cuda] [--threads N] [--tolerance T]
                        [--iteration-limit N] [--time-limit S] [--no-scaling]
                        [--precision fp64|mixed|fp64_exact] [--max-columns N]

Same options, JSON record and exit codes as the reference's QPLIB branch
(02-software/solver/src/main.cpp:64-163, docs/CLI_API.md): exit 0 for optimal, 1 for an honest
non-optimal outcome, 2 for a rejected input or option.  Only the CUDA backend exists here; box
QPs with linear constraints are rejected for it as in the reference (src/main.cpp:145).
"""
import json
import math
import sys
import time


def _num(v):
    return v if isinstance(v, float) and math.isfinite(v) else (None if isinstance(v, float) else v)


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    if len(argv) == 1 and argv[0] == '--version':
        print('GB300 box-QP engine (FISTA + FP64 verification), C-ABI libboxqp')
        return 0
    if not argv:
        print('Usage: boxqp.cli MODEL.qplib [--json] [--backend cuda] [--time-limit seconds]', file=sys.stderr)
        return 2
    try:
        from .api import QpOptions, solve_accelerated_box
        from .qplib import read_qplib
        path, args = argv[0], argv[1:]
        as_json, backend, threads, precision, max_columns = False, 'cpu', 1, 'fp64', 100000
        opt = QpOptions()
        i = 0
        while i < len(args):
            a = args[i]
            nxt = args[i + 1] if i + 1 < len(args) else None
            if a == '--json':
                as_json = True
            elif a == '--no-scaling':
                opt.scaling = False
            elif a in ('--threads', '--backend', '--tolerance', '--iteration-limit', '--time-limit', '--precision',
                       '--max-columns') and nxt is not None:
                i += 1
                if a == '--threads':
                    threads = int(float(nxt))
                elif a == '--backend':
                    backend = nxt
                elif a == '--tolerance':
                    opt.tolerance = float(nxt)
                elif a == '--iteration-limit':
                    opt.iteration_limit = int(float(nxt))
                elif a == '--time-limit':
                    opt.time_limit = float(nxt)
                elif a == '--precision':
                    precision = nxt
                else:
                    max_columns = int(float(nxt))
            else:
                raise RuntimeError('Unknown or incomplete option: ' + a)
            i += 1
        if backend not in ('cpu', 'cuda'):
            raise RuntimeError('Backend must be cpu or cuda')
        if threads < 1 or threads > 256:
            raise RuntimeError('Threads must be between 1 and 256')
        if not (opt.tolerance > 0) or opt.time_limit < 0:
            raise RuntimeError('Tolerance must be positive; limits and gap must be nonnegative')
        if precision not in ('fp64', 'mixed', 'fp64_exact'):
            raise RuntimeError('Precision must be fp64, mixed or fp64_exact')
        if backend == 'cpu':
            raise RuntimeError('this engine is the CUDA backend; use the reference CLI for --backend cpu')
        if not path.endswith('.qplib'):
            raise RuntimeError('CUDA currently supports QPLIB box QPs only')
        start = time.perf_counter()
        with open(path) as f:
            problem, rows = read_qplib(f.read(), max_columns)
        if rows:
            raise RuntimeError('CUDA currently supports convex box QPs; use CPU for linearly constrained QP')
        opt.threads = threads
        opt.precision = precision
        r = solve_accelerated_box(problem, opt, True)
        seconds = time.perf_counter() - start
        if as_json:
            rec = {'status': r.status, 'algorithm': r.algorithm, 'threads': threads,
                   'optimality_verified': r.optimality_verified, 'iterations': r.iterations, 'total_seconds': seconds,
                   'rows': 0, 'columns': problem.n, 'objective': _num(r.objective),
                   'primal_residual': _num(r.primal_residual), 'stationarity_residual': _num(r.stationarity_residual),
                   'complementarity_residual': _num(r.complementarity_residual),
                   'dual_bound_minimization_sense': _num(r.dual_bound), 'relative_gap': _num(r.relative_gap),
                   'primal': [float(v) for v in r.primal], 'row_dual': []}
            print(json.dumps(rec))
        else:
            print(f'status: {r.status}\nobjective: {r.objective!r}\niterations: {r.iterations}\n'
                  f'stationarity_residual: {r.stationarity_residual!r}')
        return 0 if r.status == 'optimal' else 1
    except Exception as exc:  # input and option errors: exit 2, as the reference CLI
        print(str(exc), file=sys.stderr)
        return 2


if __name__ == '__main__':
    sys.exit(main())
