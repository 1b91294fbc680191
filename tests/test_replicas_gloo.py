"""Multi-GPU is replicas only: each rank solves its own instances, and bench.py combines the ranks
with a barrier, the max of the per-rank times and the sum of the solves.  This runs that host logic
as two gloo ranks on the CPU."""
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

WORKER = r'''
import os, sys, time
sys.path[:0] = [{root!r}]
import bench
args = type('A', (), {{}})()
world, rank, local, pg = bench.dist_setup(args)
assert world == 2 and pg is not None
bench.barrier(pg)
t = 0.25 if rank == 0 else 0.5                      # per-rank timed region
worst = bench.allreduce_max(pg, t)
solves = bench.allreduce_sum(pg, 10 * (rank + 1))   # units processed per rank
print(f'RANK{{rank}} {{worst}} {{solves}} {{solves / worst}}', flush=True)
pg.destroy_process_group()
'''


def test_two_gloo_ranks_aggregate_like_the_benchmark():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    code = WORKER.format(root=str(ROOT))
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE='2', RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR='127.0.0.1',
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, '-c', code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
    lines = sorted(o.strip().splitlines()[-1] for o, _ in outs)
    for rank, line in enumerate(lines):
        name, worst, solves, rate = line.split()
        assert name == f'RANK{rank}'
        assert float(worst) == 0.5 and float(solves) == 30.0 and float(rate) == 60.0
