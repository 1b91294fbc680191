"""Autotuner of the FISTA step kernel's SpMV structure.

For each precision and each class of instances (average nonzeros per row x number of rows) it
times every kernel variant -- block-staged tile (0), warp-staged rows (64) and 1/2/4/8/16/32
lanes per row -- on a representative planted instance, with the engine's own step-kernel timer
(bqp_profile_step: CUDA events around back-to-back launches on the engine stream), and writes
the fastest per class to boxqp/tuning.json.  Run on the target GPU:

    python hypergrey-sih-26_gb300/boxqp/autotune.py [--quick]

The engine reads the table through tuned_variant(); a variant named explicitly in the options
always wins.
"""
import argparse
import json
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
TABLE = HERE / 'tuning.json'
VARIANTS = [0, 64, 1, 2, 4, 8, 16, 32]
# (row-length bucket lower bound, upper bound, generator: family preset and edges/vertex)
ROW_CLASSES = [(0, 4, ('graph10k', 1)), (4, 6, ('grid', None)), (6, 9, ('graph10k', 3)),
               (9, 13, ('graph10k', 5)), (13, 20, ('graph10k', 7)), (20, 48, ('graph10k', 14)),
               (48, 10 ** 9, ('graph10k', 40))]
SIZE_CLASSES = [(0, 30000, 16384), (30000, 400000, 131072), (400000, 10 ** 12, 1048576)]

_table = None


def load_table():
    global _table
    if _table is None:
        _table = json.loads(TABLE.read_text()) if TABLE.exists() else {'entries': []}
    return _table


def tuned_variant(precision, n, nnz):
    """Kernel variant for an instance from the committed table, or -1 (engine default)."""
    if precision == 'fp64_exact':
        return -1
    avg = nnz / max(n, 1)
    for e in load_table().get('entries', []):
        if e['precision'] == precision and e['row_lo'] <= avg < e['row_hi'] and e['n_lo'] <= n < e['n_hi']:
            return int(e['variant'])
    return -1


def _instance(boxqp, family, epv, n):
    n = min(n, 20000000 // (2 * epv + 1)) if epv else n  # keep samples under ~20M nonzeros
    if family == 'grid':
        side = int(round(n ** 0.5))
        return boxqp.planted('grid', seed=7, n=side * side)
    spec = boxqp.planted_spec('graph10k', seed=7, n=n)
    spec.edges_per_vertex = epv
    return boxqp.planted(spec=spec)


def tune(quick=False, launches=30):
    sys.path.insert(0, str(HERE.parent))
    import boxqp
    eng = boxqp.Engine(0)
    entries = []
    sizes = SIZE_CLASSES[1:] if quick else SIZE_CLASSES
    for precision in ('mixed', 'fp64'):
        for (n_lo, n_hi, n) in sizes:
            for (row_lo, row_hi, (family, epv)) in ROW_CLASSES:
                inst = _instance(boxqp, family, epv, n)
                times = {}
                for v in VARIANTS:
                    o = boxqp.options_struct(1e-6, 60.0, 0, precision, kernel_variant=v)
                    ident = eng.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'],
                                       inst['upper'], o)
                    eng.wait(ident)
                    ms, nbytes = eng.profile_step(ident, launches)
                    eng.release(ident)
                    times[str(v)] = ms
                best = min(times, key=times.get)
                entries.append({'precision': precision, 'row_lo': row_lo, 'row_hi': row_hi, 'n_lo': n_lo,
                                'n_hi': n_hi, 'variant': int(best), 'sample_n': inst['n'],
                                'sample_nnz': inst['nnz'], 'ms': times,
                                'gbs': nbytes / (times[best] * 1e-3) / 1e9})
                print(precision, n, family, epv, 'avg %.1f' % (inst['nnz'] / inst['n']), 'best', best,
                      {k: round(t * 1e3, 1) for k, t in times.items()}, flush=True)
    eng.close()
    out = {'device': boxqp.cuda_device_name(), 'generated': time.strftime('%Y-%m-%dT%H:%M:%SZ', time.gmtime()),
           'launches_per_timing': launches, 'entries': entries}
    TABLE.write_text(json.dumps(out, indent=1) + '\n')
    return out


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--quick', action='store_true')
    a = ap.parse_args()
    tune(quick=a.quick)
