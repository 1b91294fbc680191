"""Small, self-contained runs of the engine for profilers (ncu) and quick timing.

    python hypergrey-sih-26_gb300/boxqp/profile_case.py solve graph1m mixed
        one solve of the 1M-variable random-graph workload (BOXQP_LAUNCH=stream makes its kernels
        visible to per-kernel profilers, which cannot see inside conditional graphs)
    python hypergrey-sih-26_gb300/boxqp/profile_case.py step graph1m mixed 3
        uploads the instance and launches its FISTA step kernel 1 + 3 times alone

Presets: graph1m (n = 1,000,000, 7 edges/vertex), grid (1024 x 1024), graph10k, batch (instance 0).
"""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

import boxqp  # noqa: E402


def main(argv):
    mode, preset, precision = argv[1], argv[2], argv[3]
    launches = int(argv[4]) if len(argv) > 4 else 3
    seed = {'graph1m': 1, 'grid': 2, 'graph10k': 0, 'batch': 3}.get(preset, 1)
    inst = boxqp.planted(preset, seed=seed)
    eng = boxqp.Engine(0)
    try:
        if mode == 'solve':
            o = boxqp.options_struct(1e-6, 60.0, 200000, precision)
            x, st = eng.solve(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
            print({k: v for k, v in st.as_dict().items() if k in ('status_name', 'iterations', 'polish_iterations',
                                                                 'checks', 'device_seconds', 'bytes')})
        elif mode == 'step':
            o = boxqp.options_struct(1e-6, 60.0, 0, precision)
            ident = eng.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'], o)
            eng.wait(ident)
            ms, nbytes = eng.profile_step(ident, launches)
            print(f'step kernel: {ms * 1e3:.1f} us per launch, {nbytes / 1e6:.1f} MB algorithmic, '
                  f'{nbytes / ms / 1e6:.0f} GB/s')
            eng.release(ident)
        else:
            raise SystemExit(__doc__)
    finally:
        eng.close()


if __name__ == '__main__':
    main(sys.argv)
