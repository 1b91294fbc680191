import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT), str(ROOT / 'hypergrey-sih-26_gb300')):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (runs on the GB300 box)')


@pytest.fixture(scope='session', autouse=True)
def built_library():
    """Builds libboxqp.so and the oracle if a source is newer than the build."""
    import build as engine_build
    from oracle import oracle as O
    engine_build.build()
    O.build_oracle()
    return engine_build.LIB


@pytest.fixture(scope='session')
def golden():
    import json
    import numpy as np
    d = json.loads((ROOT / 'tests' / 'golden' / 'reference_cases.json').read_text())
    x = np.load(ROOT / 'tests' / 'golden' / 'reference_x.npz')
    return d, {k: x[k] for k in x.files}


@pytest.fixture(scope='session')
def engine():
    import boxqp
    eng = boxqp.Engine(0)
    yield eng
    eng.close()
