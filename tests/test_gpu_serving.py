"""Continuous batching on the GPU: solves that arrive while others are running join the running
batch, overlap on the device, and give the same result as when run alone."""
import time

import numpy as np
import pytest

import boxqp
from boxqp.serve import BoxQPServer
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_staggered_requests_overlap_and_match_solo_runs():
    reqs = []
    for i in range(14):
        inst = boxqp.planted('serve', seed=4, index=i, n=[3000, 20000, 60000][i % 3], lower_triplets=True)
        tol = 1e-4 if i % 2 else 1e-8
        reqs.append((inst, tol))
    server = BoxQPServer(0, mem_cap_bytes=8 << 30, latency_ms=1.0)
    try:
        solo = []
        for inst, tol in reqs:
            r = server.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper'],
                              tol).result(timeout=120)
            solo.append(r)
        futs = []
        for k, (inst, tol) in enumerate(reqs):
            futs.append(server.submit(inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'],
                                      inst['upper'], tol))
            # a burst of six (queued behind the first launch, so admitted together), then arrivals
            # staggered into the running batch
            if k >= 6:
                time.sleep(0.001 * (k % 3))
        mixed = [f.result(timeout=120) for f in futs]
        load = server.load()
    finally:
        server.close()
    assert load['peak_resident'] >= 2
    for (inst, tol), a, b in zip(reqs, solo, mixed):
        assert a.status == b.status == 'optimal'
        assert np.array_equal(a.x, b.x) and a.iterations == b.iterations
        chk = O.check(inst['hrow'], inst['hcol'], inst['hval'], inst['c'], inst['lower'], inst['upper'], b.x, tol=tol)
        assert chk['verified'] == 1.0
        # objective within 1e-7 relative at tight tolerances, within the tolerance at loose ones
        assert abs(chk['objective'] - inst['fstar']) <= max(1e-7, tol) * (1 + abs(inst['fstar']))
