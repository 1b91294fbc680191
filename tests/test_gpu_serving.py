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


def test_uploads_paused_by_a_finishing_launch_resume_exactly():
    """Large solves submitted while a long launch runs upload in chunks; when the launch ends an
    upload in progress pauses and resumes during the next launch.  Every result equals its solo
    run bit for bit."""
    eng = boxqp.Engine(0)
    try:
        long_inst = boxqp.planted('graph1m', seed=5, n=200000)
        big = [boxqp.planted('graph1m', seed=6 + k, n=300000) for k in range(3)]
        o_long = boxqp.options_struct(1e-9, 60.0, 200000, 'fp64')
        o_big = boxqp.options_struct(1e-6, 60.0, 200000, 'mixed')
        args = lambda i: (i['rowptr'], i['col'], i['val'], i['c'], i['lower'], i['upper'])
        solo = [eng.solve(*args(i), o_big) for i in big]
        ids = [eng.submit(*args(long_inst), o_long)]
        ids += [eng.submit(*args(i), o_big, copy=(k % 2 == 0)) for k, i in enumerate(big)]
        for ident in ids:
            assert eng.wait(ident, 120.0)
        for ident, inst, (xs, ss) in zip(ids[1:], big, solo):
            x, st = eng.fetch(ident, inst['n'])
            assert boxqp.STATUS_NAMES[st.status] == 'optimal'
            assert np.array_equal(x, xs) and st.iterations == ss.iterations and st.objective == ss.objective
        _, st_long = eng.fetch(ids[0], long_inst['n'])
        assert boxqp.STATUS_NAMES[st_long.status] == 'optimal'
        for ident in ids:
            eng.release(ident)
    finally:
        eng.close()
