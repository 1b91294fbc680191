"""The service route's request handling on the real engine (needs a GPU).

boxqp.service_core holds what POST /qp/solve does between the HTTP layer and the GPU (the web
framework is not needed for it, and is absent on some GPU hosts).  These tests drive it with a
real continuous-batching request loop (BoxQPServer) and check:
  * an .npz request is solved and its primal verifies with the oracle's check_qp_solution at the
    requested tolerance, objective to 1e-7 of the planted optimum;
  * concurrent requests overlap in the same running batch and each gets its own answer;
  * a request that can never fit under the loop's device-memory cap is refused with 413;
  * an admission whose device allocation fails (host-side fault injection) answers
    "engine_error" with the engine's out-of-memory message, and the next request is served.
"""
import asyncio
import io

import numpy as np
import pytest

import boxqp
from boxqp import service_core as core
from boxqp.serve import BoxQPServer
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def npz_body(inst):
    buf = io.BytesIO()
    np.savez(buf, rowptr=inst['rowptr'], col=inst['col'], val=inst['val'], c=inst['c'], lower=inst['lower'],
             upper=inst['upper'])
    return buf.getvalue()


def arrays(inst):
    return inst['rowptr'], inst['col'], inst['val'], inst['c'], inst['lower'], inst['upper']


@pytest.fixture()
def server():
    srv = BoxQPServer(0, mem_cap_bytes=8 << 30, latency_ms=2.0)
    core.set_server(srv)
    yield srv
    core.set_server(None)
    srv.close()


def test_npz_request_through_the_route_on_the_engine(server):
    inst = boxqp.planted('graph10k', seed=51, n=20000, lower_triplets=True)
    reply = asyncio.run(core.solve_npz(npz_body(inst), tolerance=1e-6, precision='mixed', time_limit=20.0))
    assert reply['engine'] == 'gb300' and reply['status'] == 'optimal', reply
    x = np.asarray(reply['primal'])
    chk = O.check(inst['hrow'], inst['hcol'], inst['hval'], inst['c'], inst['lower'], inst['upper'], x, tol=1e-6)
    assert chk['verified'] == 1.0
    assert abs(chk['objective'] - inst['fstar']) <= 1e-7 * (1 + abs(inst['fstar']))
    assert reply['objective'] == pytest.approx(chk['objective'], rel=1e-12)


def test_concurrent_requests_share_the_batch(server):
    """Six requests at once (FP64 iterations to 1e-8, long enough to overlap): each gets its own
    verified answer, and the loop held several of them resident together."""
    insts = [boxqp.planted('graph10k', seed=60 + k, n=100000 + 20000 * k) for k in range(6)]

    async def all_of():
        return await asyncio.gather(*[core.solve_arrays(*arrays(p), tolerance=1e-8, precision='fp64',
                                                        time_limit=30.0) for p in insts])
    replies = asyncio.run(all_of())
    for p, r in zip(insts, replies):
        assert r['status'] == 'optimal' and r['columns'] == p['n']
        assert abs(r['objective'] - p['fstar']) <= 1e-7 * (1 + abs(p['fstar']))
    assert server.load()['peak_resident'] >= 2


def test_request_above_the_memory_cap_is_refused():
    small = BoxQPServer(0, mem_cap_bytes=1 << 20, latency_ms=2.0)  # 1 MiB: a 20k-variable solve never fits
    core.set_server(small)
    try:
        inst = boxqp.planted('graph10k', seed=52, n=20000)
        with pytest.raises(core.HttpError) as err:
            asyncio.run(core.solve_arrays(*arrays(inst), tolerance=1e-6))
        assert err.value.status == 413 and 'memory cap' in err.value.detail
    finally:
        core.set_server(None)
        small.close()


def test_out_of_memory_at_admission_is_reported_and_the_loop_recovers(server):
    inst = boxqp.planted('graph10k', seed=53, n=20000)
    server.engine.inject_admission_oom(1)
    reply = asyncio.run(core.solve_arrays(*arrays(inst), tolerance=1e-6, time_limit=20.0))
    assert reply['status'] == 'engine_error' and 'out of memory' in reply['message'], reply
    again = asyncio.run(core.solve_arrays(*arrays(inst), tolerance=1e-6, time_limit=20.0))
    assert again['status'] == 'optimal'
    assert abs(again['objective'] - inst['fstar']) <= 1e-7 * (1 + abs(inst['fstar']))
