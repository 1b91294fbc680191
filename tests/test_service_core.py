"""The service route's request handler without the web framework (CPU): the replies for errors
the engine reports through a request's future (entries the device's admission pass rejects, a
zero Hessian, a failed admission) and at submission, with a fake request loop standing in for the
GPU engine."""
import asyncio
from concurrent.futures import Future

import numpy as np
import pytest

from boxqp import service_core
from boxqp._native import EngineError


class FailingServer:
    """Raises `at_submit` from submit, or completes every request's future with `in_future`."""

    def __init__(self, at_submit=None, in_future=None):
        self.at_submit = at_submit
        self.in_future = in_future

    def submit(self, rowptr, col, val, c, lower, upper, tolerance, precision, time_limit):
        if self.at_submit is not None:
            raise self.at_submit
        fut = Future()
        fut.set_exception(self.in_future)
        return fut


def small_request():
    # 2x2 diagonal Hessian, box [0, 1]
    rowptr = np.array([0, 1, 2], np.int32)
    col = np.array([0, 1], np.int32)
    val = np.array([2.0, 3.0])
    c = np.array([-1.0, 1.0])
    return rowptr, col, val, c, np.zeros(2), np.ones(2)


def reply(server):
    service_core.set_server(server)
    try:
        return asyncio.run(service_core.solve_arrays(*small_request(), tolerance=1e-6, precision='mixed',
                                                     time_limit=5.0))
    finally:
        service_core.set_server(None)


@pytest.mark.parametrize('where', ['submit', 'future'])
def test_rejected_entries_reply_input_rejected(where):
    exc = ValueError('Invalid Hessian')
    r = reply(FailingServer(at_submit=exc) if where == 'submit' else FailingServer(in_future=exc))
    assert r['status'] == 'input_rejected' and 'Invalid Hessian' in r['message']
    assert r['objective'] is None and r['primal'] == []


@pytest.mark.parametrize('where', ['submit', 'future'])
def test_zero_hessian_replies_unsupported(where):
    exc = EngineError(7, 'Zero-Hessian models use the CPU LP path')
    r = reply(FailingServer(at_submit=exc) if where == 'submit' else FailingServer(in_future=exc))
    assert r['status'] == 'unsupported' and 'Zero-Hessian' in r['message']


@pytest.mark.parametrize('where', ['submit', 'future'])
def test_admission_refusal_is_413(where):
    exc = EngineError(4, 'solve does not fit under the device-memory cap')
    with pytest.raises(service_core.HttpError) as e:
        reply(FailingServer(at_submit=exc) if where == 'submit' else FailingServer(in_future=exc))
    assert e.value.status == 413


def test_failed_solve_replies_engine_error():
    r = reply(FailingServer(in_future=EngineError(8, 'admission: device memory')))
    assert r['status'] == 'engine_error' and 'device memory' in r['message']
