"""The FastAPI box-QP route and the request loop's host logic (CPU: a fake request loop stands in
for the GPU engine)."""
import io
import threading
import time
from concurrent.futures import Future

import numpy as np
import pytest

pytest.importorskip('fastapi')
uvicorn = pytest.importorskip('uvicorn')
requests = pytest.importorskip('requests')

import boxqp  # noqa: E402
from boxqp import service  # noqa: E402
from boxqp.serve import SolveResult  # noqa: E402


class FakeServer:
    """Answers each request from a background thread after a delay, like the engine's collector."""

    def __init__(self, delay=0.05):
        self.delay = delay
        self.submitted = []
        self.max_in_flight = 0
        self._in_flight = 0
        self._lock = threading.Lock()

    def submit(self, rowptr, col, val, c, lower, upper, tolerance, precision, time_limit):
        fut = Future()
        t0 = time.perf_counter()
        with self._lock:
            self.submitted.append((len(c), tolerance, precision))
            self._in_flight += 1
            self.max_in_flight = max(self.max_in_flight, self._in_flight)

        def done():
            time.sleep(self.delay)
            with self._lock:
                self._in_flight -= 1
            x = np.clip(np.zeros(len(c)), lower, upper)
            fut.set_result(SolveResult('optimal', x, float('-inf') if len(c) == 3 else -1.0, 1e-9, 0.0, 50, 5, 1e-3,
                                       t0, time.perf_counter()))
        threading.Thread(target=done, daemon=True).start()
        return fut

    def load(self):
        return {'queued': 0, 'running': self._in_flight, 'peak_resident': self.max_in_flight, 'resident_bytes': 0}


class Http:
    """The app served by uvicorn on 127.0.0.1 in a background thread."""

    def __init__(self, port):
        self.base = f'http://127.0.0.1:{port}'

    def post(self, path, **kw):
        return requests.post(self.base + path, timeout=30, **kw)

    def get(self, path):
        return requests.get(self.base + path, timeout=30)


@pytest.fixture(scope='module')
def http():
    import socket
    sock = socket.socket()
    sock.bind(('127.0.0.1', 0))
    port = sock.getsockname()[1]
    sock.close()
    config = uvicorn.Config(service.app, host='127.0.0.1', port=port, log_level='error')
    srv = uvicorn.Server(config)
    t = threading.Thread(target=srv.run, daemon=True)
    t.start()
    for _ in range(200):
        if srv.started:
            break
        time.sleep(0.05)
    yield Http(port)
    srv.should_exit = True
    t.join(timeout=5)


@pytest.fixture
def client(http):
    fake = FakeServer()
    service.set_server(fake)
    yield http, fake
    service.set_server(None)


def problem(n=50):
    p = boxqp.planted('graph10k', seed=3, n=n)
    return p


def test_json_solve_roundtrip_and_json_safety(client):
    c, fake = client
    p = problem(3)
    body = {'rowptr': p['rowptr'].tolist(), 'col': p['col'].tolist(), 'val': p['val'].tolist(),
            'cost': p['c'].tolist(), 'lower': [0.0, None, 0.0], 'upper': [1.0, 1.0, None], 'tolerance': 1e-8}
    r = c.post('/qp/solve', json=body).json()
    assert r['engine'] == 'gb300' and r['status'] == 'optimal'
    assert r['objective'] is None  # -inf is not JSON: null
    assert len(r['primal']) == 3 and fake.submitted[0] == (3, 1e-8, 'mixed')


def test_npz_body(client):
    c, fake = client
    p = problem(80)
    buf = io.BytesIO()
    np.savez(buf, rowptr=p['rowptr'], col=p['col'], val=p['val'], c=p['c'], lower=p['lower'], upper=p['upper'])
    r = c.post('/qp/solve?tolerance=1e-4&precision=fp64&return_primal=false', data=buf.getvalue(),
               headers={'content-type': 'application/x-npz'}).json()
    assert r['status'] == 'optimal' and r['primal'] == [] and r['columns'] == 80
    assert fake.submitted[-1] == (80, 1e-4, 'fp64')


@pytest.mark.parametrize('mutate,code', [
    (lambda b: b.update(rowptr=[0, 1]), 400),
    (lambda b: b.update(col=[99] * len(b['col'])), 400),
    (lambda b: b.update(val=[float('nan')] + b['val'][1:]), 400),
    (lambda b: b.update(tolerance=0.0), 422),
    (lambda b: b.update(precision='fp16'), 422),
])
def test_invalid_requests_are_rejected_before_the_engine(client, mutate, code):
    c, fake = client
    p = problem(20)
    body = {'rowptr': p['rowptr'].tolist(), 'col': p['col'].tolist(), 'val': p['val'].tolist(),
            'cost': p['c'].tolist(), 'lower': p['lower'].tolist(), 'upper': p['upper'].tolist()}
    mutate(body)
    import json
    raw = json.dumps(body)  # NaN travels as a bare literal, as a non-strict client would send it
    assert c.post('/qp/solve', data=raw, headers={'content-type': 'application/json'}).status_code == code
    assert fake.submitted == []


def test_requests_overlap_instead_of_429(client):
    """Unlike the reference's single compute slot, concurrent requests are all accepted and run together."""
    c, fake = client
    fake.delay = 0.3
    p = problem(30)
    body = {'rowptr': p['rowptr'].tolist(), 'col': p['col'].tolist(), 'val': p['val'].tolist(),
            'cost': p['c'].tolist(), 'lower': p['lower'].tolist(), 'upper': p['upper'].tolist()}
    results = []
    threads = [threading.Thread(target=lambda: results.append(c.post('/qp/solve', json=body))) for _ in range(6)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert [r.status_code for r in results] == [200] * 6
    assert fake.max_in_flight >= 2
    assert c.get('/qp/load').json()['peak_resident'] >= 2
