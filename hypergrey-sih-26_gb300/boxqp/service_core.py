"""Request handling of the box-QP service route, without the web framework.

boxqp.service mounts these handlers on FastAPI (POST /qp/solve).  They hold everything the route
does between the HTTP layer and the engine: the request checks, the submission into the
continuous-batching request loop (boxqp.serve.BoxQPServer), the wait for the request's own
completion while other requests keep running in the same batch, and the reply in the reference's
normalized record shape (02-software/backend/solve.py:49-63: engine name, a status in the
reference's vocabulary, null for non-finite numbers).  Errors the HTTP layer must turn into a
status code are raised as HttpError.

Refusals:
  * 413 for a request larger than the route's limits, or one that can never fit under the
    request loop's device-memory cap (the engine's admission error);
  * 400 / 422 for malformed arrays or options;
  * a solve the engine fails after admission (an allocation that failed on the device, a CUDA
    error) answers with status "engine_error" and the engine's message; the loop keeps serving.
"""
import asyncio
import io
import math
import os
import threading

import numpy as np

MAX_VARIABLES = int(os.environ.get('BOXQP_MAX_VARIABLES', '2000000'))
MAX_NONZEROS = int(os.environ.get('BOXQP_MAX_NONZEROS', '60000000'))
MEM_CAP_BYTES = int(float(os.environ.get('BOXQP_MEM_CAP_GB', '40')) * (1 << 30))
LATENCY_MS = float(os.environ.get('BOXQP_LATENCY_MS', '2.0'))
PRECISIONS = ('mixed', 'fp64', 'fp64_exact')


class HttpError(Exception):
    def __init__(self, status, detail):
        super().__init__(detail)
        self.status = status
        self.detail = detail


def json_safe(value):
    """Unknown or infinite values are null, never non-standard JSON NaN/Infinity."""
    if isinstance(value, float) and not math.isfinite(value):
        return None
    if isinstance(value, dict):
        return {k: json_safe(v) for k, v in value.items()}
    if isinstance(value, (list, tuple)):
        return [json_safe(v) for v in value]
    return value


_server = None
_server_lock = threading.Lock()


def get_server():
    global _server
    with _server_lock:
        if _server is None:
            from .serve import BoxQPServer
            _server = BoxQPServer(0, MEM_CAP_BYTES, LATENCY_MS)
        return _server


def set_server(server):
    """Installs a request loop (tests install their own)."""
    global _server
    with _server_lock:
        _server = server


def check_arrays(rowptr, col, val, c, lower, upper):
    n = c.shape[0]
    if n < 1 or n > MAX_VARIABLES:
        raise HttpError(413, f'n must be in [1, {MAX_VARIABLES}]')
    if col.shape[0] > MAX_NONZEROS or col.shape[0] != val.shape[0]:
        raise HttpError(413 if col.shape[0] > MAX_NONZEROS else 400, 'bad nonzero count')
    if rowptr.shape[0] != n + 1 or lower.shape[0] != n or upper.shape[0] != n:
        raise HttpError(400, 'rowptr must have n+1 entries and bounds n entries')
    if rowptr[0] != 0 or rowptr[-1] != col.shape[0] or np.any(np.diff(rowptr) < 0):
        raise HttpError(400, 'invalid CSR row pointers')
    if col.shape[0] and (col.min() < 0 or col.max() >= n):
        raise HttpError(400, 'column index out of range')
    if not np.all(np.isfinite(val)) or not np.all(np.isfinite(c)):
        raise HttpError(400, 'values and costs must be finite')
    if np.any(np.isnan(lower)) or np.any(np.isnan(upper)) or np.any(lower == np.inf) or np.any(upper == -np.inf):
        raise HttpError(400, 'invalid variable bound')


def check_options(tolerance, precision, time_limit):
    if not (tolerance > 0 and math.isfinite(tolerance) and time_limit > 0 and math.isfinite(time_limit)):
        raise HttpError(422, 'tolerance and time_limit must be positive and finite')
    if precision not in PRECISIONS:
        raise HttpError(422, 'precision must be mixed, fp64 or fp64_exact')


def _unsupported(exc):
    """Reply for a model the box engine does not take (a zero Hessian goes to the reference's CPU
    LP path, src/accelerated_qp.cpp:27-28)."""
    return {'engine': 'gb300', 'status': 'unsupported', 'message': str(exc)[:300], 'objective': None, 'primal': []}


async def solve_arrays(rowptr, col, val, c, lower, upper, tolerance=1e-6, precision='mixed', time_limit=20.0,
                       return_primal=True):
    """One box QP through the request loop; returns the reply record."""
    check_arrays(rowptr, col, val, c, lower, upper)
    check_options(tolerance, precision, time_limit)
    server = get_server()
    from ._native import EngineError
    try:
        fut = server.submit(rowptr, col, val, c, lower, upper, tolerance, precision, time_limit)
    except ValueError as exc:
        return json_safe({'engine': 'gb300', 'status': 'input_rejected', 'message': str(exc), 'objective': None,
                          'primal': []})
    except EngineError as exc:
        if exc.code == 4:  # BQP_ERR_ADMISSION: can never fit under the loop's device-memory cap
            raise HttpError(413, 'request exceeds the device-memory cap: ' + str(exc)[:200])
        if exc.code == 7:  # BQP_ERR_UNSUPPORTED: a zero Hessian (the reference's CPU LP path)
            return _unsupported(exc)
        raise
    try:
        r = await asyncio.wait_for(asyncio.wrap_future(fut), timeout=time_limit + 5.0)
    except asyncio.TimeoutError:
        return {'engine': 'gb300', 'status': 'time_limit', 'message': 'no result within the time limit',
                'objective': None, 'primal': []}
    except ValueError as exc:  # entries the admission pass on the device rejected
        return json_safe({'engine': 'gb300', 'status': 'input_rejected', 'message': str(exc), 'objective': None,
                          'primal': []})
    except EngineError as exc:
        if exc.code == 4:  # refused at admission: it can never fit under the loop's memory cap
            raise HttpError(413, 'request exceeds the device-memory cap: ' + str(exc)[:200])
        if exc.code == 7:  # a zero Hessian, found by the admission pass
            return _unsupported(exc)
        return {'engine': 'gb300', 'status': 'engine_error', 'message': str(exc)[:300], 'objective': None,
                'primal': []}
    except Exception as exc:
        return {'engine': 'gb300', 'status': 'engine_error', 'message': str(exc)[:300], 'objective': None,
                'primal': []}
    return json_safe({'engine': 'gb300', 'status': r.status, 'message': '', 'objective': r.objective,
                      'stationarity_residual': r.stationarity, 'primal_residual': r.primal_residual,
                      'iterations': r.iterations, 'polish_iterations': r.polish_iterations,
                      'seconds': r.latency, 'device_seconds': r.device_seconds,
                      'primal': r.x.tolist() if return_primal else [], 'columns': int(c.shape[0])})


async def solve_npz(body, tolerance=1e-6, precision='mixed', time_limit=20.0, return_primal=True):
    """The binary request form: an .npz body with rowptr, col, val, c, lower, upper."""
    check_options(tolerance, precision, time_limit)
    try:
        z = np.load(io.BytesIO(body), allow_pickle=False)
        arrays = [np.ascontiguousarray(z[k]) for k in ('rowptr', 'col', 'val', 'c', 'lower', 'upper')]
    except Exception:
        raise HttpError(400, 'body must be an .npz with rowptr, col, val, c, lower, upper')
    rowptr, col = arrays[0].astype(np.int32), arrays[1].astype(np.int32)
    val, c, lower, upper = (a.astype(np.float64) for a in arrays[2:])
    return await solve_arrays(rowptr, col, val, c, lower, upper, tolerance, precision, time_limit, return_primal)


def bounds(values, default):
    """JSON bounds: null is an infinite bound."""
    return np.array([default if v is None else v for v in values], dtype=np.float64)
