"""FastAPI box-QP route over the continuous-batching request loop.

Mounts on the reference's demo service (02-software/backend/app.py) or runs alone:
    uvicorn boxqp.service:app
Routes:
  POST /qp/solve   one box QP, as JSON (full symmetric CSR) or as an .npz body
                   (Content-Type: application/x-npz; arrays rowptr, col, val, c, lower, upper;
                   options as query parameters) -- the binary form avoids JSON for millions of
                   nonzeros.  The request waits for its own completion while other requests keep
                   running on the GPU in the same batch.
  GET  /qp/health  engine and device
  GET  /qp/load    queued / running / peak resident solves and resident bytes
Records follow the reference's normalized shape (02-software/backend/solve.py:49-63): the engine
name, a status in the reference's vocabulary, null for non-finite numbers.
"""
import asyncio
import io
import math
import os
import threading
from typing import List, Literal, Optional

import numpy as np
from fastapi import FastAPI, HTTPException, Request
from pydantic import BaseModel, Field

MAX_VARIABLES = int(os.environ.get('BOXQP_MAX_VARIABLES', '2000000'))
MAX_NONZEROS = int(os.environ.get('BOXQP_MAX_NONZEROS', '60000000'))
MEM_CAP_BYTES = int(float(os.environ.get('BOXQP_MEM_CAP_GB', '40')) * (1 << 30))
LATENCY_MS = float(os.environ.get('BOXQP_LATENCY_MS', '2.0'))


def json_safe(value):
    """Unknown or infinite values are null, never non-standard JSON NaN/Infinity."""
    if isinstance(value, float) and not math.isfinite(value):
        return None
    if isinstance(value, dict):
        return {k: json_safe(v) for k, v in value.items()}
    if isinstance(value, (list, tuple)):
        return [json_safe(v) for v in value]
    return value


class BoxQPRequest(BaseModel):
    rowptr: List[int] = Field(..., min_length=2)
    col: List[int]
    val: List[float]
    cost: List[float] = Field(..., min_length=1)
    lower: List[Optional[float]]
    upper: List[Optional[float]]
    tolerance: float = Field(1e-6, gt=0, allow_inf_nan=False)
    precision: Literal['mixed', 'fp64', 'fp64_exact'] = 'mixed'
    time_limit: float = Field(20.0, gt=0, allow_inf_nan=False)
    return_primal: bool = True


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
    """Installs a request loop (tests install a fake one)."""
    global _server
    with _server_lock:
        _server = server


def _check_arrays(rowptr, col, val, c, lower, upper):
    n = c.shape[0]
    if n < 1 or n > MAX_VARIABLES:
        raise HTTPException(413, f'n must be in [1, {MAX_VARIABLES}]')
    if col.shape[0] > MAX_NONZEROS or col.shape[0] != val.shape[0]:
        raise HTTPException(413 if col.shape[0] > MAX_NONZEROS else 400, 'bad nonzero count')
    if rowptr.shape[0] != n + 1 or lower.shape[0] != n or upper.shape[0] != n:
        raise HTTPException(400, 'rowptr must have n+1 entries and bounds n entries')
    if rowptr[0] != 0 or rowptr[-1] != col.shape[0] or np.any(np.diff(rowptr) < 0):
        raise HTTPException(400, 'invalid CSR row pointers')
    if col.shape[0] and (col.min() < 0 or col.max() >= n):
        raise HTTPException(400, 'column index out of range')
    if not np.all(np.isfinite(val)) or not np.all(np.isfinite(c)):
        raise HTTPException(400, 'values and costs must be finite')
    if np.any(np.isnan(lower)) or np.any(np.isnan(upper)) or np.any(lower == np.inf) or np.any(upper == -np.inf):
        raise HTTPException(400, 'invalid variable bound')


async def _solve(rowptr, col, val, c, lower, upper, tolerance, precision, time_limit, return_primal):
    _check_arrays(rowptr, col, val, c, lower, upper)
    server = get_server()
    try:
        fut = server.submit(rowptr, col, val, c, lower, upper, tolerance, precision, time_limit)
    except ValueError as exc:
        return json_safe({'engine': 'gb300', 'status': 'input_rejected', 'message': str(exc), 'objective': None,
                          'primal': []})
    try:
        r = await asyncio.wait_for(asyncio.wrap_future(fut), timeout=time_limit + 5.0)
    except asyncio.TimeoutError:
        return {'engine': 'gb300', 'status': 'time_limit', 'message': 'no result within the time limit',
                'objective': None, 'primal': []}
    except Exception as exc:
        return {'engine': 'gb300', 'status': 'engine_error', 'message': str(exc)[:300], 'objective': None,
                'primal': []}
    return json_safe({'engine': 'gb300', 'status': r.status, 'message': '', 'objective': r.objective,
                      'stationarity_residual': r.stationarity, 'primal_residual': r.primal_residual,
                      'iterations': r.iterations, 'polish_iterations': r.polish_iterations,
                      'seconds': r.latency, 'device_seconds': r.device_seconds,
                      'primal': r.x.tolist() if return_primal else [], 'columns': int(c.shape[0])})


def _bounds(values, default):
    return np.array([default if v is None else v for v in values], dtype=np.float64)


app = FastAPI(title='GB300 box-QP engine', version='1.0')


@app.get('/qp/health')
def health():
    from .api import cuda_device_name
    return {'ok': True, 'engine': 'gb300', 'device': cuda_device_name()}


@app.get('/qp/load')
def load():
    return get_server().load()


@app.post('/qp/solve')
async def solve(request: Request, tolerance: float = 1e-6, precision: str = 'mixed', time_limit: float = 20.0,
                return_primal: bool = True):
    if request.headers.get('content-type', '').startswith('application/x-npz'):
        if not (tolerance > 0 and math.isfinite(tolerance) and time_limit > 0 and math.isfinite(time_limit)):
            raise HTTPException(422, 'tolerance and time_limit must be positive and finite')
        if precision not in ('mixed', 'fp64', 'fp64_exact'):
            raise HTTPException(422, 'precision must be mixed, fp64 or fp64_exact')
        try:
            z = np.load(io.BytesIO(await request.body()), allow_pickle=False)
            arrays = [np.ascontiguousarray(z[k]) for k in ('rowptr', 'col', 'val', 'c', 'lower', 'upper')]
        except Exception:
            raise HTTPException(400, 'body must be an .npz with rowptr, col, val, c, lower, upper')
        rowptr, col = arrays[0].astype(np.int32), arrays[1].astype(np.int32)
        val, c, lower, upper = (a.astype(np.float64) for a in arrays[2:])
        return await _solve(rowptr, col, val, c, lower, upper, tolerance, precision, time_limit, return_primal)
    try:
        body = BoxQPRequest.model_validate(await request.json())
    except Exception as exc:
        raise HTTPException(422, 'invalid request: ' + str(exc)[:200])
    return await _solve(np.asarray(body.rowptr, np.int32), np.asarray(body.col, np.int32),
                        np.asarray(body.val, np.float64), np.asarray(body.cost, np.float64),
                        _bounds(body.lower, -np.inf), _bounds(body.upper, np.inf), body.tolerance, body.precision,
                        body.time_limit, body.return_primal)
