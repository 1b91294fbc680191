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
The request handling itself (checks, submission, reply records in the reference's normalized
shape, 02-software/backend/solve.py:49-63) lives in boxqp.service_core, which needs no web
framework; this module adds the HTTP layer.
"""
from typing import List, Literal, Optional

import numpy as np
from fastapi import FastAPI, HTTPException, Request
from pydantic import BaseModel, Field

from . import service_core as core
from .service_core import get_server, json_safe, set_server  # noqa: F401  (re-exported)


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
    try:
        if request.headers.get('content-type', '').startswith('application/x-npz'):
            return await core.solve_npz(await request.body(), tolerance, precision, time_limit, return_primal)
        try:
            body = BoxQPRequest.model_validate(await request.json())
        except Exception as exc:
            raise core.HttpError(422, 'invalid request: ' + str(exc)[:200])
        return await core.solve_arrays(np.asarray(body.rowptr, np.int32), np.asarray(body.col, np.int32),
                                       np.asarray(body.val, np.float64), np.asarray(body.cost, np.float64),
                                       core.bounds(body.lower, -np.inf), core.bounds(body.upper, np.inf),
                                       body.tolerance, body.precision, body.time_limit, body.return_primal)
    except core.HttpError as exc:
        raise HTTPException(exc.status, exc.detail)
