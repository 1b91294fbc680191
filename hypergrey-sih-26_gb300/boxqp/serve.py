"""Continuous-batching request loop for box-QP solves on one GPU.

The reference service admits one compute request at a time and answers 429 otherwise
(02-software/backend/limits.py:10-68).  Here every request is submitted to one engine context
at once (its arrays are copied, so the caller may reuse them): the engine admits queued solves
into the running batch as device memory frees up under the context's cap, iterates all resident
solves in the same launches, and retires each one when its own tolerance is met.  With a latency
target, each device launch runs only a few milliseconds, so solves that arrive while others are
running join the batch at the next launch boundary.  A collector thread turns completions
(bqp_wait_any) into resolved futures.
"""
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .api import Engine, options_struct


@dataclass
class SolveResult:
    status: str
    x: np.ndarray
    objective: float
    stationarity: float
    primal_residual: float
    iterations: int
    polish_iterations: int
    device_seconds: float
    submitted: float     # host clock (perf_counter) at submission
    finished: float      # host clock when the collector received the completion

    @property
    def latency(self):
        return self.finished - self.submitted


class BoxQPServer:
    """Request loop: submit() returns a Future of SolveResult; solves overlap on the device."""

    def __init__(self, device=0, mem_cap_bytes=40 << 30, latency_ms=2.0):
        self.engine = Engine(device, mem_cap_bytes)
        self.engine.set_latency_target(latency_ms)
        self._pending = {}
        self._lock = threading.Lock()
        self._stop = False
        self._collector = threading.Thread(target=self._collect, name='boxqp-collector', daemon=True)
        self._collector.start()

    def submit(self, rowptr, col, val, c, lower, upper, tolerance=1e-6, precision='mixed', time_limit=30.0,
               iteration_limit=200000):
        o = options_struct(tolerance, time_limit, iteration_limit, precision)
        fut = Future()
        n = int(np.asarray(c).shape[0])
        with self._lock:  # registered before the collector can see the completion
            t0 = time.perf_counter()
            ident = self.engine.submit(rowptr, col, val, c, lower, upper, o)
            self._pending[ident] = (fut, n, t0)
        return fut

    def _collect(self):
        while not self._stop:
            ident = self.engine.wait_any(0.05)
            if ident is None:
                continue
            t1 = time.perf_counter()
            with self._lock:
                entry = self._pending.pop(ident, None)
            if entry is None:
                continue
            fut, n, t0 = entry
            try:
                x, st = self.engine.fetch(ident, n)
                self.engine.release(ident)
                fut.set_result(SolveResult(N.STATUS_NAMES.get(st.status, str(st.status)), x, st.objective,
                                           st.stationarity_residual, st.primal_residual, int(st.iterations),
                                           int(st.polish_iterations), st.device_seconds, t0, t1))
            except Exception as exc:  # the engine reported an error for this solve
                try:
                    self.engine.release(ident)
                except Exception:
                    pass
                fut.set_exception(exc)

    def load(self):
        d = self.engine.load()
        with self._lock:
            d['waiting_futures'] = len(self._pending)
        return d

    def close(self):
        self._stop = True
        self._collector.join(timeout=5)
        self.engine.close()
