"""Host-side mirror of the reference's box-QP API over the GB300 engine.

Names, argument meaning and error behaviour follow the reference's C++ interface
(02-software/solver/include/qp.hpp:5-34, include/accelerated_qp.hpp:9-17):

  QuadraticProblem / QpOptions / QpResult     the reference's records
  solve_accelerated_box(q, opt, cuda=True)    src/accelerated_qp.cpp:13-61, on the GPU engine
  check_convex_hessian(q)                     src/qp_admm.cpp:30-62 (host, in libboxqp)
  make_cuda_box(...) -> BoxIteration          src/cuda_box.cu:34-37 plugin contract
  cuda_device_name()                          src/cuda_box.cu:38

std::invalid_argument becomes ValueError; CUDA failures become EngineError.  There is no CPU
path: cuda=False raises, as the product has no CPU fallback.
"""
import math
import threading
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _native as N
from ._native import EngineError, Options, PlantedSpec, Stats, lib, ptr


# ------------------------------------------------------------------------------------------
# records
# ------------------------------------------------------------------------------------------
@dataclass
class QuadraticProblem:
    """min sense*(1/2 x'Hx + c'x + offset), lower <= x <= upper.

    `hessian_row/col/val` are the reference's lower-triangle triplets (row >= col); each
    off-diagonal entry stands for both (i, j) and (j, i) (include/qp.hpp:7-9).
    """
    cost: np.ndarray
    lower: np.ndarray
    upper: np.ndarray
    hessian_row: np.ndarray
    hessian_col: np.ndarray
    hessian_val: np.ndarray
    offset: float = 0.0
    maximize: bool = False
    integer: Optional[np.ndarray] = None
    rows: int = 0  # linear constraint rows; the box engine accepts none

    @property
    def n(self):
        return int(np.asarray(self.cost).shape[0])


@dataclass
class QpOptions:
    """Defaults of QpOptions (include/qp.hpp:24-29) plus the engine's precision choice."""
    time_limit: float = 30.0
    tolerance: float = 1e-7
    iteration_limit: int = 200000
    threads: int = 1
    scaling: bool = True
    precision: str = 'fp64'
    check_interval: int = 0  # 0: engine default (25, the reference's cadence, for the FP64 engines)


@dataclass
class QpResult:
    status: str = ''
    primal: np.ndarray = field(default_factory=lambda: np.zeros(0))
    row_dual: np.ndarray = field(default_factory=lambda: np.zeros(0))
    objective: float = math.nan
    primal_residual: float = math.inf
    stationarity_residual: float = math.inf
    complementarity_residual: float = math.inf
    iterations: int = 0
    dual_bound: float = -math.inf
    relative_gap: float = math.inf
    optimality_verified: bool = False
    algorithm: str = ''
    engine: dict = field(default_factory=dict)


# ------------------------------------------------------------------------------------------
# helpers
# ------------------------------------------------------------------------------------------
def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def options_struct(tolerance=1e-7, time_limit=30.0, iteration_limit=200000, precision='fp64',
                   check_interval=0, diagonal_gate=-1, offset=0.0, kernel_variant=-1, polish_switch=None,
                   scaling=0, lipschitz='gershgorin'):
    """bqp_options from keywords; lipschitz: 'gershgorin' (the reference's bound) or 'power'
    (device power-iteration estimate)."""
    o = Options()
    lib().bqp_options_default(o)
    o.tolerance = float(tolerance)
    o.time_limit = float(time_limit)
    o.iteration_limit = int(iteration_limit)
    o.precision = N.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    o.check_interval = int(check_interval)
    o.diagonal_gate = int(diagonal_gate)
    o.offset = float(offset)
    o.kernel_variant = int(kernel_variant)
    if polish_switch is not None:
        o.polish_switch = float(polish_switch)
    o.scaling = int(scaling)
    o.lipschitz = {'gershgorin': 0, 'power': 1}[lipschitz] if isinstance(lipschitz, str) else int(lipschitz)
    return o


def csr_from_lower(n, hrow, hcol, hval, sign=1.0):
    """Full symmetric CSR of lower-triangle triplets, built as CsrMatrix(n, rows) builds it."""
    hrow, hcol, hval = _i64(hrow), _i64(hcol), _f64(hval)
    nh = int(hrow.shape[0])
    rowptr = np.zeros(n + 1, dtype=np.int32)
    col = np.zeros(max(2 * nh, 1), dtype=np.int32)
    val = np.zeros(max(2 * nh, 1), dtype=np.float64)
    nnz = np.zeros(1, dtype=np.int64)
    rc = lib().bqp_csr_from_lower(n, nh, ptr(hrow, N.c_int64), ptr(hcol, N.c_int64), ptr(hval, N.c_double),
                                  float(sign), ptr(rowptr, N.c_int32), ptr(col, N.c_int32),
                                  ptr(val, N.c_double), ptr(nnz, N.c_int64))
    if rc != N.BQP_OK:
        raise ValueError('Invalid Hessian')
    k = int(nnz[0])
    return rowptr, col[:k].copy(), val[:k].copy()


def gershgorin(rowptr, val):
    rowptr, val = _i32(rowptr), _f64(val)
    return float(lib().bqp_gershgorin(rowptr.shape[0] - 1, ptr(rowptr, N.c_int32), ptr(val, N.c_double)))


def check_convex_hessian(q: QuadraticProblem) -> bool:
    """check_convex_hessian (src/qp_admm.cpp:30-62); ValueError on an invalid Hessian."""
    hrow, hcol, hval = _i64(q.hessian_row), _i64(q.hessian_col), _f64(q.hessian_val)
    rc = lib().bqp_check_convex(q.n, hrow.shape[0], ptr(hrow, N.c_int64), ptr(hcol, N.c_int64),
                                ptr(hval, N.c_double), 1 if q.maximize else 0)
    if rc < 0:
        raise ValueError('Invalid Hessian')
    return rc == 1


class pinned:
    """Context manager that page-locks numpy arrays (bqp_host_register) for as long as it is
    entered: submissions from them upload by asynchronous DMA with no host staging copy.  The
    arrays must be C-contiguous and stay alive while pinned."""

    def __init__(self, *arrays):
        self.arrays = [a for a in arrays if a is not None and a.nbytes > 0]
        self._done = []

    def __enter__(self):
        for a in self.arrays:
            if not a.flags['C_CONTIGUOUS']:
                raise ValueError('pinned arrays must be C-contiguous')
            rc = lib().bqp_host_register(a.ctypes.data, a.nbytes)
            if rc != N.BQP_OK:
                self.__exit__(None, None, None)
                msg = lib().bqp_last_error(None)
                raise EngineError(rc, msg.decode() if msg else 'host register failed')
            self._done.append(a)
        return self

    def __exit__(self, *exc):
        for a in self._done:
            lib().bqp_host_unregister(a.ctypes.data)
        self._done = []
        return False


def cuda_device_name(device=0):
    buf = N.ctypes.create_string_buffer(256)
    lib().bqp_device_name(device, buf, 256)
    return buf.value.decode()


# ------------------------------------------------------------------------------------------
# engine context
# ------------------------------------------------------------------------------------------
class Engine:
    """One engine context on one GPU: resident solves, continuous batching, admission cap."""

    def __init__(self, device=0, mem_cap_bytes=0):
        L = lib()
        self._ctx = L.bqp_create(int(device), int(mem_cap_bytes))
        if not self._ctx:
            msg = L.bqp_last_error(None)
            raise EngineError(2, msg.decode() if msg else 'engine creation failed')
        self.device = device
        self._borrowed = {}  # id -> input arrays of a bqp_submit_borrowed solve, kept until release

    def close(self):
        if getattr(self, '_ctx', None):
            lib().bqp_destroy(self._ctx)
            self._ctx = None
            self._borrowed = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != N.BQP_OK:
            msg = lib().bqp_last_error(self._ctx)
            text = msg.decode() if msg else ''
            if rc == 1:
                raise ValueError(text)
            raise EngineError(rc, text)

    def submit(self, rowptr, col, val, c, lower, upper, options: Options, copy=True):
        """Queues one solve and returns its id.  copy=False (bqp_submit_borrowed) skips the host
        copy of the inputs: the engine keeps references to the (contiguous) arrays until release,
        and the caller must not modify them before the solve has finished."""
        rowptr, col, val = _i32(rowptr), _i32(col), _f64(val)
        c, lower, upper = _f64(c), _f64(lower), _f64(upper)
        options = _tuned(options, c.shape[0], col.shape[0])
        ident = N.c_uint64(0)
        fn = lib().bqp_submit if copy else lib().bqp_submit_borrowed
        rc = fn(self._ctx, c.shape[0], col.shape[0], ptr(rowptr, N.c_int32), ptr(col, N.c_int32),
                ptr(val, N.c_double), ptr(c, N.c_double), ptr(lower, N.c_double),
                ptr(upper, N.c_double), options, N.ctypes.byref(ident))
        self._check(rc)
        if not copy:
            self._borrowed[ident.value] = (rowptr, col, val, c, lower, upper)
        return ident.value

    def poll(self, ident):
        st = N.c_int32(0)
        self._check(lib().bqp_poll(self._ctx, ident, N.ctypes.byref(st)))
        return st.value

    def wait(self, ident, timeout=-1.0):
        rc = lib().bqp_wait(self._ctx, ident, float(timeout))
        if rc == 6:
            return False
        self._check(rc)
        return True

    def wait_any(self, timeout=-1.0):
        """Id of the next finished asynchronous solve, or None on timeout."""
        ident = N.c_uint64(0)
        rc = lib().bqp_wait_any(self._ctx, float(timeout), N.ctypes.byref(ident))
        if rc == 6:
            return None
        self._check(rc)
        return ident.value

    def fetch(self, ident, n, out=None):
        """(x, Stats) of a finished solve; `out` (float64, contiguous, n entries) receives x."""
        if out is None:
            x = np.empty(n, dtype=np.float64)
        else:
            x = out
            if x.dtype != np.float64 or not x.flags['C_CONTIGUOUS'] or x.shape != (n,):
                raise ValueError('out must be a contiguous float64 array of n entries')
        st = Stats()
        self._check(lib().bqp_fetch(self._ctx, ident, ptr(x, N.c_double), st))
        return x, st

    def release(self, ident):
        self._check(lib().bqp_release(self._ctx, ident))
        self._borrowed.pop(ident, None)

    def resolve(self, idents):
        ids = np.ascontiguousarray(np.asarray(list(idents), dtype=np.uint64))
        self._check(lib().bqp_resolve(self._ctx, ptr(ids, N.c_uint64), ids.shape[0]))

    def set_latency_target(self, ms):
        self._check(lib().bqp_set_latency_target(self._ctx, float(ms)))

    def inject_admission_oom(self, count=1):
        """Host-side fault injection: the next `count` admissions fail as out of memory."""
        self._check(lib().bqp_inject_admission_oom(self._ctx, int(count)))

    def load(self):
        q, r, p, b = (N.c_int64(0) for _ in range(4))
        self._check(lib().bqp_load(self._ctx, N.ctypes.byref(q), N.ctypes.byref(r), N.ctypes.byref(p),
                                   N.ctypes.byref(b)))
        return {'queued': q.value, 'running': r.value, 'peak_resident': p.value, 'resident_bytes': b.value}

    def timer(self, reset=False):
        """(device ms, engine kernels, graph launches) since the last reset (CUDA events)."""
        ms, k, g = N.c_double(0), N.c_int64(0), N.c_int64(0)
        self._check(lib().bqp_timer(self._ctx, 1 if reset else 0, N.ctypes.byref(ms), N.ctypes.byref(k),
                                    N.ctypes.byref(g)))
        return ms.value, k.value, g.value

    def profile_step(self, ident, launches=50):
        """(ms per step-kernel launch, algorithmic bytes per launch) on a finished resident solve."""
        ms, b = N.c_double(0), N.c_double(0)
        self._check(lib().bqp_profile_step(self._ctx, ident, int(launches), N.ctypes.byref(ms), N.ctypes.byref(b)))
        return ms.value, b.value

    def profile_cg(self, ident, iterations=10):
        """Times the polish CG of a finished mixed solve (bqp_profile_cg); returns
        (ms per product launch, ms per vector launch, bytes per product launch, bytes per vector
        launch).  The solve's answer is scrambled afterwards: re-run it with resolve()."""
        vals = [N.c_double(0) for _ in range(4)]
        self._check(lib().bqp_profile_cg(self._ctx, ident, int(iterations), *[N.ctypes.byref(v) for v in vals]))
        return tuple(v.value for v in vals)

    def solve(self, rowptr, col, val, c, lower, upper, options: Options):
        """Synchronous solve through bqp_solve_sync; returns (x, Stats)."""
        rowptr, col, val = _i32(rowptr), _i32(col), _f64(val)
        c, lower, upper = _f64(c), _f64(lower), _f64(upper)
        options = _tuned(options, c.shape[0], col.shape[0])
        x = np.empty(c.shape[0], dtype=np.float64)
        st = Stats()
        rc = lib().bqp_solve_sync(self._ctx, c.shape[0], col.shape[0], ptr(rowptr, N.c_int32), ptr(col, N.c_int32),
                                  ptr(val, N.c_double), ptr(c, N.c_double), ptr(lower, N.c_double),
                                  ptr(upper, N.c_double), options, ptr(x, N.c_double), st)
        self._check(rc)
        return x, st


_PRECISION_NAMES = {v: k for k, v in N.PRECISIONS.items()}


def _tuned(options, n, nnz):
    """Fills kernel_variant from the autotuning table when the caller left it automatic."""
    if options.kernel_variant >= 0:
        return options
    from .autotune import tuned_variant
    v = tuned_variant(_PRECISION_NAMES.get(options.precision, 'fp64'), n, nnz)
    if v < 0:
        return options
    o = Options()
    N.ctypes.pointer(o)[0] = options
    o.kernel_variant = v
    return o


_default = {}
_default_lock = threading.Lock()


def default_engine(device=0):
    with _default_lock:
        eng = _default.get(device)
        if eng is None:
            eng = Engine(device)
            _default[device] = eng
        return eng


# ------------------------------------------------------------------------------------------
# the reference's engine API
# ------------------------------------------------------------------------------------------
def _validate(q: QuadraticProblem, opt: QpOptions):
    n = q.n
    cost, lower, upper = _f64(q.cost), _f64(q.lower), _f64(q.upper)
    # validate_linear_problem (src/mps.cpp:47-60)
    if n == 0 or lower.shape[0] != n or upper.shape[0] != n or not math.isfinite(q.offset):
        raise ValueError('Invalid linear problem dimensions or offset')
    if (not np.all(np.isfinite(cost)) or np.any(np.isnan(lower)) or np.any(np.isnan(upper))
            or np.any(lower == np.inf) or np.any(upper == -np.inf)):
        raise ValueError('Invalid variable coefficient or bound')
    if q.rows:
        raise ValueError('Accelerated box QP requires box constraints only')
    if q.integer is not None and np.any(np.asarray(q.integer)):
        raise ValueError('Accelerated box QP requires continuous variables')
    if (not (opt.tolerance > 0) or not math.isfinite(opt.tolerance) or opt.time_limit < 0
            or not math.isfinite(opt.time_limit) or opt.threads < 1):
        raise ValueError('Invalid box QP options')
    return cost, lower, upper


def solve_accelerated_box(q: QuadraticProblem, opt: QpOptions = None, cuda: bool = True,
                          engine: Engine = None) -> QpResult:
    """solve_accelerated_box (src/accelerated_qp.cpp:13-61) on the GB300 engine."""
    opt = opt or QpOptions()
    cost, lower, upper = _validate(q, opt)
    if not cuda:
        raise ValueError('this engine runs on the GPU only; the CPU path is the reference build')
    r = QpResult(algorithm='cuda_fista_box' if opt.precision == 'fp64' else f'cuda_fista_box_{opt.precision}')
    if not check_convex_hessian(q):
        r.status = 'unsupported_curvature'
        return r
    sign = -1.0 if q.maximize else 1.0
    rowptr, col, val = csr_from_lower(q.n, q.hessian_row, q.hessian_col, q.hessian_val, sign)
    if gershgorin(rowptr, val) == 0:
        raise ValueError('Zero-Hessian models use the CPU LP path')
    if np.any(lower > upper):
        r.status = 'infeasible_bounds'
        return r
    # the reference's positive-diagonal gate: no off-diagonal triplet with a non-zero value
    hrow, hcol, hval = _i64(q.hessian_row), _i64(q.hessian_col), _f64(q.hessian_val)
    off = hrow != hcol
    gate = 0
    if not np.any(hval[off] != 0):
        diag = np.zeros(q.n)
        np.add.at(diag, hrow[~off], sign * hval[~off])
        gate = 1 if np.all(diag > 0) else 0
    o = options_struct(opt.tolerance, opt.time_limit, opt.iteration_limit, opt.precision, opt.check_interval,
                       gate, sign * q.offset)
    eng = engine or default_engine()
    x, st = eng.solve(rowptr, col, val, sign * cost, lower, upper, o)
    r.status = N.STATUS_NAMES.get(st.status, str(st.status))
    r.primal = x
    r.objective = sign * st.objective
    r.primal_residual = st.primal_residual
    r.stationarity_residual = st.stationarity_residual
    r.complementarity_residual = st.complementarity_residual
    r.iterations = int(st.iterations)
    r.dual_bound = st.dual_bound
    r.relative_gap = st.relative_gap
    r.optimality_verified = bool(st.verified)
    r.engine = st.as_dict()
    return r


class BoxIteration:
    """The reference's BoxIteration plugin (include/accelerated_qp.hpp:9-13) on the GPU."""

    def __init__(self, handle, n):
        self._h = handle
        self.n = n

    def step(self, momentum):
        rc = lib().bqp_box_step(self._h, float(momentum))
        if rc != N.BQP_OK:
            raise EngineError(rc, (lib().bqp_box_last_error(self._h) or b'').decode())

    def primal(self):
        x = np.empty(self.n, dtype=np.float64)
        rc = lib().bqp_box_primal(self._h, ptr(x, N.c_double))
        if rc != N.BQP_OK:
            raise EngineError(rc, (lib().bqp_box_last_error(self._h) or b'').decode())
        return x

    def close(self):
        if self._h:
            lib().bqp_box_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_cuda_box(rowptr, col, val, cost, lower, upper, lipschitz, device=0) -> BoxIteration:
    """make_cuda_box (src/cuda_box.cu:34-37): uploads once, returns the resident iteration."""
    rowptr, col, val = _i32(rowptr), _i32(col), _f64(val)
    cost, lower, upper = _f64(cost), _f64(lower), _f64(upper)
    h = lib().bqp_box_create(device, cost.shape[0], col.shape[0], ptr(rowptr, N.c_int32), ptr(col, N.c_int32),
                             ptr(val, N.c_double), ptr(cost, N.c_double), ptr(lower, N.c_double),
                             ptr(upper, N.c_double), float(lipschitz))
    if not h:
        msg = (lib().bqp_box_last_error(None) or b'').decode()
        raise EngineError(3 if 'No CUDA device' in msg else 2, msg)
    return BoxIteration(h, cost.shape[0])


# ------------------------------------------------------------------------------------------
# planted synthetic workloads
# ------------------------------------------------------------------------------------------
PRESETS = {'graph10k': 0, 'graph1m': 1, 'grid': 2, 'batch': 3, 'serve': 4, 'tridiagonal': 5}


def planted_spec(preset, seed=1, index=0, n=0):
    spec = PlantedSpec()
    p = PRESETS[preset] if isinstance(preset, str) else int(preset)
    if lib().bqp_planted_preset(p, int(seed), int(index), int(n), spec) != N.BQP_OK:
        raise ValueError(f'bad preset {preset!r}')
    return spec


def planted(preset=None, seed=1, index=0, n=0, spec=None, lower_triplets=False):
    """Generates one planted instance; returns a dict of numpy arrays and scalars."""
    L = lib()
    if spec is None:
        spec = planted_spec(preset, seed, index, n)
    h = L.bqp_planted_create(spec)
    if not h:
        raise ValueError('planted generation failed')
    try:
        nn, nnz, nl = N.c_int64(0), N.c_int64(0), N.c_int64(0)
        fstar = N.c_double(0)
        L.bqp_planted_info(h, N.ctypes.byref(nn), N.ctypes.byref(nnz),
                           N.ctypes.byref(nl) if lower_triplets else None, N.ctypes.byref(fstar))
        n_, z_ = nn.value, nnz.value
        out = {'n': n_, 'nnz': z_, 'fstar': fstar.value,
               'rowptr': np.empty(n_ + 1, np.int32), 'col': np.empty(z_, np.int32), 'val': np.empty(z_),
               'c': np.empty(n_), 'lower': np.empty(n_), 'upper': np.empty(n_), 'xstar': np.empty(n_),
               'z': np.empty(n_)}
        L.bqp_planted_copy(h, ptr(out['rowptr'], N.c_int32), ptr(out['col'], N.c_int32),
                           ptr(out['val'], N.c_double), ptr(out['c'], N.c_double), ptr(out['lower'], N.c_double),
                           ptr(out['upper'], N.c_double), ptr(out['xstar'], N.c_double), ptr(out['z'], N.c_double))
        if lower_triplets:
            k = nl.value
            hr, hc, hv = np.empty(k, np.int64), np.empty(k, np.int64), np.empty(k)
            L.bqp_planted_copy_lower(h, ptr(hr, N.c_int64), ptr(hc, N.c_int64), ptr(hv, N.c_double))
            out['hrow'], out['hcol'], out['hval'] = hr, hc, hv
        return out
    finally:
        L.bqp_planted_free(h)


def problem_from_planted(inst) -> QuadraticProblem:
    """The reference's QuadraticProblem form (lower triplets) of a planted instance."""
    return QuadraticProblem(cost=inst['c'], lower=inst['lower'], upper=inst['upper'],
                            hessian_row=inst['hrow'], hessian_col=inst['hcol'], hessian_val=inst['hval'])


def splitmix64(state):
    s = N.c_uint64(state)
    out = lib().bqp_splitmix64(N.ctypes.byref(s))
    return out, s.value
