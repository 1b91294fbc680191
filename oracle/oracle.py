"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Libraries:
  oracle/_build/liboracle.so     the plain-C restatement in oracle/boxqp_oracle.c (always
                                 buildable: gcc + OpenMP on any host), linked with the synthetic
                                 instance generator (hypergrey-sih-26_gb300/csrc/planted.cpp, the
                                 one generator the engine and the oracle share), so a process can
                                 make the workloads without loading the engine library
  oracle/_ref/libsovereign_ref.so  the reference's own solver sources compiled by
                                 oracle/ref.mk plus oracle/ref_shim.cpp, from the copy that
                                 `make -f oracle/ref.mk stage` puts in oracle/_ref/src where the
                                 reference checkout exists (the copy travels with the working tree)
  oracle/_build/libref_cuda.so   oracle/ref_cuda_harness.c: the reference's CUDA plugin kernels
                                 (oracle/_ref/cuda_box_sm103a.cubin, built by oracle/ref.mk from
                                 the reference's cuda_box.cu) under the reference's host loop
Only the tests, the smoke check and the benchmark's CPU-baseline leg and reference arm use this
module; the engine never does.
"""
import ctypes
import subprocess
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_uint64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SRC = HERE / 'boxqp_oracle.c'
PLANTED_SRC = HERE.parent / 'hypergrey-sih-26_gb300' / 'csrc' / 'planted.cpp'
BOXQP_H = HERE.parent / 'include' / 'boxqp.h'
ORACLE_LIB = HERE / '_build' / 'liboracle.so'
REF_MK = HERE / 'ref.mk'
REF_QPLIB = HERE / '_ref' / 'qplib'
REF_LIB = HERE / '_ref' / 'libsovereign_ref.so'
REF_CUBIN = HERE / '_ref' / 'cuda_box_sm103a.cubin'
REF_CUDA_SRC = HERE / 'ref_cuda_harness.c'
REF_CUDA_LIB = HERE / '_build' / 'libref_cuda.so'

STATUS = {0: 'optimal', 1: 'iteration_limit', 2: 'time_limit', 3: 'numerical_error',
          4: 'unsupported_curvature', 5: 'infeasible_bounds', 6: 'zero_hessian'}


class OrcStats(ctypes.Structure):
    _fields_ = [('objective', c_double), ('primal_residual', c_double), ('stationarity_residual', c_double),
                ('complementarity_residual', c_double), ('dual_bound', c_double), ('relative_gap', c_double),
                ('verified', c_double), ('iterations', c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_I32P, _I64P, _F64P = POINTER(c_int32), POINTER(c_int64), POINTER(c_double)


class PlantedSpec(ctypes.Structure):
    """bqp_planted_spec of include/boxqp.h (the generator linked into liboracle.so)."""
    _fields_ = [('family', c_int32), ('edges_per_vertex', c_int32), ('n', c_int64), ('grid_side', c_int32),
                ('bounds_mode', c_int32), ('seed', c_uint64), ('lower', c_double), ('upper', c_double),
                ('frac_lower', c_double), ('frac_upper', c_double), ('interior_lo', c_double),
                ('interior_hi', c_double), ('diag_lo', c_double), ('diag_hi', c_double),
                ('weight_lo', c_double), ('weight_hi', c_double), ('shift', c_double), ('dual_lo', c_double),
                ('dual_hi', c_double)]


PRESETS = {'graph10k': 0, 'graph1m': 1, 'grid': 2, 'batch': 3, 'serve': 4, 'tridiagonal': 5}


def build_oracle(force=False):
    """Compiles the C restatement (no FMA contraction, OpenMP) and the instance generator."""
    srcs = [ORACLE_SRC, PLANTED_SRC, BOXQP_H]
    if force or not ORACLE_LIB.exists() or any(p.stat().st_mtime > ORACLE_LIB.stat().st_mtime for p in srcs):
        out = ORACLE_LIB.parent
        out.mkdir(exist_ok=True)
        c_obj, cpp_obj = out / 'boxqp_oracle.o', out / 'planted.o'
        subprocess.run(['gcc', '-O2', '-std=gnu11', '-fopenmp', '-fPIC', '-ffp-contract=off', '-c', str(ORACLE_SRC),
                        '-o', str(c_obj)], check=True, capture_output=True)
        subprocess.run(['g++', '-O3', '-std=c++17', '-fPIC', '-ffp-contract=off', '-I', str(BOXQP_H.parent), '-c',
                        str(PLANTED_SRC), '-o', str(cpp_obj)], check=True, capture_output=True)
        tmp = ORACLE_LIB.with_suffix('.tmp.so')
        subprocess.run(['g++', '-shared', '-fopenmp', str(c_obj), str(cpp_obj), '-o', str(tmp), '-lm'], check=True,
                       capture_output=True)
        tmp.replace(ORACLE_LIB)
    return ORACLE_LIB


def _make(*targets):
    """Runs oracle/ref.mk from the repository root; returns the finished process."""
    return subprocess.run(['make', '-s', '-j8', '-f', str(REF_MK), *targets], cwd=str(HERE.parent),
                          capture_output=True, text=True)


def stage_reference():
    """Copies the reference files oracle/ref.mk compiles into oracle/_ref/src (where the
    reference checkout exists; BOXQP_REFERENCE_DIR overrides its location).  True when a staged
    copy is present afterwards."""
    _make('stage')
    return (HERE / '_ref' / 'src' / 'src' / 'accelerated_qp.cpp').exists()


def build_ref_cuda(force=False):
    """Compiles the driver-API harness for the reference's CUDA kernels (with the oracle's checker);
    True on success (needs the CUDA headers and a libcuda to link against)."""
    srcs = [REF_CUDA_SRC, ORACLE_SRC]
    if not force and REF_CUDA_LIB.exists() and all(p.stat().st_mtime <= REF_CUDA_LIB.stat().st_mtime for p in srcs):
        return True
    REF_CUDA_LIB.parent.mkdir(exist_ok=True)
    tmp = REF_CUDA_LIB.with_suffix('.tmp.so')
    cmd = ['gcc', '-O2', '-std=gnu11', '-fopenmp', '-fPIC', '-shared', '-ffp-contract=off', '-I/usr/local/cuda/include',
           *[str(p) for p in srcs], '-o', str(tmp), '-L/usr/local/cuda/lib64/stubs', '-L/usr/local/cuda/lib64', '-lcuda',
           '-lm']
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        return False
    tmp.replace(REF_CUDA_LIB)
    return True


def build_ref_cubin():
    """Compiles the reference's cuda_box.cu for sm_103a into oracle/_ref (from the staged copy);
    True when the module is present afterwards."""
    if stage_reference():
        _make('cuda_cubin')
    return REF_CUBIN.exists()


def ref_cuda_solve(rowptr, col, val, hrow, hcol, hval, cost, lower, upper, tol=1e-6, iteration_limit=200000,
                   time_limit=120.0):
    """The reference's CUDA plugin (its own kernels) under its host loop; returns
    (status name, stats dict, x, (solve seconds, loop seconds))."""
    L = ctypes.CDLL(str(REF_CUDA_LIB))
    L.ref_cuda_solve.restype = c_int
    L.ref_cuda_solve.argtypes = [c_char_p, c_int64, _I32P, _I32P, _F64P, c_int64, _I64P, _I64P, _F64P, _F64P, _F64P,
                                 _F64P, c_double, c_int64, c_double, _F64P, POINTER(OrcStats), POINTER(c_int), _F64P,
                                 c_char_p, c_int]
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    hrow, hcol, hval, cost, lower, upper = _arrays(hrow, hcol, hval, cost, lower, upper)
    n = cost.shape[0]
    x = np.zeros(n)
    st = OrcStats()
    status = c_int(-1)
    secs = np.zeros(2)
    err = ctypes.create_string_buffer(512)
    rc = L.ref_cuda_solve(str(REF_CUBIN).encode(), n, _p(rowptr, c_int32), _p(col, c_int32), _p(val, c_double),
                          hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double), _p(cost, c_double),
                          _p(lower, c_double), _p(upper, c_double), tol, iteration_limit, time_limit, _p(x, c_double),
                          ctypes.byref(st), ctypes.byref(status), _p(secs, c_double), err, 512)
    if rc != 0:
        raise RuntimeError('reference CUDA plugin: ' + err.value.decode(errors='replace'))
    return STATUS.get(status.value, str(status.value)), st.as_dict(), x, (float(secs[0]), float(secs[1]))


def build_reference():
    """Builds oracle/_ref/libsovereign_ref.so from the staged reference sources; True on success."""
    if not stage_reference():
        return REF_LIB.exists()
    proc = _make('all')
    return proc.returncode == 0 and REF_LIB.exists()


def build_level_a():
    """Links the reference's own CLI and scale harness with the GB300 plugin (Level A) and with the
    engine route (the *_engine binaries); returns oracle/_ref, or None without a staged copy of the
    reference sources."""
    if not stage_reference():
        return None
    proc = _make('level_a')
    if proc.returncode != 0:
        raise RuntimeError(proc.stdout + proc.stderr)
    return HERE / '_ref'


_orc = None
_ref = None


def orc():
    global _orc
    if _orc is None:
        build_oracle()
        L = ctypes.CDLL(str(ORACLE_LIB))
        L.orc_solve_box.restype = c_int
        L.orc_solve_box.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, _F64P, _F64P, _F64P, c_int, c_double,
                                    c_double, c_int64, c_double, c_int, _F64P, POINTER(OrcStats), POINTER(c_int)]
        L.orc_solve_box_csr.restype = c_int
        L.orc_solve_box_csr.argtypes = [c_int64, _I32P, _I32P, _F64P, c_int64, _I64P, _I64P, _F64P, _F64P, _F64P,
                                        _F64P, c_double, c_int64, c_double, c_int, _F64P, POINTER(OrcStats),
                                        POINTER(c_int)]
        L.orc_check.restype = None
        L.orc_check.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, _F64P, _F64P, _F64P, c_int, c_double, _F64P,
                                c_double, POINTER(OrcStats)]
        L.orc_check_convex.restype = c_int
        L.orc_check_convex.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, c_int]
        L.orc_build_csr.restype = c_int64
        L.orc_build_csr.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, c_double, _I32P, _I32P, _F64P]
        L.orc_fista_steps.restype = None
        L.orc_fista_steps.argtypes = [c_int64, _I32P, _I32P, _F64P, _F64P, _F64P, _F64P, c_double, _F64P, _F64P,
                                      _F64P, c_int64, c_int]
        L.orc_max_abs_row_sum.restype = c_double
        L.orc_max_abs_row_sum.argtypes = [c_int64, _I32P, _F64P]
        L.orc_max_threads.restype = c_int
        L.bqp_planted_preset.restype = c_int
        L.bqp_planted_preset.argtypes = [c_int32, c_uint64, c_int64, c_int64, POINTER(PlantedSpec)]
        L.bqp_planted_create.restype = c_void_p
        L.bqp_planted_create.argtypes = [POINTER(PlantedSpec)]
        L.bqp_planted_info.restype = c_int
        L.bqp_planted_info.argtypes = [c_void_p, _I64P, _I64P, _I64P, _F64P]
        L.bqp_planted_copy.restype = c_int
        L.bqp_planted_copy.argtypes = [c_void_p, _I32P, _I32P, _F64P, _F64P, _F64P, _F64P, _F64P, _F64P]
        L.bqp_planted_copy_lower.restype = c_int
        L.bqp_planted_copy_lower.argtypes = [c_void_p, _I64P, _I64P, _F64P]
        L.bqp_planted_free.restype = None
        L.bqp_planted_free.argtypes = [c_void_p]
        _orc = L
    return _orc


def planted(preset, seed=1, index=0, n=0, lower_triplets=True):
    """One planted instance from the generator linked into liboracle.so (the engine's generator,
    so the arrays equal boxqp.planted's bit for bit); a dict of numpy arrays and scalars."""
    L = orc()
    spec = PlantedSpec()
    if L.bqp_planted_preset(PRESETS[preset] if isinstance(preset, str) else int(preset), int(seed), int(index), int(n),
                            spec) != 0:
        raise ValueError(f'bad preset {preset!r}')
    h = L.bqp_planted_create(spec)
    if not h:
        raise ValueError('planted generation failed')
    try:
        nn, nnz, nl, fstar = c_int64(0), c_int64(0), c_int64(0), c_double(0)
        L.bqp_planted_info(h, ctypes.byref(nn), ctypes.byref(nnz), ctypes.byref(nl), ctypes.byref(fstar))
        n_, z_ = nn.value, nnz.value
        out = {'n': n_, 'nnz': z_, 'fstar': fstar.value, 'rowptr': np.empty(n_ + 1, np.int32),
               'col': np.empty(z_, np.int32), 'val': np.empty(z_), 'c': np.empty(n_), 'lower': np.empty(n_),
               'upper': np.empty(n_), 'xstar': np.empty(n_), 'z': np.empty(n_)}
        L.bqp_planted_copy(h, _p(out['rowptr'], c_int32), _p(out['col'], c_int32), _p(out['val'], c_double),
                           _p(out['c'], c_double), _p(out['lower'], c_double), _p(out['upper'], c_double),
                           _p(out['xstar'], c_double), _p(out['z'], c_double))
        if lower_triplets:
            k = nl.value
            hr, hc, hv = np.empty(k, np.int64), np.empty(k, np.int64), np.empty(k)
            L.bqp_planted_copy_lower(h, _p(hr, c_int64), _p(hc, c_int64), _p(hv, c_double))
            out['hrow'], out['hcol'], out['hval'] = hr, hc, hv
        return out
    finally:
        L.bqp_planted_free(h)


def active_set_mismatches(x, inst, margin=1e-6, atol=1e-9):
    """Variables whose bound state in x differs from the planted optimum's, counted where the
    planted margin exceeds `margin`: a dual |z| > margin puts x* strictly at its bound (x must sit
    on that bound within atol), and an interior x* farther than `margin` from both bounds must not
    sit on a bound."""
    x = np.asarray(x, dtype=np.float64)
    lo, up, z, xs = (np.asarray(inst[k], dtype=np.float64) for k in ('lower', 'upper', 'z', 'xstar'))
    at_lo = np.abs(x - lo) <= atol * (1 + np.abs(lo))
    at_up = np.abs(x - up) <= atol * (1 + np.abs(up))
    want_lo = z > margin
    want_up = z < -margin
    interior = (z == 0) & (xs - lo > margin) & (up - xs > margin)
    bad = (want_lo & ~at_lo) | (want_up & ~at_up) | (interior & (at_lo | at_up))
    return int(np.count_nonzero(bad))


def ref_available():
    return REF_LIB.exists()


def ref():
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise RuntimeError('oracle/_ref is not built (the reference checkout is needed to build it)')
        L = ctypes.CDLL(str(REF_LIB))
        L.ref_solve_box.restype = c_int
        L.ref_solve_box.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, _F64P, _F64P, _F64P, c_int, c_double,
                                    c_double, c_int64, c_double, c_int, _F64P, _F64P, c_char_p, c_int]
        L.ref_solve_qp_admm.restype = c_int
        L.ref_solve_qp_admm.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, _F64P, _F64P, _F64P, c_int64,
                                        POINTER(c_int32), POINTER(c_int32), _F64P, _F64P, _F64P, c_double, c_int64,
                                        c_double, c_int, c_int, c_double, _F64P, _F64P, _F64P, c_char_p, c_int]
        L.ref_solve_diagonal_equalities.restype = c_int
        L.ref_solve_diagonal_equalities.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, _F64P, _F64P, _F64P,
                                                    c_int64, POINTER(c_int32), POINTER(c_int32), _F64P, _F64P, _F64P,
                                                    c_double, c_int64, c_int, _F64P, _F64P, _F64P, c_char_p, c_int]
        L.ref_check_rows.restype = c_int
        L.ref_check_rows.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, _F64P, _F64P, _F64P, c_int, c_double,
                                     c_int64, POINTER(c_int32), POINTER(c_int32), _F64P, _F64P, _F64P, _F64P, _F64P,
                                     c_double, _F64P]
        L.ref_check.restype = c_int
        L.ref_check.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, _F64P, _F64P, _F64P, c_int, c_double, _F64P,
                                c_double, _F64P]
        L.ref_check_convex.restype = c_int
        L.ref_check_convex.argtypes = [c_int64, c_int64, _I64P, _I64P, _F64P, c_int]
        L.ref_qplib_open.restype = c_void_p
        L.ref_qplib_open.argtypes = [c_char_p, c_char_p, c_int]
        L.ref_qplib_sizes.restype = None
        L.ref_qplib_sizes.argtypes = [c_void_p, _I64P, _I64P, _I64P, POINTER(c_int), _F64P]
        L.ref_qplib_copy.restype = None
        L.ref_qplib_copy.argtypes = [c_void_p, _I64P, _I64P, _F64P, _F64P, _F64P, _F64P]
        L.ref_qplib_rows.restype = None
        L.ref_qplib_rows.argtypes = [c_void_p, POINTER(c_int32), POINTER(c_int32), _F64P, _F64P, _F64P]
        L.ref_qplib_row_entries.restype = c_int64
        L.ref_qplib_row_entries.argtypes = [c_void_p]
        L.ref_qplib_close.restype = None
        L.ref_qplib_close.argtypes = [c_void_p]
        L.ref_last_solve_seconds.restype = c_double
        L.ref_last_solve_seconds.argtypes = []
        _ref = L
    return _ref


def _p(a, t):
    return a.ctypes.data_as(POINTER(t))


def _arrays(hrow, hcol, hval, cost, lower, upper):
    return (np.ascontiguousarray(hrow, np.int64), np.ascontiguousarray(hcol, np.int64),
            np.ascontiguousarray(hval, np.float64), np.ascontiguousarray(cost, np.float64),
            np.ascontiguousarray(lower, np.float64), np.ascontiguousarray(upper, np.float64))


def solve_box(hrow, hcol, hval, cost, lower, upper, tol=1e-7, iteration_limit=200000, time_limit=30.0,
              threads=1, maximize=False, offset=0.0):
    """Oracle solve_accelerated_box(cuda=false); returns (status, x, stats dict)."""
    hrow, hcol, hval, cost, lower, upper = _arrays(hrow, hcol, hval, cost, lower, upper)
    n = cost.shape[0]
    x = np.zeros(n)
    st = OrcStats()
    status = c_int(-1)
    rc = orc().orc_solve_box(n, hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double),
                             _p(cost, c_double), _p(lower, c_double), _p(upper, c_double), int(maximize),
                             float(offset), float(tol), int(iteration_limit), float(time_limit), int(threads),
                             _p(x, c_double), st, ctypes.byref(status))
    if rc == 1:
        raise ValueError('invalid argument')
    if rc != 0:
        raise MemoryError('oracle allocation failed')
    return STATUS[status.value], x, st.as_dict()


def solve_box_csr(rowptr, col, val, hrow, hcol, hval, cost, lower, upper, tol=1e-7, iteration_limit=200000,
                  time_limit=30.0, threads=1):
    """Oracle FISTA on an assembled full CSR (minimisation, no offset)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    hrow, hcol, hval, cost, lower, upper = _arrays(hrow, hcol, hval, cost, lower, upper)
    n = cost.shape[0]
    x = np.zeros(n)
    st = OrcStats()
    status = c_int(-1)
    rc = orc().orc_solve_box_csr(n, _p(rowptr, c_int32), _p(col, c_int32), _p(val, c_double), hrow.shape[0],
                                 _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double), _p(cost, c_double),
                                 _p(lower, c_double), _p(upper, c_double), float(tol), int(iteration_limit),
                                 float(time_limit), int(threads), _p(x, c_double), st, ctypes.byref(status))
    if rc != 0:
        raise RuntimeError('oracle failure')
    return STATUS[status.value], x, st.as_dict()


def check(hrow, hcol, hval, cost, lower, upper, x, tol=1e-7, maximize=False, offset=0.0):
    """Oracle check_qp_solution; returns the stats dict."""
    hrow, hcol, hval, cost, lower, upper = _arrays(hrow, hcol, hval, cost, lower, upper)
    x = np.ascontiguousarray(x, np.float64)
    st = OrcStats()
    orc().orc_check(cost.shape[0], hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double),
                    _p(cost, c_double), _p(lower, c_double), _p(upper, c_double), int(maximize), float(offset),
                    _p(x, c_double), float(tol), st)
    return st.as_dict()


def check_convex(n, hrow, hcol, hval, maximize=False):
    hrow = np.ascontiguousarray(hrow, np.int64)
    hcol = np.ascontiguousarray(hcol, np.int64)
    hval = np.ascontiguousarray(hval, np.float64)
    return orc().orc_check_convex(n, hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double),
                                  int(maximize))


def build_csr(n, hrow, hcol, hval, sign=1.0):
    hrow = np.ascontiguousarray(hrow, np.int64)
    hcol = np.ascontiguousarray(hcol, np.int64)
    hval = np.ascontiguousarray(hval, np.float64)
    nh = hrow.shape[0]
    rowptr = np.zeros(n + 1, np.int32)
    col = np.zeros(max(2 * nh, 1), np.int32)
    val = np.zeros(max(2 * nh, 1))
    nnz = orc().orc_build_csr(n, nh, _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double), float(sign),
                              _p(rowptr, c_int32), _p(col, c_int32), _p(val, c_double))
    if nnz < 0:
        raise ValueError('invalid Hessian')
    return rowptr, col[:nnz].copy(), val[:nnz].copy()


def fista_steps(rowptr, col, val, c, lower, upper, lipschitz, x, w, t, steps, threads=1):
    """Runs `steps` CPU FISTA iterations in place on (x, w); returns the new t."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    c = np.ascontiguousarray(c, np.float64)
    lower = np.ascontiguousarray(lower, np.float64)
    upper = np.ascontiguousarray(upper, np.float64)
    tt = np.array([t], np.float64)
    orc().orc_fista_steps(c.shape[0], _p(rowptr, c_int32), _p(col, c_int32), _p(val, c_double), _p(c, c_double),
                          _p(lower, c_double), _p(upper, c_double), float(lipschitz), _p(x, c_double),
                          _p(w, c_double), _p(tt, c_double), int(steps), int(threads))
    return float(tt[0])


def max_abs_row_sum(rowptr, val):
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    return orc().orc_max_abs_row_sum(rowptr.shape[0] - 1, _p(rowptr, c_int32), _p(val, c_double))


def max_threads():
    return orc().orc_max_threads()


# ---- the reference itself (oracle/_ref) ---------------------------------------------------
def ref_solve_box(hrow, hcol, hval, cost, lower, upper, tol=1e-7, iteration_limit=200000, time_limit=30.0,
                  threads=1, maximize=False, offset=0.0):
    hrow, hcol, hval, cost, lower, upper = _arrays(hrow, hcol, hval, cost, lower, upper)
    n = cost.shape[0]
    x = np.zeros(n)
    stats = np.zeros(8)
    msg = ctypes.create_string_buffer(256)
    rc = ref().ref_solve_box(n, hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double),
                             _p(cost, c_double), _p(lower, c_double), _p(upper, c_double), int(maximize),
                             float(offset), float(tol), int(iteration_limit), float(time_limit), int(threads),
                             _p(x, c_double), _p(stats, c_double), msg, 256)
    if rc == 1:
        raise ValueError(msg.value.decode())
    if rc != 0:
        raise RuntimeError(msg.value.decode())
    keys = ['objective', 'primal_residual', 'stationarity_residual', 'complementarity_residual', 'dual_bound',
            'relative_gap', 'verified', 'iterations']
    st = dict(zip(keys, stats.tolist()))
    st['seconds'] = float(ref().ref_last_solve_seconds())  # the solve_accelerated_box call alone
    return msg.value.decode(), x, st


def ref_solve_qp_admm(hrow, hcol, hval, cost, lower, upper, a_rowptr, a_col, a_val, row_lower, row_upper,
                      tol=1e-7, iteration_limit=200000, time_limit=30.0, scaling=True, maximize=False, offset=0.0):
    """The reference's solve_qp_admm (src/qp_admm.cpp:118-280) on a QP with constraint rows."""
    hrow, hcol, hval, cost, lower, upper = _arrays(hrow, hcol, hval, cost, lower, upper)
    a_rowptr = np.ascontiguousarray(a_rowptr, np.int32)
    a_col = np.ascontiguousarray(a_col, np.int32)
    a_val = np.ascontiguousarray(a_val, np.float64)
    row_lower = np.ascontiguousarray(row_lower, np.float64)
    row_upper = np.ascontiguousarray(row_upper, np.float64)
    n, m = cost.shape[0], a_rowptr.shape[0] - 1
    x = np.zeros(n)
    row_dual = np.zeros(m)
    stats = np.zeros(8)
    msg = ctypes.create_string_buffer(256)
    rc = ref().ref_solve_qp_admm(n, hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double),
                                 _p(cost, c_double), _p(lower, c_double), _p(upper, c_double), m,
                                 _p(a_rowptr, c_int32), _p(a_col, c_int32), _p(a_val, c_double),
                                 _p(row_lower, c_double), _p(row_upper, c_double), float(tol), int(iteration_limit),
                                 float(time_limit), 1 if scaling else 0, int(maximize), float(offset),
                                 _p(x, c_double), _p(row_dual, c_double),
                                 _p(stats, c_double), msg, 256)
    if rc == 1:
        raise ValueError(msg.value.decode())
    if rc != 0:
        raise RuntimeError(msg.value.decode())
    keys = ['objective', 'primal_residual', 'stationarity_residual', 'complementarity_residual', 'dual_bound',
            'relative_gap', 'verified', 'iterations']
    st = dict(zip(keys, stats.tolist()))
    st['row_dual'] = row_dual
    return msg.value.decode(), x, st


def ref_solve_diagonal_equalities(hrow, hcol, hval, cost, lower, upper, a_rowptr, a_col, a_val, row_lower,
                                  row_upper, tol=1e-7, iteration_limit=200000, scaling=True):
    """The reference's solve_diagonal_equalities (src/qp_dual_newton.cpp:9-66), the dual Newton
    solver solve_qp_admm tries first on diagonal Hessians with equality rows; returns (status, x,
    stats with 'row_dual')."""
    hrow, hcol, hval, cost, lower, upper = _arrays(hrow, hcol, hval, cost, lower, upper)
    a_rowptr = np.ascontiguousarray(a_rowptr, np.int32)
    a_col = np.ascontiguousarray(a_col, np.int32)
    a_val, row_lower, row_upper = (np.ascontiguousarray(v, np.float64) for v in (a_val, row_lower, row_upper))
    n, m = cost.shape[0], a_rowptr.shape[0] - 1
    x, row_dual, stats = np.zeros(n), np.zeros(m), np.zeros(8)
    msg = ctypes.create_string_buffer(256)
    rc = ref().ref_solve_diagonal_equalities(n, hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64),
                                             _p(hval, c_double), _p(cost, c_double), _p(lower, c_double),
                                             _p(upper, c_double), m, _p(a_rowptr, c_int32), _p(a_col, c_int32),
                                             _p(a_val, c_double), _p(row_lower, c_double), _p(row_upper, c_double),
                                             float(tol), int(iteration_limit), 1 if scaling else 0, _p(x, c_double),
                                             _p(row_dual, c_double), _p(stats, c_double), msg, 256)
    if rc != 0:
        raise RuntimeError(msg.value.decode())
    keys = ['objective', 'primal_residual', 'stationarity_residual', 'complementarity_residual', 'dual_bound',
            'relative_gap', 'verified', 'iterations']
    st = dict(zip(keys, stats.tolist()))
    st['row_dual'] = row_dual
    return msg.value.decode(), x, st


def ref_check_rows(hrow, hcol, hval, cost, lower, upper, a_rowptr, a_col, a_val, row_lower, row_upper, x, row_dual,
                   tol=1e-7, maximize=False, offset=0.0):
    """The reference's check_qp_solution (src/qp_admm.cpp:63-117) on a problem with linear rows."""
    hrow, hcol, hval, cost, lower, upper = _arrays(hrow, hcol, hval, cost, lower, upper)
    a_rowptr = np.ascontiguousarray(a_rowptr, np.int32)
    a_col = np.ascontiguousarray(a_col, np.int32)
    a_val, row_lower, row_upper, x, row_dual = (np.ascontiguousarray(v, np.float64)
                                                for v in (a_val, row_lower, row_upper, x, row_dual))
    stats = np.zeros(8)
    rc = ref().ref_check_rows(cost.shape[0], hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double),
                              _p(cost, c_double), _p(lower, c_double), _p(upper, c_double), int(maximize),
                              float(offset), a_rowptr.shape[0] - 1, _p(a_rowptr, c_int32), _p(a_col, c_int32),
                              _p(a_val, c_double), _p(row_lower, c_double), _p(row_upper, c_double),
                              _p(x, c_double), _p(row_dual, c_double), float(tol), _p(stats, c_double))
    if rc != 0:
        raise RuntimeError('reference checker failed')
    keys = ['objective', 'primal_residual', 'stationarity_residual', 'complementarity_residual', 'dual_bound',
            'relative_gap', 'verified']
    return dict(zip(keys, stats.tolist()))


def ref_check(hrow, hcol, hval, cost, lower, upper, x, tol=1e-7, maximize=False, offset=0.0):
    hrow, hcol, hval, cost, lower, upper = _arrays(hrow, hcol, hval, cost, lower, upper)
    x = np.ascontiguousarray(x, np.float64)
    stats = np.zeros(8)
    ref().ref_check(cost.shape[0], hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double),
                    _p(cost, c_double), _p(lower, c_double), _p(upper, c_double), int(maximize), float(offset),
                    _p(x, c_double), float(tol), _p(stats, c_double))
    keys = ['objective', 'primal_residual', 'stationarity_residual', 'complementarity_residual', 'dual_bound',
            'relative_gap', 'verified', 'iterations']
    return dict(zip(keys, stats.tolist()))


def ref_check_convex(n, hrow, hcol, hval, maximize=False):
    hrow = np.ascontiguousarray(hrow, np.int64)
    hcol = np.ascontiguousarray(hcol, np.int64)
    hval = np.ascontiguousarray(hval, np.float64)
    return ref().ref_check_convex(n, hrow.shape[0], _p(hrow, c_int64), _p(hcol, c_int64), _p(hval, c_double),
                                  int(maximize))


def ref_read_qplib(path):
    """Parses a QPLIB file with the reference's reader; returns a dict of arrays."""
    msg = ctypes.create_string_buffer(256)
    h = ref().ref_qplib_open(str(path).encode(), msg, 256)
    if not h:
        raise ValueError(msg.value.decode())
    try:
        n, nh, m = c_int64(0), c_int64(0), c_int64(0)
        mx = c_int(0)
        off = c_double(0)
        ref().ref_qplib_sizes(h, ctypes.byref(n), ctypes.byref(nh), ctypes.byref(m), ctypes.byref(mx),
                              ctypes.byref(off))
        hr, hc, hv = np.zeros(nh.value, np.int64), np.zeros(nh.value, np.int64), np.zeros(nh.value)
        cost, lo, up = np.zeros(n.value), np.zeros(n.value), np.zeros(n.value)
        ref().ref_qplib_copy(h, _p(hr, c_int64), _p(hc, c_int64), _p(hv, c_double), _p(cost, c_double),
                             _p(lo, c_double), _p(up, c_double))
        k = ref().ref_qplib_row_entries(h)
        rp, rc, rv = np.zeros(m.value + 1, np.int32), np.zeros(max(k, 1), np.int32), np.zeros(max(k, 1))
        rl, ru = np.zeros(m.value), np.zeros(m.value)
        ref().ref_qplib_rows(h, _p(rp, c_int32), _p(rc, c_int32), _p(rv, c_double), _p(rl, c_double),
                             _p(ru, c_double))
        return {'n': n.value, 'rows': m.value, 'maximize': bool(mx.value), 'offset': off.value, 'hrow': hr,
                'hcol': hc, 'hval': hv, 'cost': cost, 'lower': lo, 'upper': up, 'a_rowptr': rp, 'a_col': rc[:k],
                'a_val': rv[:k], 'row_lower': rl, 'row_upper': ru}
    finally:
        ref().ref_qplib_close(h)
