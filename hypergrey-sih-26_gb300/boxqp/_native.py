"""ctypes binding of libboxqp.so (the C-ABI declared in include/boxqp.h).

The library is the product path: there is no Python or CPU fallback.  Loading fails loudly
when the library has not been built.
"""
import ctypes
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_size_t, c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / 'libboxqp.so'

BQP_OK = 0
ERRORS = {1: 'invalid_argument', 2: 'cuda_error', 3: 'no_device', 4: 'admission', 5: 'not_found',
          6: 'not_ready', 7: 'unsupported', 8: 'no_memory'}
STATUS_NAMES = {0: 'optimal', 1: 'iteration_limit', 2: 'time_limit', 3: 'numerical_error',
                4: 'unsupported_curvature', 5: 'infeasible_bounds', 100: 'queued', 101: 'running'}
PRECISIONS = {'fp64': 0, 'mixed': 1, 'fp64_exact': 2}


class Options(ctypes.Structure):
    _fields_ = [('tolerance', c_double), ('time_limit', c_double), ('iteration_limit', c_int64),
                ('precision', c_int32), ('lipschitz', c_int32), ('check_interval', c_int32),
                ('diagonal_gate', c_int32), ('offset', c_double), ('kernel_variant', c_int32),
                ('scaling', c_int32), ('polish_switch', c_double)]


class Stats(ctypes.Structure):
    _fields_ = [('status', c_int32), ('verified', c_int32), ('iterations', c_int64),
                ('polish_iterations', c_int64), ('polish_rounds', c_int64), ('objective', c_double),
                ('primal_residual', c_double), ('stationarity_residual', c_double),
                ('complementarity_residual', c_double), ('dual_bound', c_double), ('relative_gap', c_double),
                ('lipschitz', c_double), ('device_seconds', c_double), ('bytes', c_double),
                ('device_start_ns', c_int64), ('device_end_ns', c_int64), ('checks', c_int64)]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_}
        d['status_name'] = STATUS_NAMES.get(self.status, str(self.status))
        return d


class PlantedSpec(ctypes.Structure):
    _fields_ = [('family', c_int32), ('edges_per_vertex', c_int32), ('n', c_int64), ('grid_side', c_int32),
                ('bounds_mode', c_int32), ('seed', c_uint64), ('lower', c_double), ('upper', c_double),
                ('frac_lower', c_double), ('frac_upper', c_double), ('interior_lo', c_double),
                ('interior_hi', c_double), ('diag_lo', c_double), ('diag_hi', c_double),
                ('weight_lo', c_double), ('weight_hi', c_double), ('shift', c_double), ('dual_lo', c_double),
                ('dual_hi', c_double)]


_I32P = POINTER(c_int32)
_I64P = POINTER(c_int64)
_F64P = POINTER(c_double)
_U64P = POINTER(c_uint64)

# name -> (restype, argtypes)
PROTOTYPES = {
    'bqp_options_default': (None, [POINTER(Options)]),
    'bqp_create': (c_void_p, [c_int, c_size_t]),
    'bqp_destroy': (None, [c_void_p]),
    'bqp_last_error': (c_char_p, [c_void_p]),
    'bqp_device_name': (c_int, [c_int, c_char_p, c_size_t]),
    'bqp_host_register': (c_int, [c_void_p, c_size_t]),
    'bqp_host_unregister': (c_int, [c_void_p]),
    'bqp_submit': (c_int, [c_void_p, c_int64, c_int64, _I32P, _I32P, _F64P, _F64P, _F64P, _F64P,
                           POINTER(Options), _U64P]),
    'bqp_submit_borrowed': (c_int, [c_void_p, c_int64, c_int64, _I32P, _I32P, _F64P, _F64P, _F64P, _F64P,
                                    POINTER(Options), _U64P]),
    'bqp_poll': (c_int, [c_void_p, c_uint64, _I32P]),
    'bqp_wait': (c_int, [c_void_p, c_uint64, c_double]),
    'bqp_wait_any': (c_int, [c_void_p, c_double, _U64P]),
    'bqp_fetch': (c_int, [c_void_p, c_uint64, _F64P, POINTER(Stats)]),
    'bqp_release': (c_int, [c_void_p, c_uint64]),
    'bqp_resolve': (c_int, [c_void_p, _U64P, c_int64]),
    'bqp_set_latency_target': (c_int, [c_void_p, c_double]),
    'bqp_inject_admission_oom': (c_int, [c_void_p, c_int32]),
    'bqp_load': (c_int, [c_void_p, _I64P, _I64P, _I64P, _I64P]),
    'bqp_timer': (c_int, [c_void_p, c_int32, _F64P, _I64P, _I64P]),
    'bqp_profile_step': (c_int, [c_void_p, c_uint64, c_int32, _F64P, _F64P]),
    'bqp_profile_cg': (c_int, [c_void_p, c_uint64, c_int32, _F64P, _F64P, _F64P, _F64P]),
    'bqp_solve_sync': (c_int, [c_void_p, c_int64, c_int64, _I32P, _I32P, _F64P, _F64P, _F64P, _F64P,
                               POINTER(Options), _F64P, POINTER(Stats)]),
    'bqp_box_create': (c_void_p, [c_int, c_int64, c_int64, _I32P, _I32P, _F64P, _F64P, _F64P, _F64P, c_double]),
    'bqp_box_step': (c_int, [c_void_p, c_double]),
    'bqp_box_primal': (c_int, [c_void_p, _F64P]),
    'bqp_box_destroy': (None, [c_void_p]),
    'bqp_admm_create': (c_void_p, [c_int, c_int64, c_int64, _I32P, _I32P, _F64P, _I32P, _I32P, _F64P]),
    'bqp_admm_set_rho': (c_int, [c_void_p, _F64P, c_double]),
    'bqp_admm_apply': (c_int, [c_void_p, _F64P, _F64P]),
    'bqp_admm_solve': (c_int, [c_void_p, _F64P, _F64P, c_double, c_int64, _I64P, _F64P]),
    'bqp_admm_iterate': (c_int, [c_void_p, _F64P, _F64P, _F64P, _F64P, _F64P, _F64P, c_int64, c_int64, _I64P]),
    'bqp_admm_last_error': (c_char_p, []),
    'bqp_admm_destroy': (None, [c_void_p]),
    'bqp_box_last_error': (c_char_p, [c_void_p]),
    'bqp_check_device': (c_int, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_double, c_double, c_int32, POINTER(Stats)]),
    'bqp_check_device_noalloc': (c_int, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_double, c_double, c_int32, POINTER(Stats)]),
    'bqp_gate_device': (c_int, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p, POINTER(c_double),
                                POINTER(c_int32), POINTER(c_int32)]),
    'bqp_csr_from_lower': (c_int, [c_int64, c_int64, _I64P, _I64P, _F64P, c_double, _I32P, _I32P, _F64P, _I64P]),
    'bqp_check_convex': (c_int, [c_int64, c_int64, _I64P, _I64P, _F64P, c_int32]),
    'bqp_gershgorin': (c_double, [c_int64, _I32P, _F64P]),
    'bqp_dot_ld': (c_double, [c_int64, _F64P, _F64P]),
    'bqp_planted_preset': (c_int, [c_int32, c_uint64, c_int64, c_int64, POINTER(PlantedSpec)]),
    'bqp_planted_create': (c_void_p, [POINTER(PlantedSpec)]),
    'bqp_planted_info': (c_int, [c_void_p, _I64P, _I64P, _I64P, _F64P]),
    'bqp_planted_copy': (c_int, [c_void_p, _I32P, _I32P, _F64P, _F64P, _F64P, _F64P, _F64P, _F64P]),
    'bqp_planted_copy_lower': (c_int, [c_void_p, _I64P, _I64P, _F64P]),
    'bqp_planted_free': (None, [c_void_p]),
    'bqp_splitmix64': (c_uint64, [_U64P]),
}

_lib = None


def lib():
    """Loads libboxqp.so once; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f'{LIB_PATH.name} is not built: run __graft_entry__.build() '
                               '(the engine has no CPU fallback)')
        handle = ctypes.CDLL(str(LIB_PATH))
        for name, (restype, argtypes) in PROTOTYPES.items():
            fn = getattr(handle, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = handle
    return _lib


def ptr(array, ctype):
    """Pointer to a contiguous numpy array (None stays NULL)."""
    if array is None:
        return None
    return array.ctypes.data_as(POINTER(ctype))


class EngineError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f'{ERRORS.get(code, code)}: {message}')
        self.code = code
