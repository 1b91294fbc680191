"""Host mirror of the constrained-QP ADMM inner solve on the GPU (C-ABI bqp_admm_*).

The reference's ADMM (02-software/solver/src/qp_admm.cpp:120-280) spends its iterations in the
x-update's linear system K x = rhs, K = H + sigma I + A' diag(rho) A, solved by Jacobi-
preconditioned CG (qp_admm.cpp:262-273).  AdmmSystem keeps H and A resident on the device and
runs that inner solve there as one graph launch:

    s = AdmmSystem(h_rowptr, h_col, h_val, a_rowptr, a_col, a_val, n)
    s.set_rho(rho, sigma)                      # also forms the preconditioner
    x, inner, resid = s.solve(rhs, x0, accuracy, max_inner)
    x, z, y, inner = s.iterate(c, lo, up, x, z, y, first_iteration, iterations)   # whole ADMM steps
"""
import numpy as np

from . import _native as N
from ._native import lib, ptr


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class AdmmSystem:
    """K = H + sigma I + A' diag(rho) A resident on one GPU (H: n x n CSR, A: m x n CSR)."""

    def __init__(self, h_rowptr, h_col, h_val, a_rowptr, a_col, a_val, n, device=0):
        self._keep = [_i32(h_rowptr), _i32(h_col), _f64(h_val), _i32(a_rowptr), _i32(a_col), _f64(a_val)]
        hr, hc, hv, ar, ac, av = self._keep
        self.n = int(n)
        self.m = int(ar.shape[0] - 1)
        self._s = lib().bqp_admm_create(int(device), self.n, self.m, ptr(hr, N.c_int32), ptr(hc, N.c_int32),
                                        ptr(hv, N.c_double), ptr(ar, N.c_int32), ptr(ac, N.c_int32),
                                        ptr(av, N.c_double))
        if not self._s:
            msg = lib().bqp_admm_last_error()
            raise ValueError(msg.decode() if msg else 'bqp_admm_create failed')

    def _check(self, rc):
        if rc == 1:
            raise ValueError('invalid argument')
        if rc != 0:
            msg = lib().bqp_admm_last_error()
            raise RuntimeError(msg.decode() if msg else f'bqp_admm error {rc}')

    def set_rho(self, rho, sigma):
        rho = _f64(rho)
        if rho.shape != (self.m,):
            raise ValueError('rho must have one entry per row of A')
        self._check(lib().bqp_admm_set_rho(self._s, ptr(rho, N.c_double), float(sigma)))

    def apply(self, v):
        v = _f64(v)
        out = np.empty(self.n)
        self._check(lib().bqp_admm_apply(self._s, ptr(v, N.c_double), ptr(out, N.c_double)))
        return out

    def solve(self, rhs, x0, accuracy, max_inner):
        """(x, inner iterations, final max|r|) of the reference's inner PCG from x0."""
        rhs = _f64(rhs)
        x = np.array(x0, dtype=np.float64, copy=True)
        inner = N.c_int64(0)
        resid = N.c_double(0)
        self._check(lib().bqp_admm_solve(self._s, ptr(rhs, N.c_double), ptr(x, N.c_double), float(accuracy),
                                         int(max_inner), N.ctypes.byref(inner), N.ctypes.byref(resid)))
        return x, inner.value, resid.value

    def iterate(self, c, lo, up, x, z, y, first_iteration, iterations):
        """`iterations` ADMM iterations of the reference's loop on the device (bqp_admm_iterate);
        returns (x, z, y, inner iterations in total)."""
        c, lo, up = _f64(c), _f64(lo), _f64(up)
        x = np.array(x, dtype=np.float64, copy=True)
        z = np.array(z, dtype=np.float64, copy=True)
        y = np.array(y, dtype=np.float64, copy=True)
        if c.shape != (self.n,) or x.shape != (self.n,) or any(v.shape != (self.m,) for v in (lo, up, z, y)):
            raise ValueError('c and x need n entries; lo, up, z and y one per row of A')
        total = N.c_int64(0)
        self._check(lib().bqp_admm_iterate(self._s, ptr(c, N.c_double), ptr(lo, N.c_double), ptr(up, N.c_double),
                                           ptr(x, N.c_double), ptr(z, N.c_double), ptr(y, N.c_double),
                                           int(first_iteration), int(iterations), N.ctypes.byref(total)))
        return x, z, y, total.value

    def close(self):
        if getattr(self, '_s', None):
            lib().bqp_admm_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
