"""Constrained-QP ADMM on the GPU: the device system (C-ABI bqp_admm_*) and the reference's
solve_qp_admm loop around it.

The reference's ADMM (02-software/solver/src/qp_admm.cpp:118-280) spends its iterations in the
x-update's linear system K x = rhs, K = H + sigma I + A' diag(rho) A, solved by Jacobi-
preconditioned CG (qp_admm.cpp:262-273).  AdmmSystem keeps H and A resident on the device and
runs that inner solve there as one graph launch, or whole ADMM iterations:

    s = AdmmSystem(h_rowptr, h_col, h_val, a_rowptr, a_col, a_val, n)
    s.set_rho(rho, sigma)                      # also forms the preconditioner
    x, inner, resid = s.solve(rhs, x0, accuracy, max_inner)
    x, z, y, inner = s.iterate(c, lo, up, x, z, y, first_iteration, iterations)   # whole ADMM steps

solve_qp_admm(q, rows, options) is the reference's entry point over it: the scaled set-up
(admm_setup), 25 iterations per device call, the original-model check of the primal and row
duals every 25 iterations (check_solution, the reference's check_qp_solution with rows) and the
rho adaptation every 100 (adapt_rho) on the host between calls.
"""
import math
import time
from dataclasses import dataclass

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


# ------------------------------------------------------------------------------------------
# the reference's solve_qp_admm around the device iterations
# ------------------------------------------------------------------------------------------
@dataclass
class LinearRows:
    """Linear rows row_lower <= A x <= row_upper of a QP (the reference's LinearProblem rows,
    row_lower, row_upper, include/mps.hpp), A as CSR with m rows over the n variables.  Equal
    bounds make an equality row; infinite ones a one-sided row."""
    rowptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    lower: np.ndarray
    upper: np.ndarray

    @property
    def m(self):
        return int(np.asarray(self.rowptr).shape[0] - 1)


def merge_rows(rowptr, col, val):
    """CSR of rows given as (column, value) lists, as the reference's CsrMatrix(n, rows) forms it
    (include/sparse_matrix.hpp:10-17): columns ascending, duplicates summed in input order, zero
    results dropped."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    val = np.asarray(val, dtype=np.float64)
    m = rowptr.shape[0] - 1
    row = np.repeat(np.arange(m, dtype=np.int64), np.diff(rowptr))
    order = np.lexsort((col, row))  # stable: equal (row, column) keys keep their input order
    r, c, v = row[order], col[order], val[order]
    first = np.ones(r.shape[0], dtype=bool)
    first[1:] = (r[1:] != r[:-1]) | (c[1:] != c[:-1])
    starts = np.flatnonzero(first)
    sums = v[starts].copy()
    sizes = np.diff(np.append(starts, r.shape[0]))
    for g in np.flatnonzero(sizes > 1):  # duplicates: summed one after another, as a std::map entry
        acc = 0.0
        for k in range(starts[g], starts[g] + sizes[g]):
            acc += v[k]
        sums[g] = acc
    keep = sums != 0
    rr, cc, vv = r[starts][keep], c[starts][keep], sums[keep]
    out_ptr = np.zeros(m + 1, dtype=np.int32)
    np.cumsum(np.bincount(rr, minlength=m), out=out_ptr[1:])
    return out_ptr, cc.astype(np.int32), vv


def _row_of(rowptr):
    return np.repeat(np.arange(len(rowptr) - 1), np.diff(np.asarray(rowptr, dtype=np.int64)))


def row_sums(rowptr, terms, initial=0.0):
    """Per-row sums of CSR-ordered terms, in the terms' dtype, each row summed from `initial` one
    entry after another in entry order, as the reference's loops sum them (np.add.at applies its
    updates in index order, unbuffered)."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    out = np.full(rowptr.shape[0] - 1, initial, dtype=terms.dtype)
    if len(terms):
        np.add.at(out, _row_of(rowptr), terms)
    return out


def dot_ld(a, b):
    """sum_j a_j b_j accumulated in long double in order (the reference's dot, qp_admm.cpp:23;
    bqp_dot_ld in the library)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return lib().bqp_dot_ld(a.shape[0], ptr(a, N.c_double), ptr(b, N.c_double))


class _Csr:
    """A CSR matrix for repeated products on the host: scipy's CSR product, which sums each row
    from 0 in entry order as CsrMatrix::multiply does (include/sparse_matrix.hpp:26-33), with the
    entries kept in the given order."""

    def __init__(self, rowptr, col, val, n_cols):
        import scipy.sparse as sps
        rowptr = np.asarray(rowptr, dtype=np.int64)
        self.m = sps.csr_matrix((np.asarray(val, dtype=np.float64), np.asarray(col, dtype=np.int64), rowptr),
                                shape=(rowptr.shape[0] - 1, n_cols))

    def mul(self, v):
        return self.m @ v


def csr_multiply(rowptr, col, val, v):
    """A v (CsrMatrix::multiply, include/sparse_matrix.hpp:26-33: each row's products summed from 0
    in entry order)."""
    return row_sums(rowptr, np.asarray(val, dtype=np.float64) * v[np.asarray(col, dtype=np.int64)])


def _clip(x, lo, up):
    # max(lo, min(up, x)), elementwise
    return np.maximum(lo, np.minimum(up, x))


def _norm(v):
    return float(np.max(np.abs(v))) if len(v) else 0.0


def admm_setup(q, rows, scaling=True):
    """The reference's set-up of solve_qp_admm (qp_admm.cpp:136-158) as arrays: the Hessian in
    full CSR (sign-normalised for a maximisation), variable units 1/sqrt(H_jj) on a positive
    diagonal, row scales 1/max|a_ij| of the unit-scaled rows, the bound rows x_j appended to A,
    the cost scale 1/max(1, |c|), the scaled H, A, c and bounds, the initial x = clip(0) and
    z = clip(A x), rho (0.1, x100 on rows with equal bounds) and sigma = 1e-8."""
    from .api import csr_from_lower
    n, m = q.n, rows.m
    sign = -1.0 if q.maximize else 1.0
    hrp, hci, hva = csr_from_lower(n, q.hessian_row, q.hessian_col, q.hessian_val, sign)
    hrow = _row_of(hrp)
    on_diag = hci == hrow

    def diagonal_of(values):
        d = np.zeros(n)
        d[hrow[on_diag]] = values[on_diag]
        return d

    variable = np.ones(n)
    diag0 = diagonal_of(hva)
    if scaling:
        pos = diag0 > 0
        variable[pos] = 1 / np.sqrt(np.maximum(1e-16, diag0[pos]))
    hva = hva * (variable[hrow] * variable[hci])
    arp = np.asarray(rows.rowptr, dtype=np.int64)
    acol = np.asarray(rows.col, dtype=np.int64)
    aval = np.asarray(rows.val, dtype=np.float64) * variable[acol]
    arow = _row_of(arp)
    maximum = np.zeros(m)
    np.maximum.at(maximum, arow, np.abs(aval))
    row_scale = np.ones(m + n)
    if scaling:
        row_scale[:m] = np.where(maximum > 0, 1 / np.where(maximum > 0, maximum, 1.0), 1.0)
    aval = aval * row_scale[arow]
    lo = np.concatenate([np.asarray(rows.lower, dtype=np.float64) * row_scale[:m],
                         np.asarray(q.lower, dtype=np.float64) / variable])
    up = np.concatenate([np.asarray(rows.upper, dtype=np.float64) * row_scale[:m],
                         np.asarray(q.upper, dtype=np.float64) / variable])
    c = np.asarray(q.cost, dtype=np.float64) * (sign * variable)
    cost_scale = 1 / max(1.0, _norm(c)) if scaling else 1.0
    hva = hva * cost_scale
    c = c * cost_scale
    rows_input = (np.concatenate([arp, arp[-1] + 1 + np.arange(n)]), np.concatenate([acol, np.arange(n)]),
                  np.concatenate([aval, np.ones(n)]))
    a_ptr, a_col, a_val = merge_rows(*rows_input)
    x = _clip(np.zeros(n), lo[m:], up[m:])
    z = _clip(csr_multiply(a_ptr, a_col, a_val, x), lo, up)
    rho_base = 0.1
    diagonal = diagonal_of(hva)
    diagonal_hessian = bool(np.all(diagonal > 0) and np.all(on_diag))
    return {'n': n, 'm': m, 'h': (hrp, hci, hva), 'a': (a_ptr, a_col, a_val), 'c': c, 'lo': lo, 'up': up,
            'rows_input': rows_input, 'diagonal': diagonal, 'diagonal_hessian': diagonal_hessian,
            'variable': variable, 'row_scale': row_scale, 'cost_scale': cost_scale, 'sign': sign,
            'rho_base': rho_base, 'rho': np.where(lo == up, rho_base * 100, rho_base * 1), 'sigma': 1e-8,
            'x': x, 'z': z, 'y': np.zeros(m + n)}


def transpose(rowptr, col, val, n):
    """A' in CSR (rows of A' list the rows of A in increasing order)."""
    row = _row_of(rowptr)
    order = np.argsort(np.asarray(col, dtype=np.int64), kind='stable')
    tp = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(np.bincount(np.asarray(col, dtype=np.int64), minlength=n), out=tp[1:])
    return tp, row[order].astype(np.int32), np.asarray(val)[order]


def adapt_rho(sp, x, z, y, rho_base, at=None):
    """The reference's rho adaptation (qp_admm.cpp:265-271): primal residual max|Ax - z| /
    (1 + max(|Ax|, |z|)), dual residual max|Hx + c + A'y| / (1 + max(|c|, |Hx|, |A'y|)); the
    candidate rho_base sqrt(primal / dual) (both floored at 1e-16, the result clamped to
    [1e-6, 1e6]) replaces rho_base only when it leaves [rho_base / 5, 5 rho_base]."""
    if at is None:
        at = transpose(*sp['a'], sp['n'])
    ax = csr_multiply(*sp['a'], x)
    hx = csr_multiply(*sp['h'], x)
    aty = csr_multiply(*at, y)
    primal = _norm(ax - z) / (1 + max(_norm(ax), _norm(z)))
    dual = _norm(hx + sp['c'] + aty) / (1 + max(_norm(sp['c']), max(_norm(hx), _norm(aty))))
    nxt = max(1e-6, min(1e6, rho_base * math.sqrt(max(1e-16, primal) / max(1e-16, dual))))
    return nxt if (nxt > 5 * rho_base or nxt < rho_base / 5) else rho_base


def original_violation(q, rows, x):
    """Largest bound violation of x and of the row activities A x, each scaled by
    1 + |bound| + |x_j| (variables) or 1 + |bound| + sum_k |a_ik x_k| (rows) (the reference's
    original_violation(p, x, true), src/mps.cpp:279-303); infinite for a non-finite x or
    activity.  Activities are summed in long double."""
    x = np.asarray(x, dtype=np.float64)
    if not np.all(np.isfinite(x)):
        return math.inf
    result = 0.0
    xl = x.astype(np.longdouble)
    for bound, lower in ((np.asarray(q.lower, dtype=np.float64), True), (np.asarray(q.upper, dtype=np.float64), False)):
        fin = np.isfinite(bound)
        if fin.any():
            v = (bound[fin] - xl[fin]) if lower else (xl[fin] - bound[fin])
            result = max(result, float(np.max((v / (1 + np.abs(bound[fin]) + np.abs(xl[fin]))).astype(np.float64))))
    m = rows.m if rows is not None else 0
    if m:
        rp = np.asarray(rows.rowptr, dtype=np.int64)
        term = np.asarray(rows.val, dtype=np.longdouble) * x[np.asarray(rows.col, dtype=np.int64)]
        act = row_sums(rp, term)
        scale = row_sums(rp, np.abs(term))
        if not np.all(np.isfinite(act)):
            return math.inf
        for bound, lower in ((np.asarray(rows.lower, dtype=np.float64), True),
                             (np.asarray(rows.upper, dtype=np.float64), False)):
            fin = np.isfinite(bound)
            if fin.any():
                v = (bound[fin] - act[fin]) if lower else (act[fin] - bound[fin])
                result = max(result, float(np.max((v / (1 + np.abs(bound[fin]) + scale[fin])).astype(np.float64))))
    return result


def check_solution(q, rows, x, row_dual, tol):
    """The reference's check_qp_solution (src/qp_admm.cpp:63-117) of a primal x and row duals on
    the ORIGINAL problem: objective (long double), scaled primal violation, projected-gradient
    stationarity of H x + c + A' y, complementarity |y_i (a_i x - target_i)| / (1 + |f|), the
    tangent dual bound (or the separable one when the Hessian is diagonal with a positive
    diagonal), the relative gap, and verified = max(primal, stationarity, complementarity) <= tol
    (and gap <= tol for the separable bound).  Returns a dict of those fields."""
    sign = -1.0 if q.maximize else 1.0
    n = q.n
    m = rows.m if rows is not None else 0
    out = {'objective': math.nan, 'primal_residual': math.inf, 'stationarity_residual': math.inf,
           'complementarity_residual': math.inf, 'dual_bound': -math.inf, 'relative_gap': math.inf,
           'verified': False}
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(row_dual, dtype=np.float64)
    if x.shape != (n,) or y.shape != (m,) or not np.all(np.isfinite(x)) or not np.all(np.isfinite(y)):
        return out
    hr = np.asarray(q.hessian_row, dtype=np.int64)
    hc = np.asarray(q.hessian_col, dtype=np.int64)
    hv = np.asarray(q.hessian_val, dtype=np.float64)
    cost = np.asarray(q.cost, dtype=np.float64)
    lower = np.asarray(q.lower, dtype=np.float64)
    upper = np.asarray(q.upper, dtype=np.float64)
    off = hr != hc
    # gradient scatter in the reference's order: (row, col), then the mirror of an off-diagonal term
    idx = np.stack([hr, np.where(off, hc, -1)], axis=1).ravel()
    contrib = np.stack([sign * hv * x[hc], sign * hv * x[hr]], axis=1).ravel()
    sel = idx >= 0
    gradient = np.zeros(n)
    np.add.at(gradient, idx[sel], contrib[sel])
    positive_diagonal = not np.any(hv[off] != 0)
    diagonal = linear = None
    if positive_diagonal:
        diagonal = np.zeros(n, dtype=np.longdouble)
        np.add.at(diagonal, hr[~off], (sign * hv[~off]).astype(np.longdouble))
        positive_diagonal = bool(np.all(diagonal > 0))
        if positive_diagonal:
            linear = (sign * cost).astype(np.longdouble)
    xl = x.astype(np.longdouble)
    terms = np.longdouble(0.5) * xl * gradient.astype(np.longdouble) + (sign * cost * x).astype(np.longdouble)
    value = np.cumsum(np.concatenate([[np.longdouble(sign * q.offset)], terms]))[-1]
    gradient = gradient + sign * cost
    out['objective'] = sign * float(value)
    out['primal_residual'] = original_violation(q, rows, x)
    complementarity = 0.0
    bound = value
    dual_constant = np.longdouble(sign * q.offset)
    if m:
        rp = np.asarray(rows.rowptr, dtype=np.int64)
        col = np.asarray(rows.col, dtype=np.int64)
        val = np.asarray(rows.val, dtype=np.float64)
        row = _row_of(rp)
        np.add.at(gradient, col, val * y[row])
        if positive_diagonal:
            np.add.at(linear, col, val.astype(np.longdouble) * y[row])
        act = row_sums(rp, val.astype(np.longdouble) * x[col])
        target = np.where(y >= 0, np.asarray(rows.upper, dtype=np.float64), np.asarray(rows.lower, dtype=np.float64))
        act_rows = np.flatnonzero(y != 0)
        if len(act_rows):
            yl = y[act_rows].astype(np.longdouble)
            dual_constant = np.cumsum(np.concatenate([[dual_constant], -yl * target[act_rows]]))[-1]
            corr = yl * (act[act_rows] - target[act_rows])
            bound = np.cumsum(np.concatenate([[bound], corr]))[-1]
            with np.errstate(invalid='ignore', over='ignore'):
                res = (np.abs(corr) / (1 + abs(value))).astype(np.float64)
            res[~np.isfinite(res)] = math.inf
            complementarity = float(np.max(res))
    out['complementarity_residual'] = complementarity
    with np.errstate(invalid='ignore', over='ignore'):
        res = np.abs(x - _clip(x - gradient, lower, upper)) / (1 + np.abs(x))
    res[~np.isfinite(gradient) | ~np.isfinite(res)] = math.inf
    out['stationarity_residual'] = float(np.max(res)) if n else 0.0
    # tangent affine underestimator over the box
    g = gradient
    nzg = g != 0
    tgt = np.where(g > 0, lower, upper)
    if np.any(nzg & ~np.isfinite(tgt)):
        bound = np.longdouble(-np.inf)
    else:
        bound = np.cumsum(np.concatenate([[bound], (g[nzg] * (tgt[nzg] - x[nzg])).astype(np.longdouble)]))[-1]
    if positive_diagonal:
        mn = np.maximum(lower.astype(np.longdouble), np.minimum(upper.astype(np.longdouble), -linear / diagonal))
        bound = np.cumsum(np.concatenate([[dual_constant],
                                          np.longdouble(0.5) * diagonal * mn * mn + linear * mn]))[-1]
    out['dual_bound'] = float(bound)
    out['relative_gap'] = float(abs(value - bound) / (1 + abs(value))) if np.isfinite(bound) else math.inf
    verified = math.isfinite(out['objective']) and max(out['primal_residual'], out['stationarity_residual'],
                                                       out['complementarity_residual']) <= tol
    if positive_diagonal:
        verified = verified and out['relative_gap'] <= tol
    out['verified'] = bool(verified)
    return out


def polish_diagonal(q, rows, sp, y, tol):
    """The reference's KKT polish in its diagonal-Hessian form (qp_admm.cpp:165-205), run at
    iterations 250, 1000 and 5000: rows with equal bounds or |y_i| > 1e-5 are taken as active at
    the bound y points to; the multipliers of K x = target (K the active scaled rows, x eliminated
    through the diagonal, x = -(K' lambda + c) / D) come from Jacobi-preconditioned CG on
    K D^-1 K' (a 1e-18 shift on its diagonal, stop at max|r| <= 1e-13 (1 + max|rhs|) or 20,000
    iterations); the candidate is kept only if the original model verifies.  Returns the check
    fields with 'primal' and 'row_dual', or None (no candidate, or it did not verify).  Not the
    form for a Hessian with off-diagonal terms or a zero diagonal, which the reference factors
    with its sparse LU."""
    n, m = sp['n'], sp['m']
    lo, up = sp['lo'], sp['up']
    active = np.flatnonzero((lo == up) | (np.abs(y) > 1e-5))
    if n + len(active) > 10000 or not sp['diagonal_hessian'] or not len(active):
        return None
    target = np.where(lo[active] == up[active], lo[active], np.where(y[active] > 0, up[active], lo[active]))
    if not np.all(np.isfinite(target)):
        return None
    rp_in, col_in, val_in = sp['rows_input']
    lens = np.diff(rp_in)[active]
    sel = np.concatenate([np.arange(rp_in[i], rp_in[i + 1]) for i in active]) if len(active) else np.zeros(0, int)
    sub_ptr = np.zeros(len(active) + 1, dtype=np.int64)
    np.cumsum(lens, out=sub_ptr[1:])
    k_csr = merge_rows(sub_ptr, col_in[sel], val_in[sel])
    k = _Csr(*k_csr, n)
    kt = _Csr(*transpose(*k_csr, n), len(active))
    d = sp['diagonal']
    c = sp['c']
    rhs = -k.mul(c / d) - target
    ds = row_sums(sub_ptr, val_in[sel] * val_in[sel] / d[col_in[sel]], initial=1e-18)
    residual = rhs.copy()
    zp = residual / ds
    direction = zp.copy()
    lam = np.zeros(len(active))
    rz = dot_ld(residual, zp)
    stop = 1e-13 * (1 + _norm(rhs))
    inner = 0
    while inner < 20000 and _norm(residual) > stop:
        mv = k.mul(kt.mul(direction) / d)
        den = dot_ld(direction, mv)
        if not (den > 0) or not math.isfinite(den):
            break
        alpha = rz / den
        lam = lam + alpha * direction
        residual = residual - alpha * mv
        zp = residual / ds
        nxt = dot_ld(residual, zp)
        beta = nxt / rz
        rz = nxt
        direction = zp + beta * direction
        inner += 1
    px = (-(kt.mul(lam) + c) / d) * sp['variable']
    py = np.zeros(m)
    rows_m = active < m
    py[active[rows_m]] = lam[rows_m] * sp['row_scale'][active[rows_m]] / sp['cost_scale']
    chk = check_solution(q, rows, px, py, tol)
    if not chk['verified']:
        return None
    chk['primal'] = px
    chk['row_dual'] = py
    return chk


def polish_kkt(q, rows, sp, y, tol):
    """The reference's KKT polish in its general form (qp_admm.cpp:206-230), for Hessians that are
    not a positive diagonal: rows with equal bounds or |y_i| > 1e-5 are active at the bound that
    y_i >= 0 points to (the lower one for y_i < 0); the regularised KKT system
    [[H + 1e-9 I, K'], [K, -1e-9 I]] [x; lambda] = [-c; target] is factored once (SuperLU here,
    the reference's own sparse LU there) and refined 8 times against the unregularised system;
    the candidate is kept only if the original model verifies.  At most 10,000 unknowns.
    Returns the check fields with 'primal' and 'row_dual', or None."""
    import scipy.sparse as sps
    from scipy.sparse.linalg import splu
    n, m = sp['n'], sp['m']
    lo, up = sp['lo'], sp['up']
    active = np.flatnonzero((lo == up) | (np.abs(y) > 1e-5))
    na = len(active)
    if n + na > 10000:
        return None
    target = np.where(lo[active] == up[active], lo[active], np.where(y[active] >= 0, up[active], lo[active]))
    if not np.all(np.isfinite(target)):
        return None
    reg = 1e-9
    hrp, hci, hva = sp['h']
    arp, aci, ava = sp['a']
    hrow = _row_of(hrp)
    lens = np.diff(np.asarray(arp, dtype=np.int64))[active]
    sel = np.concatenate([np.arange(arp[i], arp[i + 1]) for i in active]) if na else np.zeros(0, dtype=np.int64)
    krow = np.repeat(np.arange(na), lens)
    rows_i = np.concatenate([hrow, np.arange(n), n + krow, aci[sel], n + np.arange(na)])
    cols_i = np.concatenate([hci, np.arange(n), aci[sel], n + krow, n + np.arange(na)])
    vals = np.concatenate([hva, np.full(n, reg), ava[sel], ava[sel], np.full(na, -reg)])
    size = n + na
    mat = sps.coo_matrix((vals, (rows_i, cols_i)), shape=(size, size)).tocsc()
    shift = np.concatenate([np.full(n, reg), np.full(na, -reg)])
    rhs = np.concatenate([-sp['c'], target])
    try:
        factor = splu(mat)
    except RuntimeError:  # singular
        return None
    solution = np.zeros(size)
    residual = rhs.copy()
    for _ in range(8):
        solution = solution + factor.solve(residual)
        residual = rhs - mat @ solution + shift * solution
    if not np.all(np.isfinite(solution)):
        return None
    px = solution[:n] * sp['variable']
    py = np.zeros(m)
    rows_m = active < m
    py[active[rows_m]] = solution[n:][rows_m] * sp['row_scale'][active[rows_m]] / sp['cost_scale']
    chk = check_solution(q, rows, px, py, tol)
    if not chk['verified']:
        return None
    chk['primal'] = px
    chk['row_dual'] = py
    return chk


def solve_diagonal_equalities(q, rows, options):
    """The reference's pre-solver for a positive diagonal Hessian with only finite equality rows
    (src/qp_dual_newton.cpp:9-66), on the host as the reference runs it: whiten the variables by
    the diagonal, scale rows and magnitude, then Newton steps on the concave dual -- x(y) is the
    box projection of -(A'y + c), the Newton direction comes from Jacobi-preconditioned CG on the
    active-set Schur matrix A diag(free) A' (a 1e-12 (1 + max diag) shift), and a backtracking
    line search (Armijo 1e-4, up to 60 halvings) -- checking the original model at every
    iteration, at most 500 of them.  Returns a QpResult: 'optimal', 'iteration_limit',
    'time_limit', 'numerical_stall', 'numerical_scaling_failure' or 'unsupported_structure'
    (another structure, which solve_qp_admm hands to its ADMM)."""
    from .api import QpResult
    start = time.monotonic()
    result = QpResult(status='unsupported_structure', algorithm='diagonal_qp_dual_newton')
    n, m = q.n, rows.m
    sign = -1.0 if q.maximize else 1.0
    rl = np.asarray(rows.lower, dtype=np.float64)
    ru = np.asarray(rows.upper, dtype=np.float64)
    if not m or np.any(rl != ru) or not np.all(np.isfinite(rl)):
        return result
    hr = np.asarray(q.hessian_row, dtype=np.int64)
    hc = np.asarray(q.hessian_col, dtype=np.int64)
    hv = np.asarray(q.hessian_val, dtype=np.float64)
    if np.any((hr != hc) & (hv != 0)):
        return result
    h = np.zeros(n)
    np.add.at(h, hr, sign * hv)
    if not np.all(h > 0) or not np.all(np.isfinite(h)):
        return result
    units = 1 / np.sqrt(h)
    lo = np.asarray(q.lower, dtype=np.float64) / units
    up = np.asarray(q.upper, dtype=np.float64) / units
    c = sign * np.asarray(q.cost, dtype=np.float64) * units
    rp = np.asarray(rows.rowptr, dtype=np.int64)
    col = np.asarray(rows.col, dtype=np.int64)
    row = _row_of(rp)
    val = np.asarray(rows.val, dtype=np.float64) * units[col]
    maximum = np.zeros(m)
    np.maximum.at(maximum, row, np.abs(val))
    row_units = np.where(maximum != 0, 1 / np.where(maximum != 0, maximum, 1.0), 1.0)
    val = val * row_units[row]
    b = rl * row_units
    magnitude = 1.0
    if options.scaling:
        magnitude = max(magnitude, _norm(c), _norm(np.maximum(lo, np.minimum(up, 0.0))), _norm(b))
    units = units * magnitude
    lo, up, c = lo / magnitude, up / magnitude, c / magnitude
    b = b / magnitude
    row_units = row_units * magnitude
    if (not np.all(np.isfinite(units)) or not np.all(np.isfinite(c)) or np.any(np.isnan(lo)) or np.any(np.isnan(up))
            or not np.all(np.isfinite(b)) or not np.all(np.isfinite(row_units))):
        result.status = 'numerical_scaling_failure'
        return result
    a_csr = merge_rows(rp, col, val)
    a = _Csr(*a_csr, n)
    at = _Csr(*transpose(*a_csr, n), m)

    def evaluate(dual):
        raw = -(at.mul(dual) + c)
        free = ((raw >= lo) & (raw <= up)).astype(np.float64)
        primal = np.maximum(lo, np.minimum(up, raw))
        g = a.mul(primal) - b
        terms = np.concatenate([np.longdouble(0.5) * primal.astype(np.longdouble) * primal.astype(np.longdouble)
                                + (c * primal).astype(np.longdouble),
                                dual.astype(np.longdouble) * g.astype(np.longdouble)])
        return np.cumsum(terms)[-1], primal, g, free

    def fill(x, y):
        result.primal = x * units
        result.row_dual = y * row_units
        chk = check_solution(q, rows, result.primal, result.row_dual, options.tolerance)
        result.objective = chk['objective']
        result.primal_residual = chk['primal_residual']
        result.stationarity_residual = chk['stationarity_residual']
        result.complementarity_residual = chk['complementarity_residual']
        result.dual_bound = chk['dual_bound']
        result.relative_gap = chk['relative_gap']
        result.optimality_verified = chk['verified']
        return chk['verified']

    y = np.zeros(m)
    result.status = 'iteration_limit'
    sq = val * val
    for iteration in range(min(int(options.iteration_limit), 500)):
        value, x, gradient, mask = evaluate(y)
        result.iterations = iteration
        if fill(x, y):
            result.status = 'optimal'
            return result
        if time.monotonic() - start >= options.time_limit:
            result.status = 'time_limit'
            return result
        diagonal = row_sums(rp, sq * mask[col])
        regularization = 1e-12 * (1 + _norm(diagonal))
        diagonal = diagonal + regularization
        r = gradient.copy()
        z = r / diagonal
        direction = z.copy()
        step = np.zeros(m)
        rz = dot_ld(r, z)
        gn = _norm(gradient)
        accuracy = max(1e-12, min(.01, math.sqrt(gn)) * gn)
        inner = 0
        while inner < min(10000, 4 * m + 50) and _norm(r) > accuracy:
            mv = a.mul(at.mul(direction) * mask) + regularization * direction
            den = dot_ld(direction, mv)
            if not (den > 0) or not math.isfinite(den):
                break
            alpha = rz / den
            step = step + alpha * direction
            r = r - alpha * mv
            z = r / diagonal
            nxt = dot_ld(r, z)
            beta = nxt / rz
            rz = nxt
            direction = z + beta * direction
            if inner % 100 == 0 and time.monotonic() - start >= options.time_limit:
                break
            inner += 1
        slope = dot_ld(gradient, step)
        if not (slope > 0) or not math.isfinite(slope):
            step = gradient.copy()
            slope = dot_ld(gradient, gradient)
        length = 1.0
        for _ in range(60):
            ny = y + length * step
            nv = evaluate(ny)[0]
            if (np.isfinite(nv) and nv >= value + np.longdouble(1e-4 * length * slope)
                    - np.longdouble(1e-13) * (1 + abs(value))):
                y = ny
                break
            length *= .5
        else:
            result.status = 'numerical_stall'
            return result
    return result


def validate_linear_problem(q, rows):
    """validate_linear_problem (src/mps.cpp:47-60) for a QP with linear rows: sizes and a finite
    offset, finite costs, no NaN bound, no lower bound of +inf or upper bound of -inf (variables
    and rows), and row entries with a column below n and a finite value.  ValueError with the
    reference's messages."""
    n, m = q.n, rows.m
    cost = np.asarray(q.cost, dtype=np.float64)
    lower = np.asarray(q.lower, dtype=np.float64)
    upper = np.asarray(q.upper, dtype=np.float64)
    rl = np.asarray(rows.lower, dtype=np.float64)
    ru = np.asarray(rows.upper, dtype=np.float64)
    if (not n or lower.shape != (n,) or upper.shape != (n,) or rl.shape != (m,) or ru.shape != (m,)
            or not math.isfinite(q.offset)):
        raise ValueError('Invalid linear problem dimensions or offset')
    if (not np.all(np.isfinite(cost)) or np.any(np.isnan(lower)) or np.any(np.isnan(upper))
            or np.any(lower == np.inf) or np.any(upper == -np.inf)):
        raise ValueError('Invalid variable coefficient or bound')
    if np.any(np.isnan(rl)) or np.any(np.isnan(ru)) or np.any(rl == np.inf) or np.any(ru == -np.inf):
        raise ValueError('Invalid row bound')
    col = np.asarray(rows.col)
    # the row pointers of the CSR rows (the reference keeps rows as vectors of entries, so a
    # malformed pointer array is its 'Invalid sparse row entry' too): m + 1 entries from 0 to the
    # entry count, non-decreasing
    rowptr = np.asarray(rows.rowptr)
    if (rowptr.shape != (m + 1,) or rowptr[0] != 0 or rowptr[-1] != col.shape[0]
            or np.any(np.diff(rowptr.astype(np.int64)) < 0) or np.asarray(rows.val).shape != col.shape):
        raise ValueError('Invalid sparse row entry')
    if np.any((col < 0) | (col >= n)) or not np.all(np.isfinite(np.asarray(rows.val, dtype=np.float64))):
        raise ValueError('Invalid sparse row entry')


def solve_qp_admm(q, rows, options=None, device=0, make_system=None):
    """The reference's solve_qp_admm (qp_admm.cpp:118-280) with its iterations on the GPU.

    Mirrors its option and input checks (ValueError 'Invalid QP options' / 'Continuous QP
    required'), the statuses unsupported_curvature and infeasible_bounds, the scaled set-up, the
    check of the original model every 25 iterations and at the limit (optimal once verified,
    numerical_error on a non-finite objective or stationarity, time_limit), the diagonal-equality
    pre-solver tried first (solve_diagonal_equalities, on the host as the reference runs it), the
    KKT polish at
    iterations 250, 1000 and 5000 (on the host, as the reference runs it: polish_diagonal for a
    positive diagonal Hessian, else polish_kkt, whose factorisation is SuperLU's instead of the
    reference's own LU, so its candidates agree with the reference's to rounding) and the rho
    adaptation every 100 iterations; each 25 iterations run on the device in one
    bqp_admm_iterate call.  Not mirrored: the time checks inside the inner and polish loops.  make_system(h, a, n) -> system replaces the device system (h, a: the scaled H and A
    as CSR triples; the system needs set_rho, iterate and close)."""
    from .api import QpOptions, QpResult, check_convex_hessian
    o = options or QpOptions()
    if (not math.isfinite(o.time_limit) or o.time_limit < 0 or not math.isfinite(o.tolerance) or o.tolerance <= 0
            or o.threads < 1):
        raise ValueError('Invalid QP options')
    start = time.monotonic()
    validate_linear_problem(q, rows)
    if q.integer is not None and np.any(np.asarray(q.integer)):
        raise ValueError('Continuous QP required')
    n, m = q.n, rows.m
    result = QpResult(algorithm='scaled_admm_pcg')
    if not check_convex_hessian(q):
        result.status = 'unsupported_curvature'
        return result
    if np.any(np.asarray(q.lower) > np.asarray(q.upper)) or np.any(np.asarray(rows.lower) > np.asarray(rows.upper)):
        result.status = 'infeasible_bounds'
        return result
    # the pre-solver for diagonal Hessians with equality rows, with part of the time budget
    # (qp_admm.cpp:128-133)
    small = n <= 512
    pre = solve_diagonal_equalities(q, rows, QpOptions(
        time_limit=min(2.0 if small else 10.0, (.2 if small else .5) * o.time_limit), tolerance=o.tolerance,
        iteration_limit=o.iteration_limit, threads=o.threads, scaling=o.scaling))
    if pre.status == 'optimal':
        return pre
    sp = admm_setup(q, rows, o.scaling)
    at = transpose(*sp['a'], n)
    if make_system is None:
        system = AdmmSystem(*sp['h'], *sp['a'], n, device)
    else:
        system = make_system(sp['h'], sp['a'], n)
    try:
        system.set_rho(sp['rho'], sp['sigma'])
        x, z, y = sp['x'], sp['z'], sp['y']
        rho_base = sp['rho_base']
        dual_scale = sp['row_scale'][:m] / sp['cost_scale']
        limit = int(o.iteration_limit)
        inner_total = 0
        result.status = 'iteration_limit'
        it = 0
        while True:
            result.iterations = it
            if it % 25 == 0 or it == limit:
                result.primal = x * sp['variable']
                result.row_dual = y[:m] * dual_scale
                chk = check_solution(q, rows, result.primal, result.row_dual, o.tolerance)
                result.objective = chk['objective']
                result.primal_residual = chk['primal_residual']
                result.stationarity_residual = chk['stationarity_residual']
                result.complementarity_residual = chk['complementarity_residual']
                result.dual_bound = chk['dual_bound']
                result.relative_gap = chk['relative_gap']
                result.optimality_verified = chk['verified']
                if chk['verified']:
                    result.status = 'optimal'
                    break
                if not math.isfinite(chk['objective']) or not math.isfinite(chk['stationarity_residual']):
                    result.status = 'numerical_error'
                    break
                if time.monotonic() - start >= o.time_limit:
                    result.status = 'time_limit'
                    break
                if it in (250, 1000, 5000):
                    if sp['diagonal_hessian'] and np.any((sp['lo'] == sp['up']) | (np.abs(y) > 1e-5)):
                        pol = polish_diagonal(q, rows, sp, y, o.tolerance)
                    else:
                        pol = polish_kkt(q, rows, sp, y, o.tolerance)
                    if pol is not None:
                        result.status = 'optimal'
                        result.algorithm = 'scaled_admm_pcg_kkt_polish'
                        result.primal, result.row_dual = pol['primal'], pol['row_dual']
                        result.objective = pol['objective']
                        result.primal_residual = pol['primal_residual']
                        result.stationarity_residual = pol['stationarity_residual']
                        result.complementarity_residual = pol['complementarity_residual']
                        result.dual_bound = pol['dual_bound']
                        result.relative_gap = pol['relative_gap']
                        result.optimality_verified = True
                        break
                if it and it % 100 == 0:
                    nxt = adapt_rho(sp, x, z, y, rho_base, at)
                    if nxt != rho_base:
                        rho_base = nxt
                        system.set_rho(np.where(sp['lo'] == sp['up'], rho_base * 100, rho_base * 1), sp['sigma'])
            if it == limit:
                break
            k = min(25 - it % 25, limit - it)
            x, z, y, inner = system.iterate(sp['c'], sp['lo'], sp['up'], x, z, y, it, k)
            inner_total += int(inner)
            it += k
        result.engine = {'inner_iterations': inner_total, 'rho_base': rho_base, 'seconds': time.monotonic() - start}
        return result
    finally:
        system.close()
