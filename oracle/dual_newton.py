"""CPU restatement of the reference's diagonal-Hessian equality solver (TEST INFRASTRUCTURE ONLY).

solve_qp_admm (02-software/solver/src/qp_admm.cpp:128-133) first tries
solve_diagonal_equalities (src/qp_dual_newton.cpp:9-66) on QPs whose Hessian is a positive
diagonal and whose rows are all finite equalities, and returns its answer when that verifies.
This module restates it step for step (array arithmetic in the reference's order: row sums and
long double dot products accumulate sequentially), together with the reference's checker for a
problem with linear rows (check_qp_solution, qp_admm.cpp:63-117, with original_violation,
src/mps.cpp:279-303) as plain loops.  tests/test_dual_newton_oracle.py pins both to the
reference built in oracle/_ref.
"""
import math

import numpy as np

LD = np.longdouble


def _seq_rowsums(rowptr, terms):
    """Per-row sums of CSR-ordered terms, each row summed from 0 in entry order."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    out = np.zeros(len(rowptr) - 1, dtype=terms.dtype)
    lens = np.diff(rowptr)
    for k in range(int(lens.max()) if len(lens) else 0):
        rows_k = np.flatnonzero(lens > k)
        out[rows_k] += terms[rowptr[rows_k] + k]
    return out


def multiply(csr, v):
    rowptr, col, val = csr
    return _seq_rowsums(rowptr, val * v[col])


def dot(a, b):
    """Sum of a_j b_j in long double, in order (qp_dual_newton.cpp:35)."""
    if len(a) == 0:
        return 0.0
    return float(np.cumsum(np.asarray(a, dtype=LD) * np.asarray(b, dtype=LD))[-1])


def norm(v):
    return float(np.max(np.abs(v))) if len(v) else 0.0


def merge_rows(rows, n):
    """CsrMatrix(n, rows): per row, columns ascending, duplicates summed in input order, zeros dropped."""
    rowptr, col, val = [0], [], []
    for r in rows:
        merged = {}
        for j, v in r:
            merged[j] = merged.get(j, 0.0) + v
        for j in sorted(merged):
            if merged[j] != 0:
                col.append(j)
                val.append(merged[j])
        rowptr.append(len(col))
    return np.array(rowptr, np.int64), np.array(col, np.int64), np.array(val, np.float64)


def transpose(csr, n):
    rowptr, col, val = csr
    row = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    order = np.argsort(col, kind='stable')
    tp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(col, minlength=n), out=tp[1:])
    return tp, row[order], val[order]


def check_rows(hrow, hcol, hval, cost, lower, upper, rows, row_lower, row_upper, x, row_dual, tol, maximize=False,
               offset=0.0):
    """check_qp_solution (qp_admm.cpp:63-117) for a problem with linear rows, as plain loops;
    rows is a list of [(column, value), ...] per row.  Returns the checker's fields."""
    sign = -1.0 if maximize else 1.0
    n, m = len(cost), len(rows)
    out = {'objective': math.nan, 'primal_residual': math.inf, 'stationarity_residual': math.inf,
           'complementarity_residual': math.inf, 'dual_bound': -math.inf, 'relative_gap': math.inf,
           'verified': False}
    x = [float(v) for v in x]
    y = [float(v) for v in row_dual]
    if len(x) != n or len(y) != m or not all(math.isfinite(v) for v in x) or not all(math.isfinite(v) for v in y):
        return out
    gradient = [0.0] * n
    value = LD(sign * offset)
    positive_diagonal = True
    for i, j, v in zip(hrow, hcol, hval):
        gradient[i] += sign * v * x[j]
        if i != j:
            gradient[j] += sign * v * x[i]
            if v != 0:
                positive_diagonal = False
    diagonal = linear = None
    if positive_diagonal:
        diagonal = [LD(0)] * n
        for i, j, v in zip(hrow, hcol, hval):
            if i == j:
                diagonal[i] += sign * v
        positive_diagonal = all(d > 0 for d in diagonal)
        if positive_diagonal:
            linear = [LD(sign * c) for c in cost]
    for j in range(n):
        value += LD(0.5) * LD(x[j]) * LD(gradient[j]) + LD(sign * cost[j] * x[j])
        gradient[j] += sign * cost[j]
    out['objective'] = sign * float(value)
    out['primal_residual'] = _violation(lower, upper, rows, row_lower, row_upper, x)
    complementarity = 0.0
    bound = value
    dual_constant = LD(sign * offset)
    for i in range(m):
        activity = LD(0)
        for j, a in rows[i]:
            activity += LD(a) * LD(x[j])
            gradient[j] += a * y[i]
            if positive_diagonal:
                linear[j] += LD(a) * LD(y[i])
        target = row_upper[i] if y[i] >= 0 else row_lower[i]
        if y[i] != 0:
            dual_constant -= LD(y[i]) * LD(target)
            correction = LD(y[i]) * (activity - LD(target))
            bound += correction
            residual = float(abs(correction) / (1 + abs(value)))
            if not math.isfinite(residual):
                residual = math.inf
            complementarity = max(complementarity, residual)
    out['complementarity_residual'] = complementarity
    stationarity = 0.0
    for j in range(n):
        g = gradient[j]
        clipped = max(lower[j], min(upper[j], x[j] - g))
        residual = abs(x[j] - clipped) / (1 + abs(x[j]))
        if not math.isfinite(g) or not math.isfinite(residual):
            residual = math.inf
        stationarity = max(stationarity, residual)
        if g != 0:
            target = lower[j] if g > 0 else upper[j]
            if math.isfinite(target):
                bound += LD(g * (target - x[j]))
            else:
                bound = LD(-np.inf)
    out['stationarity_residual'] = stationarity
    if positive_diagonal:
        bound = dual_constant
        for j in range(n):
            mn = max(LD(lower[j]), min(LD(upper[j]), -linear[j] / diagonal[j]))
            bound += LD(0.5) * diagonal[j] * mn * mn + linear[j] * mn
    out['dual_bound'] = float(bound)
    out['relative_gap'] = float(abs(value - bound) / (1 + abs(value))) if np.isfinite(bound) else math.inf
    verified = math.isfinite(out['objective']) and max(out['primal_residual'], stationarity, complementarity) <= tol
    if positive_diagonal:
        verified = verified and out['relative_gap'] <= tol
    out['verified'] = verified
    return out


def _violation(lower, upper, rows, row_lower, row_upper, x):
    """original_violation(p, x, true) (src/mps.cpp:279-303)."""
    result = 0.0

    def check(activity, bound, is_lower, scale):
        nonlocal result
        if not math.isfinite(bound):
            return
        v = (LD(bound) - activity) if is_lower else (activity - LD(bound))
        v /= LD(1 + abs(bound)) + scale
        result = max(result, float(v))

    for j in range(len(x)):
        if not math.isfinite(x[j]):
            return math.inf
        check(LD(x[j]), lower[j], True, LD(abs(x[j])))
        check(LD(x[j]), upper[j], False, LD(abs(x[j])))
    for i, r in enumerate(rows):
        activity = LD(0)
        scale = LD(0)
        for j, a in r:
            term = LD(a) * LD(x[j])
            activity += term
            scale += abs(term)
        if not np.isfinite(activity):
            return math.inf
        check(activity, row_lower[i], True, scale)
        check(activity, row_upper[i], False, scale)
    return result


def solve_diagonal_equalities_restated(hrow, hcol, hval, cost, lower, upper, rows, row_lower, row_upper, tol=1e-7,
                                       iteration_limit=200000, scaling=True):
    """solve_diagonal_equalities (qp_dual_newton.cpp:9-66) for a minimisation: rows is a list of
    [(column, value), ...] per row.  Returns (status, iterations, x, row_dual, check fields)."""
    n, m = len(cost), len(rows)
    if not m:
        return 'unsupported_structure', 0, None, None, None
    if any(row_lower[i] != row_upper[i] or not math.isfinite(row_lower[i]) for i in range(m)):
        return 'unsupported_structure', 0, None, None, None
    h = np.zeros(n)
    for i, j, v in zip(hrow, hcol, hval):
        if i != j and v != 0:
            return 'unsupported_structure', 0, None, None, None
        h[i] += v
    if np.any(~(h > 0)) or not np.all(np.isfinite(h)):
        return 'unsupported_structure', 0, None, None, None
    units = 1 / np.sqrt(h)
    lo = np.asarray(lower, dtype=np.float64) / units
    up = np.asarray(upper, dtype=np.float64) / units
    c = np.asarray(cost, dtype=np.float64) * units
    srows, row_units, b = [], np.zeros(m), np.zeros(m)
    for i in range(m):
        r = [(j, v * units[j]) for j, v in rows[i]]
        maximum = 0.0
        for _, v in r:
            maximum = max(maximum, abs(v))
        row_units[i] = 1 / maximum if maximum else 1.0
        srows.append([(j, v * row_units[i]) for j, v in r])
        b[i] = row_lower[i] * row_units[i]
    magnitude = 1.0
    if scaling:
        for j in range(n):
            magnitude = max(magnitude, abs(c[j]))
            magnitude = max(magnitude, abs(max(lo[j], min(up[j], 0.0))))
        for rhs in b:
            magnitude = max(magnitude, abs(rhs))
    units = units * magnitude
    lo, up, c = lo / magnitude, up / magnitude, c / magnitude
    b = b / magnitude
    row_units = row_units * magnitude
    if (not np.all(np.isfinite(units)) or not np.all(np.isfinite(c)) or np.any(np.isnan(lo)) or np.any(np.isnan(up))
            or not np.all(np.isfinite(b)) or not np.all(np.isfinite(row_units))):
        return 'numerical_scaling_failure', 0, None, None, None
    a = merge_rows(srows, n)
    at = transpose(a, n)

    def evaluate(dual):
        primal = multiply(at, dual)
        raw = -(primal + c)
        free = ((raw >= lo) & (raw <= up)).astype(np.float64)
        primal = np.maximum(lo, np.minimum(up, raw))
        terms = LD(0.5) * primal.astype(LD) * primal.astype(LD) + (c * primal).astype(LD)
        g = multiply(a, primal) - b
        value = np.cumsum(np.concatenate([[LD(0)], terms, dual.astype(LD) * g.astype(LD)]))[-1]
        return value, primal, g, free

    y = np.zeros(m)
    status = 'iteration_limit'
    iterations = 0
    x_out = y_out = chk = None
    for iteration in range(min(iteration_limit, 500)):
        value, x, gradient, mask = evaluate(y)
        iterations = iteration
        x_out = x * units
        y_out = y * row_units
        chk = check_rows(hrow, hcol, hval, cost, lower, upper, rows, row_lower, row_upper, x_out, y_out, tol)
        if chk['verified']:
            return 'optimal', iterations, x_out, y_out, chk
        diagonal = np.zeros(m)
        for i in range(m):
            for j, v in srows[i]:
                diagonal[i] += v * v * mask[j]
        regularization = 1e-12 * (1 + norm(diagonal))
        diagonal = diagonal + regularization
        r = gradient.copy()
        z = r / diagonal
        direction = z.copy()
        step = np.zeros(m)
        rz = dot(r, z)
        accuracy = max(1e-12, min(.01, math.sqrt(norm(gradient))) * norm(gradient))
        inner = 0
        while inner < min(10000, 4 * m + 50) and norm(r) > accuracy:
            work = multiply(at, direction) * mask
            mv = multiply(a, work) + regularization * direction
            den = dot(direction, mv)
            if not (den > 0) or not math.isfinite(den):
                break
            alpha = rz / den
            step = step + alpha * direction
            r = r - alpha * mv
            z = r / diagonal
            nxt = dot(r, z)
            beta = nxt / rz
            rz = nxt
            direction = z + beta * direction
            inner += 1
        slope = dot(gradient, step)
        if not (slope > 0) or not math.isfinite(slope):
            step = gradient.copy()
            slope = dot(gradient, gradient)
        length = 1.0
        accepted = False
        for _ in range(60):
            ny = y + length * step
            nv, _, _, _ = evaluate(ny)
            if np.isfinite(nv) and nv >= value + LD(1e-4 * length * slope) - LD(1e-13 * (1 + abs(value))):
                y = ny
                accepted = True
                break
            length *= .5
        if not accepted:
            return 'numerical_stall', iterations, x_out, y_out, chk
    return status, iterations, x_out, y_out, chk
