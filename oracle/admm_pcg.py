"""CPU restatement of the reference's ADMM inner solve (TEST INFRASTRUCTURE ONLY).

Follows 02-software/solver/src/qp_admm.cpp:
  * preconditioner (qp_admm.cpp:153-156): diag(H) + sigma, then rho_i a_ij^2 added over the rows
    i of A in order and their entries in order;
  * system (qp_admm.cpp:157-161): out = H v; t = A v; t_i *= rho_i; product = A' t;
    out_j += sigma v_j + product_j;
  * inner CG (qp_admm.cpp:262-273): r = rhs - K x, pre = r / M, d = pre, rz = dot(r, pre); while
    inner < max_inner and max|r| > accuracy: kd = K d, den = dot(d, kd) (stop unless positive and
    finite), alpha = rz / den, x += alpha d, r -= alpha kd, pre = r / M, beta = dot(r, pre) / rz,
    d = pre + beta d;
  * dot (qp_admm.cpp:23) accumulates in long double, norm (qp_admm.cpp:22) is max |.|.
solve_qp_admm_restated restates the whole ADMM loop around it (qp_admm.cpp:136-280, with the rho
adaptation every 100 iterations, below the first polish at iteration 250); it reproduces the
reference's solve_qp_admm primal bit for bit (tests/golden/reference_admm.npz, generated from the
reference itself), which pins the inner solve restatement too.
"""
import numpy as np


def csr_matvec(rowptr, col, val, v):
    """Row sums in entry order (the reference's CsrMatrix::multiply)."""
    out = np.zeros(len(rowptr) - 1)
    for i in range(len(rowptr) - 1):
        s = 0.0
        for k in range(rowptr[i], rowptr[i + 1]):
            s += val[k] * v[col[k]]
        out[i] = s
    return out


def transpose(rowptr, col, val, n):
    """A' by a stable counting sort (rows of A' list the rows of A in increasing order)."""
    m = len(rowptr) - 1
    cnt = np.zeros(n + 1, dtype=np.int64)
    for k in range(rowptr[m]):
        cnt[col[k] + 1] += 1
    trp = np.cumsum(cnt)
    nxt = trp[:-1].copy()
    tci = np.zeros(rowptr[m], dtype=np.int32)
    tva = np.zeros(rowptr[m])
    for i in range(m):
        for k in range(rowptr[i], rowptr[i + 1]):
            p = nxt[col[k]]
            nxt[col[k]] += 1
            tci[p] = i
            tva[p] = val[k]
    return trp.astype(np.int32), tci, tva


def dot(a, b):
    s = np.longdouble(0)
    for x, y in zip(a, b):
        s += np.longdouble(x) * np.longdouble(y)
    return float(s)


class AdmmSystemOracle:
    def __init__(self, h, a, n):
        self.h = h            # (rowptr, col, val)
        self.a = a
        self.n = n
        self.at = transpose(*a, n)

    def set_rho(self, rho, sigma):
        self.rho = np.asarray(rho, dtype=np.float64)
        self.sigma = float(sigma)
        hrp, hci, hva = self.h
        diag = np.zeros(self.n)
        for i in range(self.n):
            for k in range(hrp[i], hrp[i + 1]):
                if hci[k] == i:
                    diag[i] = hva[k]
        pre = diag + self.sigma
        arp, aci, ava = self.a
        for i in range(len(arp) - 1):
            for k in range(arp[i], arp[i + 1]):
                pre[aci[k]] += self.rho[i] * ava[k] * ava[k]
        self.precond = pre

    def apply(self, v):
        out = csr_matvec(*self.h, v)
        t = csr_matvec(*self.a, v) * self.rho
        product = csr_matvec(*self.at, t)
        return out + (self.sigma * v + product)

    def solve(self, rhs, x0, accuracy, max_inner):
        x = np.array(x0, dtype=np.float64, copy=True)
        r = rhs - self.apply(x)
        pre = r / self.precond
        d = pre.copy()
        rz = dot(r, pre)
        inner = 0
        while inner < max_inner and np.max(np.abs(r)) > accuracy:
            kd = self.apply(d)
            den = dot(d, kd)
            if not (den > 0) or not np.isfinite(den):
                break
            alpha = rz / den
            x = x + alpha * d
            r = r - alpha * kd
            pre = r / self.precond
            nrz = dot(r, pre)
            beta = nrz / rz
            rz = nrz
            d = pre + beta * d
            inner += 1
        return x, inner, float(np.max(np.abs(r))) if len(r) else 0.0


def _csr_from_rows(rows, n_cols):
    """CsrMatrix(n, rows) of the reference (sparse_matrix.hpp:10-17): per row, columns merged in a
    std::map (ascending, duplicates summed in input order), zeros dropped."""
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
    return np.array(rowptr, np.int32), np.array(col, np.int32), np.array(val, np.float64)


def _clip(x, lo, up):
    # std::max(lo, std::min(up, x)) elementwise
    t = np.where(x < up, x, up)
    return np.where(lo < t, t, lo)


def scale_qp_admm(n, hrow, hcol, hval, cost, lower, upper, a_rowptr, a_col, a_val, row_lower, row_upper,
                  scaling=True, maximize=False):
    """The reference's set-up of solve_qp_admm (qp_admm.cpp:136-161): variable units, row scales
    and the cost scale; A with the bound rows appended; the initial x and z and rho (0.1, x100 on
    equality rows), sigma 1e-8 (a maximisation negates the Hessian and the cost first).  Returns a
    dict of the scaled problem."""
    m = len(a_rowptr) - 1
    sign = -1.0 if maximize else 1.0
    # hessian(q) (qp_admm.cpp:24-29): lower-triangle terms (sign-normalised) mirrored, merged per row
    hrows = [[] for _ in range(n)]
    for i, j, v in zip(hrow, hcol, hval):
        hrows[i].append((j, sign * v))
        if i != j:
            hrows[j].append((i, sign * v))
    hrp, hci, hva = _csr_from_rows(hrows, n)
    hva = hva.copy()
    variable = np.ones(n)
    diagonal = np.zeros(n)
    for i in range(n):
        for k in range(hrp[i], hrp[i + 1]):
            if hci[k] == i:
                diagonal[i] = hva[k]
    if scaling:
        for j in range(n):
            if diagonal[j] > 0:
                variable[j] = 1 / np.sqrt(max(1e-16, diagonal[j]))
    for i in range(n):
        for k in range(hrp[i], hrp[i + 1]):
            hva[k] *= variable[i] * variable[hci[k]]
    rows = []
    lo_all, up_all = [], []
    row_scale = np.ones(m + n)
    for i in range(m):
        r = [(int(a_col[k]), float(a_val[k])) for k in range(a_rowptr[i], a_rowptr[i + 1])]
        maximum = 0.0
        r2 = []
        for j, v in r:
            v = v * variable[j]
            maximum = max(maximum, abs(v))
            r2.append((j, v))
        if scaling and maximum > 0:
            row_scale[i] = 1 / maximum
        rows.append([(j, v * row_scale[i]) for j, v in r2])
        lo_all.append(row_lower[i] * row_scale[i])
        up_all.append(row_upper[i] * row_scale[i])
    for j in range(n):
        rows.append([(j, 1.0)])
        lo_all.append(lower[j] / variable[j])
        up_all.append(upper[j] / variable[j])
    c = np.array(cost, dtype=np.float64) * (sign * variable)
    cost_scale = 1 / max(1.0, float(np.max(np.abs(c)))) if scaling else 1.0
    hva = hva * cost_scale
    c = c * cost_scale
    rows_input = rows
    arp, aci, ava = _csr_from_rows(rows, n)
    lo_all = np.array(lo_all)
    up_all = np.array(up_all)
    rho = np.where(lo_all == up_all, 0.1 * 100, 0.1 * 1)
    x = _clip(np.zeros(n), lo_all[m:], up_all[m:])
    z = _clip(csr_matvec(arp, aci, ava, x), lo_all, up_all)
    return {'h': (hrp, hci, hva), 'a': (arp, aci, ava), 'c': c, 'lo': lo_all, 'up': up_all, 'rho': rho,
            'sigma': 1e-8, 'variable': variable, 'row_scale': row_scale, 'cost_scale': cost_scale, 'x': x, 'z': z,
            'y': np.zeros(m + n), 'rows_input': rows_input}


def adapt_rho(sp, system, x, z, y, rho_base):
    """The reference's rho adaptation (qp_admm.cpp:265-271), run at every 100th iteration: scaled
    primal residual max|Ax - z| / (1 + max(|Ax|, |z|)) and dual residual max|Hx + c + A'y| /
    (1 + max(|c|, |Hx|, |A'y|)) (max norms); the candidate rho_base sqrt(primal / dual), both
    floored at 1e-16 and the result clamped to [1e-6, 1e6], replaces rho_base only when it leaves
    [rho_base / 5, 5 rho_base].  Returns the (possibly unchanged) rho_base."""
    ax = csr_matvec(*sp['a'], x)
    hx = csr_matvec(*sp['h'], x)
    aty = csr_matvec(*system.at, y)

    def norm(v):
        return float(np.max(np.abs(v))) if len(v) else 0.0

    primal = norm(ax - z)
    dual = norm(hx + sp['c'] + aty)
    primal /= 1 + max(norm(ax), norm(z))
    dual /= 1 + max(norm(sp['c']), max(norm(hx), norm(aty)))
    nxt = max(1e-6, min(1e6, rho_base * np.sqrt(max(1e-16, primal) / max(1e-16, dual))))
    return nxt if (nxt > 5 * rho_base or nxt < rho_base / 5) else rho_base


def solve_qp_admm_restated(n, hrow, hcol, hval, cost, lower, upper, a_rowptr, a_col, a_val, row_lower, row_upper,
                           iteration_limit, scaling=True, inner=None, info=None):
    """The reference's solve_qp_admm (qp_admm.cpp:136-280) for a minimisation with inequality rows,
    up to an iteration limit below its first polish (250), where no check before the limit
    verifies: returns the primal after `iteration_limit` ADMM iterations (the reference's
    result.primal, x times the variable units).  The rho adaptation runs at iterations 100 and 200
    (adapt_rho); a changed rho_base re-forms rho and the preconditioner (the reference's setup()).

    inner(system, rhs, x0, accuracy, max_inner) -> x replaces the restated inner CG when given
    (system: the scaled H and A as CSR triples, rho, sigma); it is how a GPU inner solve is run
    inside the restated loop.  info, a dict, receives 'rho_base': the rho_base after each
    adaptation."""
    assert iteration_limit < 250
    sp = scale_qp_admm(n, hrow, hcol, hval, cost, lower, upper, a_rowptr, a_col, a_val, row_lower, row_upper,
                       scaling)
    (hrp, hci, hva), (arp, aci, ava) = sp['h'], sp['a']
    c, lo_all, up_all, rho, sigma = sp['c'], sp['lo'], sp['up'], sp['rho'], sp['sigma']
    sys_ = AdmmSystemOracle((hrp, hci, hva), (arp, aci, ava), n)
    sys_.set_rho(rho, sigma)
    x, z, y = sp['x'], sp['z'], sp['y']
    rho_base = 0.1
    for iteration in range(iteration_limit):
        if iteration and iteration % 100 == 0:
            nxt = adapt_rho(sp, sys_, x, z, y, rho_base)
            if info is not None:
                info.setdefault('rho_base', []).append(nxt)
            if nxt != rho_base:
                rho_base = nxt
                rho = np.where(lo_all == up_all, rho_base * 100, rho_base * 1)
                sys_.set_rho(rho, sigma)
        solve = None
        if inner is not None:
            def solve(rhs, x0, accuracy, max_inner, rho=rho):
                return inner(((hrp, hci, hva), (arp, aci, ava), rho, sigma), rhs, x0, accuracy, max_inner), 0
        x, z, y, _ = admm_iteration(sys_, c, lo_all, up_all, x, z, y, iteration, solve)
    return x * sp['variable']


def admm_iteration(system, c, lo, up, x, z, y, iteration, solve=None):
    """One iteration of the reference's ADMM loop (qp_admm.cpp:255-279) on the scaled problem, with
    system's rho and sigma (AdmmSystemOracle after set_rho): rhs = A'(rho z - y) + (sigma x - c),
    the inner accuracy min(1e-7, 0.05 / (iteration + 1)^1.6) (1 + max|rhs|) and limit
    min(4000, 2n + 20), the inner PCG from x, then the relaxed (1.6) z and y updates and
    x = 1.6 next - 0.6 x.  solve(rhs, x0, accuracy, max_inner) -> (next, inner) replaces the
    restated PCG when given.  Returns (x, z, y, inner iterations)."""
    rho, sigma = system.rho, system.sigma
    n = system.n
    yz = rho * z - y
    rhs = csr_matvec(*system.at, yz)
    rhs = rhs + (sigma * x - c)
    accuracy = min(1e-7, .05 / (iteration + 1) ** 1.6) * (1 + float(np.max(np.abs(rhs))))
    max_inner = min(4000, 2 * n + 20)
    if solve is None:
        nxt, inner, _ = system.solve(rhs, x, accuracy, max_inner)
    else:
        nxt, inner = solve(rhs, x, accuracy, max_inner)
    ax = csr_matvec(*system.a, nxt)
    relaxed = 1.6 * ax - .6 * z
    nz = _clip(relaxed + y / rho, lo, up)
    y = y + rho * (relaxed - nz)
    return 1.6 * nxt - .6 * x, nz, y, inner


def solve_qp_admm_full_restated(n, hrow, hcol, hval, cost, lower, upper, a_rowptr, a_col, a_val, row_lower,
                                row_upper, tol, iteration_limit=200000, scaling=True):
    """The reference's whole solve_qp_admm (qp_admm.cpp:118-280) for a minimisation whose Hessian is
    diagonal, rows not all equalities (so its dual Newton pre-solver declines): the checks of the
    original model every 25 iterations (oracle.dual_newton.check_rows), the rho adaptation every
    100, and the KKT polish at iterations 250, 1000 and 5000 in its diagonal-Hessian form
    (qp_admm.cpp:165-205: active rows from |y| > 1e-5 or equal bounds, CG on K D^-1 K' for the
    row multipliers, x = -(K' lambda + c) / D, accepted when the original model verifies).
    Returns (status, iterations, primal, row_dual, check fields, polished)."""
    from oracle.dual_newton import check_rows
    m = len(a_rowptr) - 1
    sp = scale_qp_admm(n, hrow, hcol, hval, cost, lower, upper, a_rowptr, a_col, a_val, row_lower, row_upper,
                       scaling)
    (hrp, hci, hva), (arp, aci, ava) = sp['h'], sp['a']
    diag = np.zeros(n)
    offdiag = False
    for i in range(n):
        for k in range(hrp[i], hrp[i + 1]):
            if hci[k] == i:
                diag[i] = hva[k]
            else:
                offdiag = True
    assert not offdiag and np.all(diag > 0), 'the restated polish covers positive diagonal Hessians only'
    orig_rows = [[(int(a_col[k]), float(a_val[k])) for k in range(a_rowptr[i], a_rowptr[i + 1])] for i in range(m)]
    c, lo_all, up_all, rho, sigma = sp['c'], sp['lo'], sp['up'], sp['rho'], sp['sigma']
    sys_ = AdmmSystemOracle((hrp, hci, hva), (arp, aci, ava), n)
    sys_.set_rho(rho, sigma)
    x, z, y = sp['x'], sp['z'], sp['y']
    variable, row_scale, cost_scale = sp['variable'], sp['row_scale'], sp['cost_scale']
    rows_in = sp['rows_input']

    def check(px, py):
        return check_rows(hrow, hcol, hval, cost, lower, upper, orig_rows, row_lower, row_upper, px, py, tol)

    def polish():
        active = [i for i in range(m + n) if lo_all[i] == up_all[i] or abs(y[i]) > 1e-5]
        if n + len(active) > 10000:
            return None
        assert active, 'with no active row the reference polishes by its sparse LU, not restated'
        target = []
        for i in active:
            t = lo_all[i] if lo_all[i] == up_all[i] else (up_all[i] if y[i] > 0 else lo_all[i])
            if not np.isfinite(t):
                return None
            target.append(t)
        k = _csr_from_rows([rows_in[i] for i in active], n)
        kt = transpose(*k, n)
        rhs = csr_matvec(*k, c / diag)
        ds = np.full(len(active), 1e-18)
        for r, i in enumerate(active):
            rhs[r] = -rhs[r] - target[r]
            for j, v in rows_in[i]:
                ds[r] += v * v / diag[j]
        residual = rhs.copy()
        zp = residual / ds
        direction = zp.copy()
        lam = np.zeros(len(active))
        rz = dot(residual, zp)
        stop = 1e-13 * (1 + float(np.max(np.abs(rhs))))
        inner = 0
        while inner < 20000 and float(np.max(np.abs(residual))) > stop:
            work = csr_matvec(*kt, direction) / diag
            mv = csr_matvec(*k, work)
            den = dot(direction, mv)
            if not (den > 0) or not np.isfinite(den):
                break
            alpha = rz / den
            lam = lam + alpha * direction
            residual = residual - alpha * mv
            zp = residual / ds
            nxt = dot(residual, zp)
            beta = nxt / rz
            rz = nxt
            direction = zp + beta * direction
            inner += 1
        work = -(csr_matvec(*kt, lam) + c) / diag
        px = work * variable
        py = np.zeros(m)
        for r, i in enumerate(active):
            if i < m:
                py[i] = lam[r] * row_scale[i] / cost_scale
        chk = check(px, py)
        return (px, py, chk) if chk['verified'] else None

    rho_base = 0.1
    status = 'iteration_limit'
    result = None
    for iteration in range(iteration_limit + 1):
        if iteration % 25 == 0 or iteration == iteration_limit:
            px = x * variable
            py = y[:m] * (row_scale[:m] / cost_scale)
            chk = check(px, py)
            result = (px, py, chk)
            if chk['verified']:
                return 'optimal', iteration, px, py, chk, False
            if not np.isfinite(chk['objective']) or not np.isfinite(chk['stationarity_residual']):
                return 'numerical_error', iteration, px, py, chk, False
            if iteration in (250, 1000, 5000):
                pol = polish()
                if pol is not None:
                    return ('optimal', iteration) + pol + (True,)
            if iteration and iteration % 100 == 0:
                nxt = adapt_rho(sp, sys_, x, z, y, rho_base)
                if nxt != rho_base:
                    rho_base = nxt
                    rho = np.where(lo_all == up_all, rho_base * 100, rho_base * 1)
                    sys_.set_rho(rho, sigma)
        if iteration == iteration_limit:
            break
        x, z, y, _ = admm_iteration(sys_, c, lo_all, up_all, x, z, y, iteration)
    return (status, iteration_limit) + result + (False,)
