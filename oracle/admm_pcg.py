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
Parity unpinned: the reference exposes this inner solve only inside its ADMM loop, so there are
no golden vectors for it; the GPU solve is compared with this restatement.
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
