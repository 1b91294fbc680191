"""QPLIB reader for the box-QP path.

Restates read_qplib (02-software/solver/src/qp.cpp:67-117): whitespace tokens with '#' comments,
name / type / sense, n (and m for linear constraints), one-based lower-triangle Hessian entries
(an off-diagonal entry contributes half its listed value to each side of the symmetric Hessian,
src/qp.cpp:82-84), the cost vector as default + sparse entries, the offset, the constraint matrix
and row bounds when present, the infinity marker, the variable bounds, the three start vectors
(parsed and ignored, src/qp.cpp:100-101) and the name sections.  The same validation errors are
raised (as ValueError).  The reference caps counts at 100,000 variables / rows and 5,000,000
entries (src/qp.cpp:33,75); `max_columns` keeps that default and can be raised.
"""
import math

import numpy as np

from .api import QuadraticProblem


class _Tokens:
    def __init__(self, text):
        self.lines = iter(text.splitlines())
        self.pending = []
        self.at = 0

    def token(self):
        while self.at == len(self.pending):
            try:
                line = next(self.lines)
            except StopIteration:
                raise ValueError('Truncated QPLIB input')
            line = line.split('#', 1)[0]
            self.pending = line.split()
            self.at = 0
        t = self.pending[self.at]
        self.at += 1
        return t

    def number(self):
        # The reference parses long double: decimal literals beyond the double range (an infinity
        # marker such as 1e+400) are finite there; here they become +-inf, which the bound
        # conversion maps to infinity exactly as the reference does.  'inf'/'nan' text is rejected.
        t = self.token()
        try:
            x = float(t)
        except ValueError:
            raise ValueError('Invalid QPLIB number')
        if math.isnan(x) or (math.isinf(x) and any(c.isalpha() and c not in 'eE' for c in t)):
            raise ValueError('Invalid QPLIB number')
        return x

    def count(self, maximum=5000000):
        v = self.number()
        if v < 0 or v > maximum or math.floor(v) != v:
            raise ValueError('Invalid or oversized QPLIB count')
        return int(v)

    def index(self, n):
        i = self.count(n)
        if i == 0:
            raise ValueError('QPLIB indices are one-based')
        return i - 1

    def vector(self, n, infinity=math.inf):
        def convert(v):
            if abs(v) >= infinity:
                return -math.inf if v < 0 else math.inf
            return v
        default = convert(self.number())
        out = np.full(n, default, dtype=np.float64)
        entries = self.count(n)
        seen = set()
        for _ in range(entries):
            j = self.index(n)
            if j in seen:
                raise ValueError('Duplicate QPLIB vector entry')
            seen.add(j)
            out[j] = convert(self.number())
        return out


def read_qplib(text, max_columns=100000):
    """Parses QPLIB text; returns (QuadraticProblem, rows) where rows > 0 means linear constraints."""
    q, m, _ = _parse(text, max_columns)
    return q, m


def read_qplib_rows(text, max_columns=100000):
    """Parses QPLIB text with its linear constraints; returns (QuadraticProblem, LinearRows), the
    rows in CSR with each row's entries in file order (the reference appends them to its row
    vectors as it reads them, src/qp.cpp:88-94) and the row bounds; LinearRows with no rows for
    a box or unconstrained model."""
    from .admm import LinearRows
    q, m, (ri, rj, rv, row_lower, row_upper) = _parse(text, max_columns)
    ri = np.asarray(ri, dtype=np.int64)
    order = np.argsort(ri, kind='stable')
    rowptr = np.zeros(m + 1, dtype=np.int32)
    if m:
        np.cumsum(np.bincount(ri, minlength=m), out=rowptr[1:])
    return q, LinearRows(rowptr, np.asarray(rj, dtype=np.int32)[order], np.asarray(rv, dtype=np.float64)[order],
                         np.asarray(row_lower, dtype=np.float64), np.asarray(row_upper, dtype=np.float64))


def _parse(text, max_columns):
    r = _Tokens(text)
    r.token()  # name
    typ, sense = r.token(), r.token()
    if len(typ) != 3 or typ[1] != 'C' or typ[0] not in 'CDQ' or typ[2] not in 'NBL':
        raise ValueError('unsupported_qplib_type: continuous quadratic objective with linear/box constraints required')
    if sense not in ('minimize', 'maximize'):
        raise ValueError('Invalid QPLIB objective sense')
    n = r.count(max_columns)
    if n == 0:
        raise ValueError('Empty QPLIB model')
    m = r.count(max_columns) if typ[2] == 'L' else 0
    nz = r.count()
    hrow, hcol, hval, seen = [], [], [], set()
    for _ in range(nz):
        i, j, v = r.index(n), r.index(n), r.number()
        if i < j or (i, j) in seen or not math.isfinite(v):
            raise ValueError('Invalid QPLIB Hessian entry')
        seen.add((i, j))
        hrow.append(i)
        hcol.append(j)
        hval.append(v if i == j else 0.5 * v)
    cost = r.vector(n)
    offset = r.number()
    ri, rj, rv = [], [], []
    row_lower = row_upper = np.zeros(0)
    if m:
        cnt = r.count()
        entries = set()
        for _ in range(cnt):
            i, j, v = r.index(m), r.index(n), r.number()
            if (i, j) in entries or not math.isfinite(v):
                raise ValueError('Invalid QPLIB matrix entry')
            entries.add((i, j))
            ri.append(i)
            rj.append(j)
            rv.append(v)
    infinity = r.number()
    if infinity <= 0:
        raise ValueError('Invalid infinity marker')
    if m:
        row_lower = r.vector(m, infinity)
        row_upper = r.vector(m, infinity)
    if typ[2] != 'N':
        lower, upper = r.vector(n, infinity), r.vector(n, infinity)
    else:
        lower, upper = np.full(n, -np.inf), np.full(n, np.inf)
    r.vector(n)
    if m:
        r.vector(m)
    r.vector(n)
    names = r.count(n)
    named = set()
    for _ in range(names):
        j = r.index(n)
        if j in named:
            raise ValueError('Duplicate variable name entry')
        named.add(j)
        r.token()
    names = r.count(m)
    named = set()
    for _ in range(names):
        i = r.index(m)
        if i in named:
            raise ValueError('Duplicate row name entry')
        named.add(i)
        r.token()
    if r.at < len(r.pending):
        raise ValueError('Unexpected trailing QPLIB tokens')
    for line in r.lines:
        if line.split('#', 1)[0].strip():
            raise ValueError('Unexpected trailing QPLIB content')
    q = QuadraticProblem(cost=cost, lower=lower, upper=upper, hessian_row=np.asarray(hrow, np.int64),
                         hessian_col=np.asarray(hcol, np.int64), hessian_val=np.asarray(hval, np.float64),
                         offset=offset, maximize=sense == 'maximize', rows=m)
    return q, m, (ri, rj, rv, row_lower, row_upper)


def write_qplib(path, q: QuadraticProblem, name='GENERATED'):
    """Writes a box QP in QPLIB text (type QCB); the inverse of read_qplib for box problems."""
    n = q.n
    lines = [name, 'QCB', 'maximize' if q.maximize else 'minimize', str(n)]
    hr, hc, hv = np.asarray(q.hessian_row), np.asarray(q.hessian_col), np.asarray(q.hessian_val)
    lines.append(str(len(hr)))
    for i, j, v in zip(hr, hc, hv):
        lines.append(f'{i + 1} {j + 1} {(v if i == j else 2 * v):.17g}')

    def vec(values, inf=1e20):
        vals = [(-inf if v == -math.inf else inf if v == math.inf else v) for v in values]
        out = ['0', str(len(vals))]
        out += [f'{k + 1} {v:.17g}' for k, v in enumerate(vals)]
        return out
    lines += vec(q.cost) + [f'{q.offset:.17g}', '1e20'] + vec(q.lower) + vec(q.upper)
    lines += ['0', '0', '0', '0', '0', '0']  # start vectors x0, z0 (defaults, no entries); no names
    with open(path, 'w') as f:
        f.write('\n'.join(lines) + '\n')
