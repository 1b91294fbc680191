"""Rebuilds the inputs of the golden fixtures (tests/golden/reference_cases.json)."""
import numpy as np

import boxqp


def inputs(rec):
    """Returns (problem dict with hrow/hcol/hval/cost/lower/upper, planted instance or None)."""
    if 'problem' in rec:
        p = {k: np.asarray(v) for k, v in rec['problem'].items()}
        p['hrow'] = p['hrow'].astype(np.int64)
        p['hcol'] = p['hcol'].astype(np.int64)
        return p, None
    g = rec['generator']
    inst = boxqp.planted(g['preset'], seed=g.get('seed', 1), index=g.get('index', 0), n=g.get('n', 0),
                         lower_triplets=True)
    p = {'hrow': inst['hrow'], 'hcol': inst['hcol'], 'hval': inst['hval'], 'cost': inst['c'],
         'lower': inst['lower'], 'upper': inst['upper']}
    if g.get('open_bounds'):
        # one-sided boxes: no lower bound where j % k == 0, no upper bound where j % k == 1
        k = int(g['open_bounds'])
        j = np.arange(len(p['lower']))
        p['lower'] = np.where(j % k == 0, -np.inf, p['lower'])
        p['upper'] = np.where(j % k == 1, np.inf, p['upper'])
        inst = dict(inst, lower=p['lower'], upper=p['upper'])
    if g.get('zero_rows_every'):
        # Hessian rows and columns of every k-th variable removed: those variables are linear only
        k = int(g['zero_rows_every'])
        keep = (p['hrow'] % k != 0) & (p['hcol'] % k != 0)
        p['hrow'], p['hcol'], p['hval'] = p['hrow'][keep], p['hcol'][keep], p['hval'][keep]
        csr = boxqp.csr_from_lower(len(p['cost']), p['hrow'], p['hcol'], p['hval'], 1.0)
        inst = dict(inst, rowptr=csr[0], col=csr[1], val=csr[2], hrow=p['hrow'], hcol=p['hcol'], hval=p['hval'],
                    nnz=len(csr[1]))
    if g.get('fixed_every'):
        # fixed variables: l = u = the planted optimum where j % k == 0 (the optimum is unchanged)
        k = int(g['fixed_every'])
        fix = np.arange(len(p['lower'])) % k == 0
        p['lower'] = np.where(fix, inst['xstar'], p['lower'])
        p['upper'] = np.where(fix, inst['xstar'], p['upper'])
        inst = dict(inst, lower=p['lower'], upper=p['upper'])
    return p, inst


def args(p):
    return p['hrow'], p['hcol'], p['hval'], p['cost'], p['lower'], p['upper']
