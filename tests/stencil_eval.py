"""Numpy evaluation of the stencil tables exported by libpicuda (test helper only).

Each row of the table is {out_sector, src_sector, kind, cls, dr, dc, alpha_off, beta_off}:
kind 0 ADD  y[a,b] += (alpha[a] + beta[b]) x[a,b]
kind 1 LEFT y[a,b] += alpha[a] x[a+dr, b]
kind 2 RIGHT y[a,b] += beta[b] x[a, b+dc]
kind 3 SAND y[a,b] += alpha[a] beta[b] x[a+dr, b+dc]
"""
import numpy as np


def _shifted(X, dr, dc, n):
    """Z[a, b] = X[a+dr, b+dc] (zero outside) for an n x n output."""
    m = X.shape[0]
    Z = np.zeros((n, n), dtype=X.dtype)
    a0, a1 = max(0, -dr), min(n, m - dr)
    b0, b1 = max(0, -dc), min(n, m - dc)
    if a1 > a0 and b1 > b0:
        Z[a0:a1, b0:b1] = X[a0 + dr:a1 + dr, b0 + dc:b1 + dc]
    return Z


def evaluate(basis, table, coef, x):
    x = np.asarray(x, dtype=np.complex128)
    y = np.zeros_like(x)
    blocks = [x[o:o + n * n].reshape((n, n), order="F") for o, n in zip(basis.offsets, basis.dims)]
    out = [np.zeros((n, n), dtype=np.complex128) for n in basis.dims]
    for (s, src, kind, cls, dr, dc, ao, bo) in table:
        n = basis.dims[s]
        Z = _shifted(blocks[src], dr, dc, n)
        al = coef[ao:ao + n] if ao >= 0 else None
        be = coef[bo:bo + n] if bo >= 0 else None
        if kind == 0:
            out[s] += (al[:, None] + be[None, :]) * Z
        elif kind == 1:
            out[s] += al[:, None] * Z
        elif kind == 2:
            out[s] += be[None, :] * Z
        else:
            out[s] += (al[:, None] * be[None, :]) * Z
    for s, (o, n) in enumerate(zip(basis.offsets, basis.dims)):
        y[o:o + n * n] = out[s].reshape(-1, order="F")
    return y
