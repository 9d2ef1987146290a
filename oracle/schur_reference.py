"""Dense Schur transform of (C^d)^N from standard Young paths (TEST INFRASTRUCTURE ONLY).

A restatement of the reference's deliberately exponential, test-only Schur oracle
(test/test_dense_schur_reference.jl:5-23): every standard Young path from the empty
partition to a sector lambda (src/pbody.jl:45-51, _removal_paths) supplies one multiplicity
copy of lambda, and the product of the one-box Clebsch-Gordan transitions along the path
(src/pbody.jl:266-315, _path_isometry, with the transitions of src/geometry.jl:172-196)
supplies that copy's rows of the transform.  Stacking the copies of all sectors gives an
orthogonal d^N x d^N matrix S.  For a permutation-invariant operator rho on (C^d)^N,
S rho S^T is block diagonal with one identical physical block per copy, and the stored PI
coefficient block of sector lambda is sqrt(f^lambda) times that physical block
(src/basis.jl:163-175).

This ties the PI coordinates themselves -- sector order, GT order, column-major blocks, the
sqrt(f) scale and the CG signs -- to the full 2^N Lindbladian: the PI Liouvillian must
equal Psi o L_full o Phi with Phi(x) = S^T (+)_copies (x_lambda / sqrt f) S and
Psi(rho) = sqrt(f) [S rho S^T]_(lambda, copy 1).  Only tests import this module.
"""
from __future__ import annotations

import math

import numpy as np

from . import pi_oracle as O


def removal_paths(endpoint, p):
    """Paths [centre, ..., endpoint] removing p corners from endpoint (pbody.jl:45-51); with
    p = N the centre is the empty partition and there are f^endpoint paths."""
    endpoint = tuple(endpoint)
    if p == 0:
        return [[endpoint]]
    out = []
    for row in O.removable_corners(endpoint):
        for tail in removal_paths(O.remove_corner(endpoint, row), p - 1):
            out.append(tail + [endpoint])
    return out


def onebox_maps(lower, upper, D):
    """maps[label][upper index, lower index] = CG(lower pattern, label, upper pattern)
    (geometry.jl:172-196)."""
    lp, up = O.gt_patterns(lower), O.gt_patterns(upper)
    maps = [np.zeros((len(up), len(lp))) for _ in range(D)]
    by_weight = {}
    for ui, u in enumerate(up):
        by_weight.setdefault(O.content(u, D), []).append(ui)
    for li, low in enumerate(lp):
        w = O.content(low, D)
        for label in range(D):
            pw = tuple(w[k] + (1 if k == label else 0) for k in range(D))
            for ui in by_weight.get(pw, ()):
                maps[label][ui, li] = O.cgc(low, label, up[ui], D)
    return maps


def path_isometry(path, D):
    """U[endpoint pattern, centre pattern, word] along one path (pbody.jl:266-315): word
    w = sum_s label_s D^(s-1) takes the local label of stage s from its base-D digit s."""
    p = len(path) - 1
    dims = [len(O.gt_patterns(x)) for x in path]
    words = D ** p
    U = np.zeros((dims[-1], dims[0], words))
    if p == 0:
        U[:, :, 0] = np.eye(dims[0])
        return U
    transitions = [onebox_maps(path[s], path[s + 1], D) for s in range(p)]
    for word in range(words):
        cur = np.eye(dims[0])
        for s in range(p):
            label = (word // D ** s) % D
            cur = transitions[s][label] @ cur
        U[:, :, word] = cur
    return U


def dense_schur_reference(N, D):
    """The transform S (D^N x D^N) and its copy labels (sector, multiplicity, row range),
    sectors in the reference's descending partition order (test_dense_schur_reference.jl:5-23)."""
    pieces, labels = [], []
    offset = 0
    for sector in O.partitions(N, D):
        paths = removal_paths(sector, N)
        if len(paths) != O.symmetric_group_dimension(sector):
            raise AssertionError("path count differs from f^lambda")
        for m, path in enumerate(paths):
            U = path_isometry(path, D)
            block = U.reshape(U.shape[0], D ** N)  # the centre (empty partition) has one pattern
            pieces.append(block)
            labels.append((tuple(sector), m, range(offset, offset + block.shape[0])))
            offset += block.shape[0]
    return np.vstack(pieces), labels


def site_operator(X, site, N, D):
    """X acting on one site; the site's digit in the full index is the word digit of that
    stage (least significant first), matching path_isometry's word order."""
    out = np.ones((1, 1), dtype=np.complex128)
    for s in reversed(range(N)):  # most significant digit first in the Kronecker product
        out = np.kron(out, X if s == site else np.eye(D))
    return out


def collective_sum(X, N, D):
    return sum(site_operator(X, s, N, D) for s in range(N))


def full_lindbladian(model, N, D):
    """rho -> L rho on (C^D)^N for the model's terms (terms.jl:118-149): Hamiltonians
    rate/hbar * sum_i X_i, LocalJump rate * sum_i D[L_i], CollectiveJump rate * D[sum_i L_i]."""
    H = np.zeros((D ** N, D ** N), dtype=np.complex128)
    jumps = []
    for t in model.terms:
        op = np.asarray(t.operator, dtype=np.complex128)
        if t.kind == "H":
            H = H + (t.rate / t.hbar) * collective_sum(op, N, D)
        elif t.kind == "LJ":
            for s in range(N):
                jumps.append((t.rate, site_operator(op, s, N, D)))
        elif t.kind == "CJ":
            jumps.append((t.rate, collective_sum(op, N, D)))
        else:
            raise ValueError(f"unsupported term kind {t.kind}")

    def L(rho):
        out = -1j * (H @ rho - rho @ H)
        for rate, K in jumps:
            KK = K.conj().T @ K
            out = out + rate * (K @ rho @ K.conj().T - 0.5 * (KK @ rho + rho @ KK))
        return out

    return L


class SchurMaps:
    """Phi (PI coefficients -> full operator) and Psi (full operator -> PI coefficients) of a
    basis, from the dense Schur transform."""

    def __init__(self, basis: "O.PIBasis"):
        N, D = basis.N, basis.d
        self.basis = basis
        self.S, self.labels = dense_schur_reference(N, D)
        self.sqrt_f = {tuple(p): math.sqrt(float(O.symmetric_group_dimension(p))) for p in basis.sectors}

    def phi(self, x):
        b = self.basis
        B = np.zeros(self.S.shape, dtype=np.complex128)
        for sector, _, rng in self.labels:
            if sector not in b.index:
                continue
            s = b.index[sector]
            n, o = b.dims[s], b.offsets[s]
            blk = np.asarray(x[o:o + n * n]).reshape((n, n), order="F") / self.sqrt_f[sector]
            B[rng.start:rng.stop, rng.start:rng.stop] = blk
        return self.S.T @ B @ self.S

    def psi(self, rho, check=True):
        b = self.basis
        B = self.S @ rho @ self.S.T
        out = np.zeros(len(b), dtype=np.complex128)
        first = {}
        for sector, m, rng in self.labels:
            blk = B[rng.start:rng.stop, rng.start:rng.stop]
            if sector in first:
                if check and np.abs(blk - first[sector]).max() > 1e-10 * max(1.0, np.abs(blk).max()):
                    raise AssertionError("multiplicity copies of a sector differ")
                continue
            first[sector] = blk
            if sector in b.index:
                s = b.index[sector]
                n, o = b.dims[s], b.offsets[s]
                out[o:o + n * n] = (self.sqrt_f[sector] * blk).reshape(-1, order="F")
        return out

    def offblock_norm(self, rho):
        """Norm of S rho S^T outside the copies' diagonal blocks."""
        B = self.S @ rho @ self.S.T
        for _, _, rng in self.labels:
            B[rng.start:rng.stop, rng.start:rng.stop] = 0
        return float(np.linalg.norm(B))

    def liouvillian(self, model):
        """The PI Liouvillian Psi o L_full o Phi, dense, column by column."""
        L = full_lindbladian(model, self.basis.N, self.basis.d)
        n = len(self.basis)
        out = np.zeros((n, n), dtype=np.complex128)
        e = np.zeros(n, dtype=np.complex128)
        for k in range(n):
            e[k] = 1.0
            out[:, k] = self.psi(L(self.phi(e)))
            e[k] = 0.0
        return out
