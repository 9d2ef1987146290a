"""CPU restatement of the PI Schur-block Liouvillian path (TEST INFRASTRUCTURE ONLY).

This module is the oracle that the CUDA library is checked against.  It restates, in
exact rational arithmetic (``fractions.Fraction``) and numpy/scipy, the algorithms of
PermutationalInvariantDynamics.jl v0.1.0 on the hot path; every function cites the
reference file and lines it follows.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` may import it; the product never does.

Conventions kept from the reference:
  * sectors are partitions of N into d parts in descending lexicographic order
    (partitions.jl:29-46, basis.jl:27);
  * GT patterns are stored row by row and sorted by ascending entry tuple
    (gtpatterns.jl:92-106), which fixes the in-block index map;
  * a PI coordinate vector is the concatenation of column-major n x n blocks
    (basis.jl:31, basis.jl:90-93); offsets here are 0-based;
  * stored coefficients are sqrt(f^nu) times the physical Schur block
    (basis.jl:709-714, source_protocol.jl:15-34).
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

# --------------------------------------------------------------------------------------
# Combinatorics: partitions.jl
# --------------------------------------------------------------------------------------


def partitions(N: int, d: int):
    """Partitions of N into exactly d nonincreasing parts, descending lexicographic.

    Follows partitions.jl:29-46 (recursive enumeration with decreasing first part).
    """
    if N < 0:
        raise ValueError("N must be nonnegative")
    if d < 1:
        raise ValueError("d must be positive")
    out = []

    def rec(prefix, left, cap):
        if len(prefix) == d:
            if left == 0:
                out.append(tuple(prefix))
            return
        for x in range(min(cap, left), -1, -1):
            prefix.append(x)
            rec(prefix, left - x, x)
            prefix.pop()

    rec([], N, N)
    return out


def removable_corners(p):
    """One-based rows from which a box can be removed (partitions.jl:54)."""
    D = len(p)
    return [i + 1 for i in range(D) if p[i] > (0 if i == D - 1 else p[i + 1])]


def remove_corner(p, row):
    """Remove one box from the one-based ``row`` (partitions.jl:69-73)."""
    if row not in removable_corners(p):
        raise ValueError(f"row {row} is not a removable corner of {p}")
    return tuple(p[i] - (1 if i == row - 1 else 0) for i in range(len(p)))


def symmetric_group_dimension(p) -> int:
    """Exact f^p by the hook-length formula (partitions.jl:119-127)."""
    n = sum(p)
    if n == 0:
        return 1
    den = 1
    D = len(p)
    for i in range(D):
        for j in range(1, p[i] + 1):
            below = sum(1 for k in range(i + 1, D) if p[k] >= j)
            den *= p[i] - j + below + 1
    return math.factorial(n) // den


def unitary_group_dimension(p) -> int:
    """Exact dim of the U(d) irrep p (Weyl dimension formula)."""
    D = len(p)
    num = Fraction(1)
    for i in range(D):
        for j in range(i + 1, D):
            num *= Fraction(p[i] - p[j] + j - i, j - i)
    assert num.denominator == 1
    return int(num)


def commutant_dimension(N: int, d: int) -> int:
    """binomial(N + d^2 - 1, d^2 - 1): dimension of the PI operator space."""
    return math.comb(N + d * d - 1, d * d - 1)


def one_box_branch_weight(lam, mu) -> Fraction:
    """Exact |lam| f^mu / f^lam for removing one corner (partitions.jl:519-543)."""
    D = len(lam)
    if sum(mu) != sum(lam) - 1:
        raise ValueError("mu must have exactly one box fewer")
    rows = [i for i in range(D) if lam[i] == mu[i] + 1]
    if not rows:
        raise ValueError("mu is not obtained by removing one box")
    row = rows[0]
    for i in range(D):
        if lam[i] != mu[i] + (1 if i == row else 0):
            raise ValueError("mu is not obtained by removing one box")
    shifted = [lam[i] + D - (i + 1) for i in range(D)]
    pivot = shifted[row]
    result = Fraction(pivot)
    for index in range(row):
        diff = shifted[index] - pivot
        result *= Fraction(diff + 1, diff)
    for index in range(row + 1, D):
        diff = pivot - shifted[index]
        result *= Fraction(diff - 1, diff)
    return result


# --------------------------------------------------------------------------------------
# GT patterns: gtpatterns.jl
# --------------------------------------------------------------------------------------


def _gidx(i, k):
    """0-based storage index of entry i of row k (gtpatterns.jl:17)."""
    return k * (k - 1) // 2 + i - 1


def gt_entry(g, i, k):
    return g[_gidx(i, k)]


def gt_patterns(p):
    """All GT patterns with top row p, sorted by ascending entry tuple (gtpatterns.jl:78-106)."""
    D = len(p)
    out = []

    def interlacing_rows(upper):
        k = len(upper) - 1
        res = []

        def rec(v, i):
            if i > k:
                res.append(list(v))
                return
            for x in range(upper[i - 1], upper[i] - 1, -1):
                v.append(x)
                rec(v, i + 1)
                v.pop()

        rec([], 1)
        return res

    def descend(rows):
        if len(rows) == D:
            ordered = list(reversed(rows))
            out.append(tuple(x for row in ordered for x in row))
            return
        for row in interlacing_rows(rows[-1]):
            rows.append(row)
            descend(rows)
            rows.pop()

    descend([list(p)])
    out.sort()
    return out


def content(g, D):
    """Weight content: successive row-sum differences (gtpatterns.jl:44-71)."""
    vals = []
    for K in range(1, D + 1):
        v = sum(gt_entry(g, i, K) for i in range(1, K + 1))
        v -= sum(gt_entry(g, i, K - 1) for i in range(1, K))
        vals.append(v)
    return tuple(vals)


def shape(g, D):
    return tuple(gt_entry(g, i, D) for i in range(1, D + 1))


def triangular_shift(mu, lam, j, D):
    """Shift row positions (tau_{j+1..D}) or None (gtpatterns.jl:109-122)."""
    if not (0 <= j < D):
        return None
    tau = []
    for k in range(1, D + 1):
        dif = [gt_entry(lam, i, k) - gt_entry(mu, i, k) for i in range(1, k + 1)]
        if k <= j:
            if any(dif):
                return None
        else:
            if dif.count(1) == 1 and all(x in (0, 1) for x in dif):
                tau.append(dif.index(1) + 1)
            else:
                return None
    return tau


def _p(g, i, k):
    return gt_entry(g, i, k) + k - i


def cgc_exact(mu, j, lam, D):
    """Exact (sign, q) with CG = sign*sqrt(q), or None for zero (cgc.jl:6-39)."""
    if sum(shape(lam, D)) != sum(shape(mu, D)) + 1:
        return None
    tau = triangular_shift(mu, lam, j, D)
    if tau is None:
        return None
    tj = tau[0]
    q = Fraction(1)
    for k in range(1, j + 1):
        q *= Fraction(_p(mu, tj, j + 1) - _p(mu, k, j))
    for k in range(1, j + 2):
        if k == tj:
            continue
        q /= Fraction(_p(mu, tj, j + 1) - _p(mu, k, j + 1))
    sign = 1
    for l in range(j + 2, D + 1):
        tprev = tau[l - j - 2]
        tl = tau[l - j - 1]
        sign *= -1 if tprev < tl else 1
        for k in range(1, l + 1):
            if k == tl:
                continue
            q *= Fraction(_p(mu, tprev, l - 1) - _p(mu, k, l) + 1,
                          _p(mu, tl, l) - _p(mu, k, l))
        for k in range(1, l):
            if k == tprev:
                continue
            q *= Fraction(_p(mu, tl, l) - _p(mu, k, l - 1),
                          _p(mu, tprev, l - 1) - _p(mu, k, l - 1) + 1)
    if q < 0 and abs(float(q)) < 1e-14:
        q = abs(q)
    if q < 0:
        raise ValueError("negative squared CG coefficient")
    if q == 0:
        return None
    return sign, q


def sqrt_exact_ratio(q: Fraction) -> float:
    """sqrt of the correctly rounded Float64 of an exact rational (partitions.jl:130-160)."""
    return math.sqrt(float(q))


def cgc(mu, j, lam, D):
    r = cgc_exact(mu, j, lam, D)
    if r is None:
        return 0.0
    sign, q = r
    return float(sign) * sqrt_exact_ratio(q)


# --------------------------------------------------------------------------------------
# Basis: basis.jl
# --------------------------------------------------------------------------------------


class PIBasis:
    """Sectors, GT patterns and 0-based block offsets (basis.jl:11-35)."""

    def __init__(self, N: int, d: int = 2, sectors=None):
        if N < 0:
            raise ValueError("N must be nonnegative")
        if d < 1:
            raise ValueError("d must be positive")
        if sectors is None:
            ps = partitions(N, d)
        else:
            ps = [tuple(int(v) for v in s) for s in sectors]
        if not all(sum(p) == N and len(p) == d for p in ps):
            raise ValueError("all sectors must partition N into d parts")
        if len(set(ps)) != len(ps):
            raise ValueError("duplicate sector")
        ps = sorted(ps, reverse=True)
        self.N, self.d = N, d
        self.sectors = ps
        self.patterns = [gt_patterns(p) for p in ps]
        self.dims = [len(g) for g in self.patterns]
        offs = [0]
        for n in self.dims:
            offs.append(offs[-1] + n * n)
        self.offsets = offs
        self.index = {p: i for i, p in enumerate(ps)}

    def __len__(self):
        return self.offsets[-1]

    def block(self, x, s):
        n = self.dims[s]
        o = self.offsets[s]
        return x[o:o + n * n].reshape((n, n), order="F")


def trace_functional(b: PIBasis):
    """Sparse trace vector: sqrt(f^nu) on every block diagonal (source_protocol.jl:15-34)."""
    idx, val = [], []
    for s, p in enumerate(b.sectors):
        n = b.dims[s]
        scale = math.sqrt(float(symmetric_group_dimension(p)))
        for a in range(n):
            idx.append(b.offsets[s] + a + a * n)
            val.append(scale)
    return np.array(idx, dtype=np.int64), np.array(val, dtype=np.complex128)


# --------------------------------------------------------------------------------------
# One-body geometry: geometry.jl
# --------------------------------------------------------------------------------------


def onebody_transitions(parent_patterns, child_patterns, D):
    """Per child: [(parent index, 0-based local label, CG)] (geometry.jl:465-490)."""
    parent_by_weight = {}
    for pidx, parent in enumerate(parent_patterns):
        parent_by_weight.setdefault(content(parent, D), []).append(pidx)
    transitions = [[] for _ in child_patterns]
    for cidx, child in enumerate(child_patterns):
        cw = content(child, D)
        for label in range(D):
            pw = tuple(cw[l] + (1 if l == label else 0) for l in range(D))
            for pidx in parent_by_weight.get(pw, ()):
                value = cgc(child, label, parent_patterns[pidx], D)
                if value != 0.0:
                    transitions[cidx].append((pidx, label, value))
    return transitions


def pack_onebody_contractions(left, right):
    """Cell (a, c) -> [(i, j, x*y)] in child / left / right order (geometry.jl:405-439)."""
    cells = {}
    for cidx in range(len(left)):
        for (a, i, x) in left[cidx]:
            for (c, j, y) in right[cidx]:
                value = x * y
                if value == 0.0:
                    continue
                cells.setdefault((a, c), []).append((i, j, value))
    return cells


class OneBodyGeometry:
    """Contraction tables, branch scales and sector connections (geometry.jl:519-562)."""

    def __init__(self, b: PIBasis):
        D = b.d
        self.basis = b
        removed = [[remove_corner(p, r) for r in removable_corners(p)] for p in b.sectors]
        pattern_cache = {}
        transition_cache = {}
        for si, children in enumerate(removed):
            for mu in children:
                if mu not in pattern_cache:
                    pattern_cache[mu] = gt_patterns(mu)
                transition_cache[(si, mu)] = onebody_transitions(
                    b.patterns[si], pattern_cache[mu], D)
        self.contractions = {}
        self.scales = {}
        self.connections = {}
        for li, l in enumerate(b.sectors):
            for ni, n in enumerate(b.sectors):
                common = [mu for mu in removed[li] if mu in removed[ni]]
                if not common:
                    continue
                self.connections[(li, ni)] = common
                for mu in common:
                    key = (li, mu, ni)
                    self.contractions[key] = pack_onebody_contractions(
                        transition_cache[(li, mu)], transition_cache[(ni, mu)])
                    sq = one_box_branch_weight(l, mu) * one_box_branch_weight(n, mu)
                    self.scales[key] = sqrt_exact_ratio(sq)

    def connection(self, li, ni):
        return self.connections.get((li, ni), [])


def _contract(terms, X):
    """sum(conj(z) X[i,j]) with a zero initial value (geometry.jl:867-870)."""
    v = 0j
    for (i, j, z) in terms:
        v += z * X[i, j]
    return v


def collective_sparse_block(geom: OneBodyGeometry, s: int, X):
    """Sparse block of sum_i X_i in sector s (geometry.jl:840-865)."""
    n = geom.basis.dims[s]
    acc = {}
    for mu in geom.connection(s, s):
        scale = geom.scales[(s, mu, s)]
        for cell, terms in geom.contractions[(s, mu, s)].items():
            acc[cell] = acc.get(cell, 0j) + scale * _contract(terms, X)
    rows, cols, vals = [], [], []
    for (a, c), v in acc.items():
        if v != 0:
            rows.append(a)
            cols.append(c)
            vals.append(v)
    return sp.csc_matrix((np.array(vals, dtype=np.complex128), (rows, cols)), shape=(n, n))


def onebody_contraction(geom: OneBodyGeometry, key, X):
    """Rectangular C[a,c] = contract(table[a,c], X) (liouvillian.jl:2370-2383)."""
    li, mu, ni = key
    nl, nn = geom.basis.dims[li], geom.basis.dims[ni]
    rows, cols, vals = [], [], []
    for (a, c), terms in geom.contractions[key].items():
        v = _contract(terms, X)
        if v != 0:
            rows.append(a)
            cols.append(c)
            vals.append(v)
    return sp.csr_matrix((np.array(vals, dtype=np.complex128), (rows, cols)), shape=(nl, nn))


# --------------------------------------------------------------------------------------
# Spin helpers and model terms: spin.jl, terms.jl, model_zoo.jl
# --------------------------------------------------------------------------------------


def spin_matrices(d: int = 2):
    """Spin-j matrices in ascending |-j>..|j> order (spin.jl:13-36)."""
    j = (d - 1) / 2
    jp = np.zeros((d, d), dtype=np.complex128)
    for column in range(1, d):
        m = -j + (column - 1)
        jp[column, column - 1] = math.sqrt((j - m) * (j + m + 1))
    jm = jp.conj().T.copy()
    jx = (jp + jm) * 0.5
    jy = (jp - jm) / (2j)
    jz = np.diag([-j + k for k in range(d)]).astype(np.complex128)
    return dict(j=j, jx=jx, jy=jy, jz=jz, jp=jp, jm=jm)


class Term:
    """One model term.  kind in {"H", "LJ", "CJ"} (terms.jl:118-149)."""

    def __init__(self, kind, operator, rate=1.0, hbar=1.0):
        self.kind = kind
        self.operator = np.asarray(operator, dtype=np.complex128)
        self.rate = float(rate)
        self.hbar = float(hbar)


def CollectiveHamiltonian(H, rate=1.0, hbar=1.0):
    return Term("H", H, rate, hbar)


LocalHamiltonian = CollectiveHamiltonian


def LocalJump(L, rate=1.0):
    return Term("LJ", L, rate)


def CollectiveJump(L, rate=1.0):
    return Term("CJ", L, rate)


class PIModel:
    def __init__(self, basis: PIBasis, terms):
        self.basis = basis
        self.terms = list(terms)


def qubit_ensemble_model(N_or_basis, hamiltonian=None, emission=0.0, dephasing=0.0,
                         pumping=0.0, collective_emission=0.0, collective_dephasing=0.0,
                         collective_pumping=0.0, sectors=None):
    """Six-rate qubit model; zero rates omitted (spin.jl:437-519)."""
    b = N_or_basis if isinstance(N_or_basis, PIBasis) else PIBasis(N_or_basis, 2, sectors)
    s = spin_matrices(2)
    terms = []
    if hamiltonian is not None:
        terms.append(CollectiveHamiltonian(hamiltonian))
    for rate, op, coll in ((emission, s["jm"], False), (dephasing, s["jz"], False),
                           (pumping, s["jp"], False), (collective_emission, s["jm"], True),
                           (collective_dephasing, s["jz"], True),
                           (collective_pumping, s["jp"], True)):
        if rate != 0:
            terms.append(CollectiveJump(op, rate) if coll else LocalJump(op, rate))
    return PIModel(b, terms)


def driven_qubits(N, drive=0.7, detuning=0.0, emission=0.12, pumping=0.02, dephasing=0.0,
                  sectors=None):
    """H = drive*jx + detuning*jz with local channels (model_zoo.jl:214-242)."""
    s = spin_matrices(2)
    h = (drive / 2) * (2 * s["jx"]) + (detuning / 2) * (2 * s["jz"])
    return qubit_ensemble_model(N, hamiltonian=h, emission=emission, pumping=pumping,
                                dephasing=dephasing, sectors=sectors)


def boundary_time_crystal(N, omega=1.5, kappa=1.0):
    """Symmetric-sector BTC: H = omega*Jx, collective rate 2kappa/N (model_zoo.jl:312-325)."""
    b = PIBasis(N, 2, sectors=[(N, 0)])
    s = spin_matrices(2)
    return PIModel(b, [CollectiveHamiltonian(s["jx"], rate=omega),
                       CollectiveJump(s["jm"], rate=2 * kappa / N)])


# --------------------------------------------------------------------------------------
# Plan: compile_term + fusion (liouvillian.jl:1290-1371, 1700-1738)
# --------------------------------------------------------------------------------------


class Plan:
    """Fused static kernel: H blocks, loss blocks, collective gains, one-body gains."""

    def __init__(self, model: PIModel, geom: OneBodyGeometry | None = None):
        b = model.basis
        self.basis = b
        if b.d != 2:
            raise ValueError("the oracle plan builder is restricted to qubits (d == 2)")
        geom = geom or OneBodyGeometry(b)
        self.geom = geom
        S = len(b.sectors)
        ham = [sp.csc_matrix((n, n), dtype=np.complex128) for n in b.dims]
        loss = [sp.csc_matrix((n, n), dtype=np.complex128) for n in b.dims]
        have_h = have_q = False
        self.collective_gains = []   # (blocks, rate)
        self.onebody_gains = []      # (branches [(li, ni, bscale)], contractions, rate)
        for t in model.terms:
            if t.kind == "H":
                scale = t.rate / t.hbar
                blocks = [collective_sparse_block(geom, s, t.operator) for s in range(S)]
                ham = [ham[s] + scale * blocks[s] for s in range(S)]
                have_h = True
            elif t.kind == "CJ":
                K = [collective_sparse_block(geom, s, t.operator) for s in range(S)]
                Q = [(k.conj().T @ k).tocsc() for k in K]
                self.collective_gains.append((K, t.rate))
                loss = [loss[s] + t.rate * Q[s] for s in range(S)]
                have_q = True
            elif t.kind == "LJ":
                LL = t.operator.conj().T @ t.operator
                Q = [collective_sparse_block(geom, s, LL) for s in range(S)]
                loss = [loss[s] + t.rate * Q[s] for s in range(S)]
                have_q = True
                branches, contr = [], []
                for li in range(S):
                    for ni in range(S):
                        for mu in geom.connection(li, ni):
                            key = (li, mu, ni)
                            branches.append((li, ni, geom.scales[key]))
                            contr.append(onebody_contraction(geom, key, t.operator))
                self.onebody_gains.append((branches, contr, t.rate))
            else:
                raise ValueError(f"unsupported term kind {t.kind}")
        self.ham = [h.tocsc() for h in ham] if have_h else None
        self.loss = [q.tocsc() for q in loss] if have_q else None
        self.trace_idx, self.trace_val = trace_functional(b)

    def __len__(self):
        return len(self.basis)


def apply(plan: Plan, x):
    """y = L x, fused static kernel order (liouvillian.jl:3070-3105)."""
    b = plan.basis
    x = np.asarray(x, dtype=np.complex128)
    y = np.zeros(len(b), dtype=np.complex128)
    S = len(b.sectors)
    for s in range(S):
        n, o = b.dims[s], b.offsets[s]
        X = x[o:o + n * n].reshape((n, n), order="F")
        Y = np.zeros((n, n), dtype=np.complex128)
        if plan.ham is not None:
            H = plan.ham[s]
            Y += -1j * (H @ X - (H.T @ X.T).T)
        for blocks, rate in plan.collective_gains:
            K = blocks[s]
            left = K @ X
            Y += rate * (K.conj() @ left.T).T
        if plan.loss is not None:
            Q = plan.loss[s]
            Y -= 0.5 * (Q @ X + (Q.T @ X.T).T)
        y[o:o + n * n] += Y.reshape(-1, order="F")
    for branches, contr, rate in plan.onebody_gains:
        for (li, ni, bscale), C in zip(branches, contr):
            nl, ol = b.dims[li], b.offsets[li]
            nn, on = b.dims[ni], b.offsets[ni]
            X = x[on:on + nn * nn].reshape((nn, nn), order="F")
            T = C @ X
            T = (C.conj() @ T.T).T
            y[ol:ol + nl * nl] += (rate * bscale) * T.reshape(-1, order="F")
    return y


def materialize(plan: Plan):
    """Dense L from the same plan (the sparse-materialization oracle, liouvillian.jl:3450-3456)."""
    n = len(plan)
    L = np.zeros((n, n), dtype=np.complex128)
    e = np.zeros(n, dtype=np.complex128)
    for k in range(n):
        e[k] = 1.0
        L[:, k] = apply(plan, e)
        e[k] = 0.0
    return L


def commutator_superoperator(H):
    """Column-major vec of -i(HX - XH)."""
    n = H.shape[0]
    I = np.eye(n)
    return -1j * (np.kron(I, H) - np.kron(H.T, I))


def dissipator_superoperator(K):
    """Column-major vec of K X K' - (K'K X + X K'K)/2."""
    n = K.shape[0]
    I = np.eye(n)
    Q = K.conj().T @ K
    return np.kron(K.conj(), K) - 0.5 * (np.kron(I, Q) + np.kron(Q.T, I))


# --------------------------------------------------------------------------------------
# States and observables: basis.jl:1067, spin.jl:79-86, highlevel.jl:665-677
# --------------------------------------------------------------------------------------


def iid_pure_state(b: PIBasis, psi):
    """|psi><psi|^N in the symmetric sector (basis.jl:1067-1079), qubits only."""
    if b.d != 2:
        raise ValueError("qubit-only restatement")
    psi = np.asarray(psi, dtype=np.complex128)
    sym = (b.N, 0)
    if sym not in b.index:
        raise ValueError("the fully symmetric sector is absent")
    s = b.index[sym]
    n = b.dims[s]
    v = np.zeros(n, dtype=np.complex128)
    for a in range(n):  # a = number of level-1 (|g>) occupations
        v[a] = math.sqrt(math.comb(b.N, a)) * psi[0] ** a * psi[1] ** (b.N - a)
    x = np.zeros(len(b), dtype=np.complex128)
    o = b.offsets[s]
    x[o:o + n * n] = np.outer(v, v.conj()).reshape(-1, order="F")
    return x


def computational_product_state(b: PIBasis, level: int):
    """|level><level|^N, level one-based (spin.jl:79-86)."""
    psi = np.zeros(b.d, dtype=np.complex128)
    psi[level - 1] = 1.0
    return iid_pure_state(b, psi)


def collective_operator(b: PIBasis, X, geom: OneBodyGeometry | None = None):
    """Stored coefficients sqrt(f^nu) * block of sum_i X_i (geometry.jl:1282-1308)."""
    geom = geom or OneBodyGeometry(b)
    out = np.zeros(len(b), dtype=np.complex128)
    for s, p in enumerate(b.sectors):
        n, o = b.dims[s], b.offsets[s]
        B = collective_sparse_block(geom, s, np.asarray(X, dtype=np.complex128)).toarray()
        out[o:o + n * n] = math.sqrt(float(symmetric_group_dimension(p))) * B.reshape(-1, order="F")
    return out


def expectation(op_data, rho_data):
    """dot(op.data, rho.data) (highlevel.jl:672-677)."""
    return np.vdot(op_data, rho_data)


def trace(plan: Plan, x):
    return np.sum(plan.trace_val * x[plan.trace_idx])


# --------------------------------------------------------------------------------------
# Krylov: krylov.jl (GMRES, steady state) and krylov_extensions.jl (expv)
# --------------------------------------------------------------------------------------


def complex_givens(a, b):
    """(c, s) rotating [a; b] onto its norm (krylov.jl:710-716)."""
    if b == 0:
        return 1.0, 0j
    if a == 0:
        return 0.0, 1 + 0j
    scale = abs(a) + abs(b)
    normab = scale * math.sqrt(abs(a / scale) ** 2 + abs(b / scale) ** 2)
    alpha = a / abs(a)
    return abs(a) / normab, alpha * np.conj(b) / normab


def upper_triangular_solve(H, g, k):
    """Back substitution on the leading k x k block (krylov.jl:718-730)."""
    y = np.zeros(k, dtype=np.complex128)
    for i in range(k - 1, -1, -1):
        s = g[i]
        for j in range(i + 1, k):
            s -= H[i, j] * y[j]
        if H[i, i] == 0:
            raise np.linalg.LinAlgError(f"singular at {i}")
        y[i] = s / H[i, i]
    return y


def gmres(x, apply_fn, b, m, atol, rtol, maxiter):
    """Restarted GMRES(m) with MGS x2 and complex Givens (krylov.jl:732-787)."""
    n = len(x)
    m = min(m, n)
    bnorm = np.linalg.norm(b)
    tol = atol + rtol * bnorm
    rawtol = tol
    iterations = 0
    r = b - apply_fn(x)
    beta = np.linalg.norm(r)
    if beta <= tol and beta <= rawtol:
        return dict(converged=True, iterations=0, restarts=0, residual=beta)
    restarts = 0
    V = np.zeros((n, m + 1), dtype=np.complex128)
    while iterations < maxiter:
        H = np.zeros((m + 1, m), dtype=np.complex128)
        g = np.zeros(m + 1, dtype=np.complex128)
        cs = np.zeros(m)
        sn = np.zeros(m, dtype=np.complex128)
        V[:, 0] = r / beta
        g[0] = beta
        kdone = 0
        for j in range(min(m, maxiter - iterations)):
            w = apply_fn(V[:, j])
            for _ in range(2):
                for i in range(j + 1):
                    hij = np.vdot(V[:, i], w)
                    H[i, j] += hij
                    w = w - hij * V[:, i]
            H[j + 1, j] = np.linalg.norm(w)
            if H[j + 1, j] != 0:
                V[:, j + 1] = w / H[j + 1, j]
            for i in range(j):
                h1, h2 = H[i, j], H[i + 1, j]
                c, s = cs[i], sn[i]
                H[i, j] = c * h1 + s * h2
                H[i + 1, j] = -np.conj(s) * h1 + c * h2
            c, s = complex_givens(H[j, j], H[j + 1, j])
            cs[j], sn[j] = c, s
            h1, h2 = H[j, j], H[j + 1, j]
            H[j, j] = c * h1 + s * h2
            H[j + 1, j] = 0
            g1, g2 = g[j], g[j + 1]
            g[j] = c * g1 + s * g2
            g[j + 1] = -np.conj(s) * g1 + c * g2
            iterations += 1
            kdone = j + 1
            if abs(g[j + 1]) <= tol:
                break
        y = upper_triangular_solve(H, g, kdone)
        x += V[:, :kdone] @ y
        restarts += 1
        r = b - apply_fn(x)
        beta = np.linalg.norm(r)
        if beta <= tol and beta <= rawtol:
            return dict(converged=True, iterations=iterations, restarts=restarts, residual=beta)
    return dict(converged=False, iterations=iterations, restarts=restarts, residual=beta)


def estimated_operator_scale(apply_fn, n, probes=3, seed=0x51CA1E):
    """max ||L r|| / ||r|| over random complex normal probes (krylov.jl:156-169).

    The reference draws its probes from Julia's MersenneTwister; the oracle uses numpy's
    PCG64 with the same seed value, so the scale agrees to tolerance, not bitwise.
    """
    rng = np.random.default_rng(seed)
    scale = 0.0
    for _ in range(probes):
        r = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)
        scale = max(scale, np.linalg.norm(apply_fn(r)) / np.linalg.norm(r))
    return scale


def krylov_steady_state(plan: Plan, krylovdim=30, maxiter=500, atol=1e-10, rtol=1e-8,
                        operator_scale=None, initial_state=None, apply_fn=None):
    """Trace-bordered GMRES steady state (L/s + v t^H) rho = v (krylov.jl:797-891)."""
    n = len(plan)
    L = apply_fn or (lambda z: apply(plan, z))
    t = np.zeros(n, dtype=np.complex128)
    t[plan.trace_idx] = plan.trace_val
    v = t / np.vdot(t, t)
    x = v.copy() if initial_state is None else np.array(initial_state, dtype=np.complex128)
    s = operator_scale if operator_scale is not None else estimated_operator_scale(L, n)
    if not (np.isfinite(s) and s > 0):
        raise ValueError("operator_scale must be finite and positive")
    inv = 1.0 / s

    def bordered(z):
        y = inv * L(z)
        alpha = np.vdot(t, z)
        return y + alpha * v

    res = gmres(x, bordered, v, krylovdim, atol, rtol, maxiter)
    r = L(x)
    residual = np.linalg.norm(r)
    normalized = residual / s
    terr = abs(np.vdot(t, x) - 1)
    tol = atol + rtol * max(np.linalg.norm(x), 1.0)
    converged = res["converged"] and normalized <= tol and terr <= atol + rtol
    if not converged:
        raise RuntimeError(f"steady state did not converge: {res} {normalized} {terr}")
    return x, dict(residual=residual, normalized_residual=normalized, trace_error=terr,
                   iterations=res["iterations"], restarts=res["restarts"], operator_scale=s)


def _expv_arnoldi(ws, A):
    """Arnoldi with MGS x2 and near-breakdown enlargement (krylov_extensions.jl:1346-1401)."""
    current = ws["current"]
    beta = np.linalg.norm(current)
    V, H = ws["V"], ws["H"]
    n, mp1 = V.shape
    m = mp1 - 1
    if beta == 0:
        return dict(beta=0.0, zero_state=True, k=0, used=0, completed=True, enlarged=False,
                    q=0, coeff_count=0, next_remainder=0.0)
    H[:] = 0
    V[:, 0] = current / beta
    k = 0
    exact_breakdown = False
    near_breakdown = False
    breakfactor = math.sqrt(np.finfo(float).eps)
    for j in range(m):
        w = A(V[:, j])
        image_norm = np.linalg.norm(w)
        for _ in range(2):
            for i in range(j + 1):
                alpha = np.vdot(V[:, i], w)
                H[i, j] += alpha
                w = w - alpha * V[:, i]
        H[j + 1, j] = np.linalg.norm(w)
        k = j + 1
        if H[j + 1, j] == 0 or (j + 1) == n:
            exact_breakdown = True
            break
        near_breakdown |= abs(H[j + 1, j]) <= breakfactor * max(image_norm, np.finfo(float).tiny)
        V[:, j + 1] = w / H[j + 1, j]
    q = k + (0 if exact_breakdown else 1)
    S = np.zeros((q, q), dtype=np.complex128)
    S[:k, :k] = H[:k, :k]
    if not exact_breakdown:
        S[k, k - 1] = H[k, k - 1]
    used = k
    enlarged = False
    next_remainder = 0.0
    if not exact_breakdown and near_breakdown:
        enlarged = True
        used += 1
        w = A(V[:, q - 1])
        for _ in range(2):
            for i in range(q):
                alpha = np.vdot(V[:, i], w)
                S[i, q - 1] += alpha
                w = w - alpha * V[:, i]
        next_remainder = np.linalg.norm(w)
    coeff_count = q if enlarged else k
    completed = exact_breakdown or (enlarged and (q == n or next_remainder == 0))
    return dict(beta=beta, zero_state=False, k=k, used=used, completed=completed,
                enlarged=enlarged, q=q, coeff_count=coeff_count, next_remainder=next_remainder,
                S=S)


def _expv_project(ws, h, f):
    """Small exponential, trial state and defect estimate (krylov_extensions.jl:1403-1426)."""
    if f["zero_state"]:
        ws["trial"][:] = 0
        return 0.0, 0, True
    k, q = f["k"], f["q"]
    E = sla.expm(h * f["S"])
    cc = f["coeff_count"]
    ws["trial"][:] = f["beta"] * (ws["V"][:, :cc] @ E[:cc, 0])
    if f["completed"]:
        err = 0.0
    elif f["enlarged"]:
        err = f["beta"] * abs(h) * f["next_remainder"] * abs(E[q - 1, 0])
    else:
        err = f["beta"] * abs(E[k, 0])
    return float(err), k, f["completed"]


def krylov_expv(A, b, t, krylovdim=30, atol=1e-10, rtol=1e-8, initial_step=None,
                minimum_step=None, maximum_step=None, max_steps=10_000, safety=0.9,
                ws=None):
    """Adaptive restarted-Arnoldi exp(tA) b (krylov_extensions.jl:1452-1573)."""
    n = len(b)
    m = min(n, krylovdim)
    if ws is None or ws["V"].shape != (n, m + 1):
        ws = dict(V=np.zeros((n, m + 1), dtype=np.complex128),
                  H=np.zeros((m + 1, m), dtype=np.complex128),
                  current=np.zeros(n, dtype=np.complex128),
                  trial=np.zeros(n, dtype=np.complex128))
    time = float(t)
    total = abs(time)
    info = dict(accepted_steps=0, rejected_steps=0, operator_applications=0,
                estimated_error=0.0, arnoldi_factorizations=0, trial_evaluations=0)
    if total == 0:
        return np.array(b, dtype=np.complex128), dict(info, converged=True, reached_time=0.0)
    hmax = total if maximum_step is None else float(maximum_step)
    hmin = 0.0 if minimum_step is None else float(minimum_step)
    h0 = hmax if initial_step is None else float(initial_step)
    hmax = min(hmax, total)
    h = min(h0, hmax)
    ws["current"][:] = b
    reached = 0.0
    attempts = 0
    direction = math.copysign(1.0, time)
    f = None
    while reached < total and attempts < max_steps:
        attempts += 1
        h = min(h, total - reached)
        if f is None:
            f = _expv_arnoldi(ws, A)
            info["operator_applications"] += f["used"]
            info["arnoldi_factorizations"] += 1
        err, k, breakdown = _expv_project(ws, direction * h, f)
        finite = bool(np.all(np.isfinite(ws["trial"]))) and math.isfinite(err)
        trial_norm = np.linalg.norm(ws["trial"]) if finite else np.linalg.norm(ws["current"])
        fraction = h / total
        localtol = fraction * (atol + rtol * trial_norm)
        accept = finite and (breakdown or err <= localtol)
        if accept:
            ws["current"][:] = ws["trial"]
            remaining = total - reached
            reached = total if h == remaining else reached + h
            info["accepted_steps"] += 1
            info["estimated_error"] += err
            f = None
        else:
            info["rejected_steps"] += 1
        if not finite:
            factor = 0.2
        elif breakdown:
            factor = 5.0
        elif err == 0:
            factor = 2.0
        else:
            factor = safety * (localtol / err) ** (1.0 / max(k, 1))
            factor = min(max(factor, 0.2), 5.0)
        if not accept:
            factor = min(factor, 0.5)
        hnew = min(hmax, h * factor)
        if not accept and (hnew < hmin or hnew == 0 or (reached > 0 and reached + hnew == reached)):
            break
        h = max(hnew, hmin)
    info["trial_evaluations"] = attempts
    converged = reached == total
    if not converged:
        raise RuntimeError(f"expv reached {reached} of {total}")
    return ws["current"].copy(), dict(info, converged=True, reached_time=direction * reached)


def saved_times(tspan, saveat):
    """Saved-time grid (highlevel.jl:434-465)."""
    t0, t1 = float(tspan[0]), float(tspan[1])
    if saveat is None:
        return [t0, t1]
    if np.isscalar(saveat):
        step = float(saveat)
        count = int(math.floor((t1 - t0) / step + 1e-12)) + 1
        # Julia's float range t0:step:t1 computes t0 + i*step with correction; here we
        # use the same closed form and append t1 when the grid stops short.
        ts = [t0 + i * step for i in range(count) if t0 + i * step <= t1]
        if not ts or ts[-1] < t1:
            ts.append(t1)
        return ts
    ts = [float(v) for v in saveat]
    return ts


def solve_dynamics_expv(plan: Plan, rho0, tspan, saveat=None, observables=None,
                        krylovdim=30, atol=1e-10, rtol=1e-8, save_states=True):
    """solve_dynamics(...; algorithm=:expv) with streamed observables (highlevel.jl:559-733)."""
    ts = saved_times(tspan, saveat)
    current = np.array(rho0, dtype=np.complex128)
    A = lambda z: apply(plan, z)
    obs = observables or {}
    values = {k: [expectation(o, current)] for k, o in obs.items()}
    states = [current.copy()] if save_states else None
    ws = None
    infos = []
    for i in range(1, len(ts)):
        dt = ts[i] - ts[i - 1]
        if dt != 0:
            current, info = krylov_expv(A, current, dt, krylovdim=krylovdim, atol=atol,
                                        rtol=rtol, ws=ws)
            infos.append(info)
        for k, o in obs.items():
            values[k].append(expectation(o, current))
        if save_states:
            states.append(current.copy())
    return dict(t=ts, states=states, values={k: np.array(v) for k, v in values.items()},
                infos=infos)


# --------------------------------------------------------------------------------------
# Fixed-step RK4: evolution.jl (evolve!) and the default solve_dynamics algorithm
# --------------------------------------------------------------------------------------


def evolve_rk4(A, src, tspan, steps=256):
    """evolve!(dest, L, src, tspan; steps) (evolution.jl:75-118).

    Three scratch vectors k1, k2 (the stage sum) and tmp; per step
    k1 = L dest; k2 = k1; tmp = dest + (h/2) k1; k1 = L tmp; k2 += 2 k1;
    tmp = dest + (h/2) k1; k1 = L tmp; k2 += 2 k1; tmp = dest + h k1; k1 = L tmp;
    k2 += k1; dest += (h/6) k2, with h = (t1 - t0) / steps.
    """
    if steps <= 0:
        raise ValueError("steps must be positive")
    t0, t1 = float(tspan[0]), float(tspan[1])
    h = (t1 - t0) / steps
    dest = np.array(src, dtype=np.complex128)
    for _ in range(steps):
        k1 = A(dest)
        k2 = k1.copy()
        tmp = dest + (h / 2) * k1
        k1 = A(tmp)
        k2 = k2 + 2 * k1
        tmp = dest + (h / 2) * k1
        k1 = A(tmp)
        k2 = k2 + 2 * k1
        tmp = dest + h * k1
        k1 = A(tmp)
        k2 = k2 + k1
        dest = dest + (h / 6) * k2
    return dest


def solve_dynamics_rk4(plan: Plan, rho0, tspan, saveat=None, observables=None,
                       steps_per_interval=64, save_states=True):
    """solve_dynamics(...; algorithm=:auto) on a matrix-free source: RK4 per saved interval
    with `steps_per_interval` steps, skipping zero-length intervals (highlevel.jl:559-566,
    623-631, 693-712; the :auto choice is highlevel.jl:1482-1523)."""
    if steps_per_interval <= 0:
        raise ValueError("steps_per_interval must be positive")
    ts = saved_times(tspan, saveat)
    current = np.array(rho0, dtype=np.complex128)
    A = lambda z: apply(plan, z)
    obs = observables or {}
    values = {k: [expectation(o, current)] for k, o in obs.items()}
    states = [current.copy()] if save_states else None
    for i in range(1, len(ts)):
        if ts[i] != ts[i - 1]:
            current = evolve_rk4(A, current, (ts[i - 1], ts[i]), steps=steps_per_interval)
        for k, o in obs.items():
            values[k].append(expectation(o, current))
        if save_states:
            states.append(current.copy())
    return dict(t=ts, states=states, values={k: np.array(v) for k, v in values.items()})


# --------------------------------------------------------------------------------------
# Adjoint and Arnoldi spectra: liouvillian.jl (apply_adjoint!), krylov.jl (spectrum)
# --------------------------------------------------------------------------------------


def adjoint_matrix(plan: Plan):
    """The adjoint generator: conjugate transpose of the PI-coordinate matrix, the operator
    apply_adjoint! applies (liouvillian.jl:3275-3324; duality in
    test_liouvillian_properties.jl:145-150)."""
    return materialize(plan).conj().T


def ritz_order(values, which):
    """_ritz_order (krylov.jl:893-898), stable like Julia's sortperm."""
    if which == "LR":
        return np.argsort(-values.real, kind="stable")
    if which == "LM":
        return np.argsort(-np.abs(values), kind="stable")
    if which == "SM":
        return np.argsort(np.abs(values), kind="stable")
    raise ValueError("which must be :LR, :LM, or :SM")


def krylov_liouvillian_spectrum(A, n, nev=6, krylovdim=None, which="LR", initial_vector=None, atol=1e-10,
                                rtol=1e-8, vectors=False, rng=None, require_convergence=True):
    """krylov_liouvillian_spectrum (krylov.jl:914-962): m-step Arnoldi with two modified
    Gram-Schmidt passes per step, breakdown test |H[j+1,j]| <= eps max(|L v_j|, tiny), Ritz
    values of H[1:k,1:k], residuals |H[k+1,k] y_k|, tolerance atol + rtol max_j |H[:,j]|."""
    if not (0 < nev <= n):
        raise ValueError("nev must lie between 1 and the operator dimension")
    krylovdim = max(20, 2 * nev + 4) if krylovdim is None else krylovdim
    m = min(n, max(krylovdim, nev + 1))
    V = np.zeros((n, m + 1), dtype=np.complex128)
    H = np.zeros((m + 1, m), dtype=np.complex128)
    if initial_vector is None:
        rng = rng if rng is not None else np.random.default_rng(0)
        q = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
    else:
        q = np.array(initial_vector, dtype=np.complex128)
    nq = np.linalg.norm(q)
    if not nq > 0:
        raise ValueError("initial_vector must be nonzero")
    V[:, 0] = q / nq
    k = 0
    eps = np.finfo(float).eps
    for j in range(m):
        w = A(V[:, j])
        image_norm = np.linalg.norm(w)
        for _ in range(2):
            for i in range(j + 1):
                hij = np.vdot(V[:, i], w)
                H[i, j] += hij
                w = w - hij * V[:, i]
        H[j + 1, j] = np.linalg.norm(w)
        k = j + 1
        if j == m - 1 or abs(H[j + 1, j]) <= eps * max(image_norm, np.finfo(float).tiny):
            break
        V[:, j + 1] = w / H[j + 1, j]
    vals, Y = np.linalg.eig(H[:k, :k])
    order = ritz_order(vals, which)[:min(nev, k)]
    vals, Y = vals[order], Y[:, order]
    residuals = np.abs(H[k, k - 1] * Y[-1, :])
    scale = max(max((np.linalg.norm(H[:k + 1, j]) for j in range(k)), default=0.0), np.finfo(float).tiny)
    tol = atol + rtol * scale
    converged = residuals <= tol
    if require_convergence and not converged.all():
        raise ValueError("Arnoldi spectrum did not converge")
    out = dict(values=vals, residuals=residuals, converged=converged, iterations=k, krylov_dimension=m,
               dimension=n, which=which, residual_scale=scale, residual_tolerance=tol)
    if vectors:
        out["vectors"] = V[:, :k] @ Y
    return out


def _mgs2(q, V, k):
    """_orthogonalize! (krylov.jl:973-978): two modified Gram-Schmidt passes against the
    first k columns of V; returns |q|."""
    for _ in range(2):
        for i in range(k):
            q -= np.vdot(V[:, i], q) * V[:, i]
    return np.linalg.norm(q)


def _orthonormalize_columns(R, ncols):
    """_orthonormalize_columns! (krylov.jl:980-995): two-pass Gram-Schmidt over the columns,
    dropping those whose norm falls to sqrt(eps) of their initial norm; returns the count
    kept in the leading columns."""
    kept = 0
    threshold = np.sqrt(np.finfo(float).eps)
    for j in range(ncols):
        col = R[:, j].copy()
        initial = np.linalg.norm(col)
        for _ in range(2):
            for i in range(kept):
                col -= np.vdot(R[:, i], col) * R[:, i]
        beta = np.linalg.norm(col)
        if beta <= threshold * max(initial, np.finfo(float).tiny):
            continue
        R[:, kept] = col / beta
        kept += 1
    return kept


def harmonic_arnoldi_spectrum(A, n, nev=6, krylovdim=None, thickdim=None, maxrestarts=20, target=0.0,
                              initial_vector=None, initial_subspace=None, atol=1e-10, rtol=1e-8,
                              vectors=False, rng=None, require_convergence=True):
    """harmonic_arnoldi_spectrum without a projector (krylov.jl:1378-1551): thick-restarted
    Arnoldi whose Ritz pairs come from the harmonic pencil (Z^H Z, Z^H V), Z = L V - sigma V,
    sigma = target, or -max(sqrt(eps) * scale, atol) for target 0 (scale = the largest
    basis-image norm).  Once the basis spans the whole space (k == n) the extraction is
    ordinary Rayleigh-Ritz on V^H L V.  Pairs are ordered by distance to the target; the
    converged pairs plus the nearest others (up to thickdim) seed the next cycle."""
    eps = np.finfo(float).eps
    tiny = np.finfo(float).tiny
    if not (0 < nev <= n):
        raise ValueError("nev must lie between 1 and the operator dimension")
    if maxrestarts < 0:
        raise ValueError("maxrestarts must be nonnegative")
    krylovdim = max(30, 3 * nev + 6) if krylovdim is None else krylovdim
    thickdim = max(nev + 2, 2 * nev) if thickdim is None else thickdim
    m = min(n, max(krylovdim, nev + 2))
    keep = min(m - 1, max(thickdim, nev))
    if initial_vector is not None and initial_subspace is not None:
        raise ValueError("initial_vector and initial_subspace are mutually exclusive")
    rng = rng if rng is not None else np.random.default_rng(0)

    def randn():
        return (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)

    breakfactor = np.sqrt(eps)
    V = np.zeros((n, m), dtype=np.complex128)
    LV = np.zeros((n, m), dtype=np.complex128)
    nkeep = 0
    if initial_subspace is not None:
        S = np.asarray(initial_subspace, dtype=np.complex128)
        for column in range(min(S.shape[1], keep)):
            q = S[:, column].copy()
            seednorm = np.linalg.norm(q)
            beta = _mgs2(q, V, nkeep)
            if beta <= breakfactor * max(seednorm, seednorm * eps, tiny):
                continue
            V[:, nkeep] = q / beta
            nkeep += 1
        if nkeep == 0:
            raise ValueError("initial_subspace has no independent component in the selected symmetry sector")
    else:
        q = randn() if initial_vector is None else np.array(initial_vector, dtype=np.complex128)
        nq = np.linalg.norm(q)
        if not nq > breakfactor * max(nq, tiny):
            raise ValueError("initial_vector has zero component in the selected symmetry sector")
        V[:, 0] = q / nq
        nkeep = 1
    initial_retained = nkeep
    applications = 0
    best = None
    history = []
    requested = complex(target)
    for cycle in range(maxrestarts + 1):
        k = nkeep
        for j in range(nkeep):
            LV[:, j] = A(V[:, j])
            applications += 1
        while k < m:
            q = LV[:, k - 1].copy()
            image_norm = np.linalg.norm(q)
            beta = _mgs2(q, V, k)
            if beta <= breakfactor * max(image_norm, tiny):
                q = randn()
                seednorm = np.linalg.norm(q)
                beta = _mgs2(q, V, k)
                if beta <= breakfactor * max(seednorm, seednorm * eps, tiny):
                    break
            V[:, k] = q / beta
            k += 1
            LV[:, k - 1] = A(V[:, k - 1])
            applications += 1
        exhausted = k == n
        Vk, LVk = V[:, :k], LV[:, :k]
        scale = max(max(np.linalg.norm(LVk[:, j]) for j in range(k)), tiny)
        sigma = complex(-max(np.sqrt(eps) * scale, atol)) if requested == 0 else requested
        if exhausted:
            lam, Y = sla.eig(Vk.conj().T @ LVk)
        else:
            Z = LVk - sigma * Vk
            mu, Y = sla.eig(Z.conj().T @ Z, Z.conj().T @ Vk)
            lam = sigma + mu
        finite = np.flatnonzero(np.isfinite(lam.real) & np.isfinite(lam.imag))
        if finite.size == 0:
            raise ValueError("Ritz extraction returned no finite eigenvalues; enlarge krylovdim or change the "
                             "initial vector")
        order = finite[np.argsort(np.abs(lam[finite] - requested), kind="stable")]
        sel = order[:min(nev, order.size)]
        vals = lam[sel]
        X = Vk @ Y[:, sel]
        LX = LVk @ Y[:, sel]
        nx = np.linalg.norm(X, axis=0)
        X, LX = X / nx, LX / nx
        residuals = np.linalg.norm(LX - X * vals, axis=0)
        tol = atol + rtol * scale
        converged = residuals <= tol
        history.append(dict(cycle=cycle, subspace_dimension=k, locked=int(converged.sum()),
                            maximum_residual=float(residuals.max()), residual_scale=scale,
                            ritz_extraction="rayleigh_ritz" if exhausted else "harmonic",
                            search_space_exhausted=exhausted))
        best = dict(values=vals, residuals=residuals, converged=converged, restarts=cycle,
                    iterations=applications, krylov_dimension=m, retained_dimension=keep,
                    final_retained_dimension=nkeep, initial_retained_dimension=initial_retained,
                    locked=int(converged.sum()), dimension=n, target=requested, harmonic_shift=sigma,
                    algorithm="harmonic", ritz_extraction="rayleigh_ritz" if exhausted else "harmonic",
                    search_space_exhausted=exhausted, residual_scale=scale, residual_tolerance=tol,
                    restart_history=list(history))
        if vectors:
            best["vectors"] = X
        if vals.size >= nev and converged.all():
            return best
        if exhausted:
            if require_convergence:
                raise ValueError("Rayleigh--Ritz extraction in the complete search space did not converge")
            return best
        if cycle == maxrestarts:
            break
        retain = [int(idx) for j, idx in enumerate(sel) if converged[j]]
        for idx in order:
            if int(idx) in retain:
                continue
            retain.append(int(idx))
            if len(retain) >= min(keep, order.size):
                break
        R = Vk @ Y[:, retain]
        nkeep = _orthonormalize_columns(R, len(retain))
        if nkeep == 0:
            raise ValueError("harmonic restart lost the retained invariant subspace")
        V[:, :nkeep] = R[:, :nkeep]
    if require_convergence:
        raise ValueError("thick-restarted harmonic Arnoldi did not converge")
    return best


def _arnoldi_expand(A, V, H, first, last):
    """_arnoldi_expand! (krylov.jl:1000-1015), 0-based columns first..last-1: two modified
    Gram-Schmidt passes per step, breakdown at |h| <= eps * max(|L v_j|, tiny); returns the
    number of basis columns with images."""
    eps = np.finfo(float).eps
    k = first
    for j in range(first, last):
        w = A(V[:, j])
        image_norm = np.linalg.norm(w)
        H[:j + 1, j] = 0
        for _ in range(2):
            for i in range(j + 1):
                hij = np.vdot(V[:, i], w)
                H[i, j] += hij
                w = w - hij * V[:, i]
        H[j + 1, j] = np.linalg.norm(w)
        k = j + 1
        if abs(H[j + 1, j]) <= eps * max(image_norm, np.finfo(float).tiny):
            break
        V[:, j + 1] = w / H[j + 1, j]
    return k


def _selected_ritz_order(values, which, target):
    """_selected_ritz_order (krylov.jl:996-998)."""
    if target is None:
        return ritz_order(values, which)
    return np.argsort(np.abs(values - target), kind="stable")


def implicitly_restarted_arnoldi_spectrum(A, n, nev=6, krylovdim=None, retained_dimension=None, maxrestarts=20,
                                          which="LR", target=None, initial_vector=None, atol=1e-10, rtol=1e-8,
                                          vectors=False, rng=None, require_convergence=True):
    """implicitly_restarted_arnoldi_spectrum (krylov.jl:1035-1110): m-step Arnoldi, then per
    restart exact shifts at the unwanted Ritz values applied by implicit QR steps on the
    Hessenberg matrix, truncation to the retained columns and re-expansion."""
    if not (0 < nev <= n):
        raise ValueError("nev must lie between 1 and the operator dimension")
    krylovdim = max(30, 3 * nev + 6) if krylovdim is None else krylovdim
    retained_dimension = max(nev, min(2 * nev, krylovdim - 1)) if retained_dimension is None else retained_dimension
    m = min(n, max(krylovdim, nev + 1))
    keep = min(m - 1, max(retained_dimension, nev))
    eps = np.finfo(float).eps
    V = np.zeros((n, m + 1), dtype=np.complex128)
    H = np.zeros((m + 1, m), dtype=np.complex128)
    if initial_vector is None:
        rng = rng if rng is not None else np.random.default_rng(0)
        q = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
    else:
        q = np.array(initial_vector, dtype=np.complex128)
    nq = np.linalg.norm(q)
    if not nq > 0:
        raise ValueError("initial_vector must be nonzero")
    V[:, 0] = q / nq
    t = None if target is None else complex(target)
    k = _arnoldi_expand(A, V, H, 0, m)
    applications = k
    best = None
    for cycle in range(maxrestarts + 1):
        vals_all, Y_all = np.linalg.eig(H[:k, :k])
        order = _selected_ritz_order(vals_all, which, t)
        sel = order[:min(nev, k)]
        vals, Y = vals_all[sel], Y_all[:, sel]
        residuals = np.abs(H[k, k - 1] * Y[-1, :])
        scale = max(max(np.linalg.norm(H[:k + 1, j]) for j in range(k)), np.finfo(float).tiny)
        tol = atol + rtol * scale
        converged = residuals <= tol
        best = dict(values=vals, residuals=residuals, converged=converged, iterations=applications, restarts=cycle,
                    krylov_dimension=m, retained_dimension=keep, dimension=n, which=which, target=t,
                    algorithm="implicit_qr_arnoldi", residual_scale=scale, residual_tolerance=tol)
        if vectors:
            best["vectors"] = V[:, :k] @ Y
        if vals.size >= nev and converged.all():
            return best
        if cycle == maxrestarts or k <= keep:
            break
        Hs = H[:k, :k].copy()
        Qt = np.eye(k, dtype=np.complex128)
        for shift in vals_all[order[keep:]]:
            Q, _ = np.linalg.qr(Hs - shift * np.eye(k))
            Hs = Q.conj().T @ Hs @ Q
            Qt = Qt @ Q
        Vp = V[:, :k] @ Qt
        q = Vp[:, keep] * Hs[keep, keep - 1]
        if H[k, k - 1] != 0:
            q = q + (H[k, k - 1] * Qt[k - 1, keep - 1]) * V[:, k]
        beta = _mgs2(q, Vp, keep)
        if not beta > np.sqrt(eps) * max(scale, np.finfo(float).tiny):
            break
        V[:, :keep] = Vp[:, :keep]
        V[:, keep] = q / beta
        H[:] = 0
        H[:keep, :keep] = Hs[:keep, :keep]
        H[keep, keep - 1] = beta
        k = _arnoldi_expand(A, V, H, keep, m)
        applications += k - keep
    if require_convergence:
        raise ValueError("implicitly restarted Arnoldi did not converge")
    return best
