"""Host-side mirror of the reference's basis, model and state API for qubit ensembles.

Names, argument meanings and errors follow PermutationalInvariantDynamics.jl
(src/basis.jl, src/spin.jl, src/terms.jl, src/model_zoo.jl); only what the CUDA backend
accepts is provided (d = 2; collective/local Hamiltonians, local and collective jumps).
Combinatorial and Clebsch-Gordan quantities come from libpicuda's host-side lowering, so
the Python layer holds no numerical method of its own.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import PiArgumentError, PiDimensionMismatch


class PIBasis:
    """Equation-(7) PI operator basis for N qubits (basis.jl:11-35).

    sectors: partitions (N-k, k) in descending lexicographic order; patterns: GT entry
    triples (m, lam1, lam2) in ascending order; offsets: 0-based block offsets (the Julia
    basis stores the same offsets 1-based); len(basis) = sum n^2.
    """

    def __init__(self, N: int, d: int = 2, sectors=None):
        if N < 0:
            raise PiArgumentError("N must be nonnegative")
        if d < 1:
            raise PiArgumentError("d must be positive")
        if d != 2:
            raise PiArgumentError("the CUDA backend supports qubit ensembles (d == 2) only")
        if sectors is None:
            ps = [(N - k, k) for k in range(N // 2 + 1)]
        else:
            ps = [tuple(int(v) for v in s) for s in sectors]
        for p in ps:
            if len(p) != 2 or sum(p) != N or p[0] < p[1] or p[1] < 0:
                raise PiArgumentError("all sectors must partition N into d parts")
        if len(set(ps)) != len(ps):
            raise PiArgumentError("duplicate sector")
        ps.sort(reverse=True)
        self.N, self.d = N, d
        self.sectors = ps
        self.ks = [p[1] for p in ps]
        self.dims = [p[0] - p[1] + 1 for p in ps]
        self.patterns = [[(m, p[0], p[1]) for m in range(p[1], p[0] + 1)] for p in ps]
        offs = [0]
        for n in self.dims:
            offs.append(offs[-1] + n * n)
        self.offsets = offs
        self.index = {p: i for i, p in enumerate(ps)}

    def __len__(self):
        return self.offsets[-1]

    def __repr__(self):
        return f"PIBasis(N={self.N}, d={self.d}, sectors={len(self.sectors)}, dimension={len(self)})"

    def sector_index(self, p):
        p = tuple(p)
        if p not in self.index:
            raise PiArgumentError(f"sector {p} is absent")
        return self.index[p]

    def coefficient_block(self, data, p):
        """Column-major view of the stored block C_nu (basis.jl:90-93)."""
        s = self.sector_index(p)
        n, o = self.dims[s], self.offsets[s]
        return np.asarray(data)[o:o + n * n].reshape((n, n), order="F")

    def multiplicity_scales(self):
        """sqrt(f^nu) per sector (the stored-coefficient scale, basis.jl:100-103)."""
        lib = _lib.load()
        out = []
        for k in self.ks:
            f, r = C.c_double(), C.c_double()
            _lib.check(lib.pi_sector_multiplicity(self.N, k, C.byref(f), C.byref(r)),
                       "pi_sector_multiplicity")
            out.append(r.value)
        return np.array(out)

    def trace_functional(self):
        """(indices, values): sqrt(f^nu) on every block diagonal (source_protocol.jl:15-34)."""
        scales = self.multiplicity_scales()
        idx, val = [], []
        for s, n in enumerate(self.dims):
            o = self.offsets[s]
            for a in range(n):
                idx.append(o + a + a * n)
                val.append(scales[s])
        return np.array(idx, dtype=np.int64), np.array(val, dtype=np.complex128)


@dataclass
class PIState:
    """Density-state coordinates in a PIBasis (basis.jl:55-76)."""
    basis: PIBasis
    data: np.ndarray

    def __post_init__(self):
        self.data = np.ascontiguousarray(self.data, dtype=np.complex128)
        if self.data.shape != (len(self.basis),):
            raise PiDimensionMismatch("coefficient vector has wrong length")

    def copy(self):
        return PIState(self.basis, self.data.copy())


@dataclass
class PIOperator:
    """Operator coordinates in a PIBasis (basis.jl:37-53)."""
    basis: PIBasis
    data: np.ndarray

    def __post_init__(self):
        self.data = np.ascontiguousarray(self.data, dtype=np.complex128)
        if self.data.shape != (len(self.basis),):
            raise PiDimensionMismatch("coefficient vector has wrong length")


def spin_matrices(d: int = 2):
    """Spin-j matrices in ascending |-j>..|j> order (spin.jl:13-36); for d = 2 the local
    order is (|g>, |e>) and jm = |g><e|."""
    j = (d - 1) / 2
    jp = np.zeros((d, d), dtype=np.complex128)
    for column in range(1, d):
        m = -j + (column - 1)
        jp[column, column - 1] = math.sqrt((j - m) * (j + m + 1))
    jm = jp.conj().T.copy()
    return dict(j=j, jx=(jp + jm) * 0.5, jy=(jp - jm) / 2j,
                jz=np.diag([-j + k for k in range(d)]).astype(np.complex128), jp=jp, jm=jm)


@dataclass
class Term:
    kind: int
    operator: np.ndarray
    rate: float = 1.0
    hbar: float = 1.0

    def __post_init__(self):
        self.operator = np.asarray(self.operator, dtype=np.complex128)
        if self.operator.shape != (2, 2):
            raise PiArgumentError("one-body operators must be 2x2 for qubit ensembles")
        if callable(self.rate) or not np.isscalar(self.rate):
            raise PiArgumentError("the CUDA backend requires fixed numeric rates (autonomous models)")
        self.rate = float(self.rate)
        self.hbar = float(self.hbar)


def CollectiveHamiltonian(H, rate=1.0, hbar=1.0, check=True):
    """-(i/hbar) rate [sum_i H_i, rho] (terms.jl:126-136)."""
    H = np.asarray(H, dtype=np.complex128)
    if check and not np.array_equal(H, H.conj().T):
        raise PiArgumentError("Hamiltonian prototype must be Hermitian")
    return Term(_lib.PI_TERM_HAMILTONIAN, H, rate, hbar)


def LocalHamiltonian(H, rate=1.0, hbar=1.0, check=True):
    """Same microscopic action as CollectiveHamiltonian (terms.jl:114-124)."""
    return CollectiveHamiltonian(H, rate, hbar, check)


def LocalJump(L, rate=1.0):
    """rate * sum_i D[L_i] (terms.jl:138-145)."""
    return Term(_lib.PI_TERM_LOCAL_JUMP, L, rate)


def CollectiveJump(L, rate=1.0):
    """rate * D[sum_i L_i] (terms.jl:147-153)."""
    return Term(_lib.PI_TERM_COLLECTIVE_JUMP, L, rate)


@dataclass
class PIModel:
    basis: PIBasis
    terms: list = field(default_factory=list)

    def __post_init__(self):
        self.terms = list(self.terms)
        for t in self.terms:
            if not isinstance(t, Term):
                raise PiArgumentError(
                    f"unsupported PI term {type(t).__name__} for the CUDA backend "
                    "(p-body, direct, correlated and time-dependent terms are not lowered)")


def qubit_ensemble_model(N_or_basis, hamiltonian=None, emission=0, dephasing=0, pumping=0,
                         collective_emission=0, collective_dephasing=0, collective_pumping=0,
                         sectors=None):
    """Standard six-rate qubit model; fixed zero rates are omitted (spin.jl:437-519)."""
    b = N_or_basis if isinstance(N_or_basis, PIBasis) else PIBasis(N_or_basis, 2, sectors)
    s = spin_matrices(2)
    terms = []
    if hamiltonian is not None:
        terms.append(CollectiveHamiltonian(hamiltonian))
    for rate, op, coll in ((emission, s["jm"], False), (dephasing, s["jz"], False),
                           (pumping, s["jp"], False), (collective_emission, s["jm"], True),
                           (collective_dephasing, s["jz"], True), (collective_pumping, s["jp"], True)):
        if rate != 0:
            terms.append(CollectiveJump(op, rate) if coll else LocalJump(op, rate))
    return PIModel(b, terms)


class Models:
    """Recipe namespace mirroring PermutationalInvariantDynamics.Models (model_zoo.jl)."""

    @staticmethod
    def driven_qubits(N, drive=0.7, detuning=0.0, emission=0.12, pumping=0.02, dephasing=0.0,
                      sectors=None):
        """H = drive*jx + detuning*jz with local channels (model_zoo.jl:214-242)."""
        s = spin_matrices(2)
        h = (drive / 2) * (2 * s["jx"]) + (detuning / 2) * (2 * s["jz"])
        return qubit_ensemble_model(N, hamiltonian=h, emission=emission, pumping=pumping,
                                    dephasing=dephasing, sectors=sectors)

    @staticmethod
    def boundary_time_crystal(N, omega=1.5, kappa=1.0):
        """Symmetric-sector BTC, H = omega*Jx, collective rate 2kappa/N (model_zoo.jl:312-325)."""
        if N <= 0:
            raise PiArgumentError("N must be positive")
        b = PIBasis(N, 2, sectors=[(N, 0)])
        s = spin_matrices(2)
        return PIModel(b, [CollectiveHamiltonian(s["jx"], rate=omega),
                           CollectiveJump(s["jm"], rate=2 * kappa / N)])

    @staticmethod
    def local_pump_decay(N, down=1.0, up=0.25, sectors=None):
        """Independent emission and pumping (model_zoo.jl:266-279)."""
        b = PIBasis(N, 2, sectors)
        s = spin_matrices(2)
        return PIModel(b, [LocalJump(s["jm"], rate=down), LocalJump(s["jp"], rate=up)])

    @staticmethod
    def independent_dephasing(N, gamma=1.0, sectors=None):
        """One-qubit coherence decays as exp(-gamma t) (model_zoo.jl:248-257)."""
        b = PIBasis(N, 2, sectors)
        s = spin_matrices(2)
        return PIModel(b, [LocalJump(2 * s["jz"], rate=gamma / 2)])

    @staticmethod
    def steady_superradiance(N, collective_decay=1.0, pump=1.0):
        """Collective emission with local pumping (model_zoo.jl:296-310)."""
        b = PIBasis(N, 2)
        s = spin_matrices(2)
        return PIModel(b, [CollectiveJump(s["jm"], rate=collective_decay),
                           LocalJump(s["jp"], rate=pump)])


def iid_pure_state(b: PIBasis, psi) -> PIState:
    """|psi><psi|^N in the fully symmetric sector (basis.jl:1067-1079)."""
    psi = np.asarray(psi, dtype=np.complex128)
    if psi.shape != (b.d,):
        raise PiDimensionMismatch("psi must have d entries")
    if not math.isclose(float(np.vdot(psi, psi).real), 1.0, rel_tol=1.5e-8):
        raise PiArgumentError("psi must be normalized")
    s = b.sector_index((b.N, 0))
    n = b.dims[s]
    v = np.zeros(n, dtype=np.complex128)
    for a in range(n):  # a = number of |g> occupations (GT content)
        v[a] = math.sqrt(math.comb(b.N, a)) * psi[0] ** a * psi[1] ** (b.N - a)
    data = np.zeros(len(b), dtype=np.complex128)
    o = b.offsets[s]
    data[o:o + n * n] = np.outer(v, v.conj()).reshape(-1, order="F")
    return PIState(b, data)


def computational_product_state(b: PIBasis, level: int) -> PIState:
    """|level><level|^N with a one-based local level (spin.jl:79-86)."""
    if not (1 <= level <= b.d):
        raise PiArgumentError(f"level must be a one-based local-state index in 1:{b.d}")
    psi = np.zeros(b.d, dtype=np.complex128)
    psi[level - 1] = 1.0
    return iid_pure_state(b, psi)


def collective_operator(b: PIBasis, X) -> PIOperator:
    """PI coordinates of sum_i X_i: sqrt(f^nu) times each Schur block (geometry.jl:1282-1308)."""
    lib = _lib.load()
    X = np.asarray(X, dtype=np.complex128)
    if X.shape != (2, 2):
        raise PiDimensionMismatch("X must be 2x2")
    op = np.ascontiguousarray(X.reshape(-1, order="F").view(np.float64))
    data = np.zeros(len(b), dtype=np.complex128)
    scales = b.multiplicity_scales()
    for s, k in enumerate(b.ks):
        n, o = b.dims[s], b.offsets[s]
        blk = np.zeros(n * n, dtype=np.complex128)
        _lib.check(lib.pi_collective_block(b.N, k, _lib.dptr(op), _lib.dptr(blk.view(np.float64))),
                   "pi_collective_block")
        data[o:o + n * n] = scales[s] * blk
    return PIOperator(b, data)


def collective_spin(b: PIBasis, component: str) -> PIOperator:
    """J_alpha = sum_i j_alpha (spin.jl:52-77)."""
    s = spin_matrices(b.d)
    table = {"x": "jx", "y": "jy", "z": "jz", "plus": "jp", "+": "jp", "minus": "jm", "-": "jm"}
    if component not in table:
        raise PiArgumentError("component must be :x, :y, :z, :plus, or :minus")
    return collective_operator(b, s[table[component]])


def expectation(op, rho) -> complex:
    """dot(op.data, rho.data) (highlevel.jl:672-677)."""
    od = op.data if hasattr(op, "data") else np.asarray(op)
    rd = rho.data if hasattr(rho, "data") else np.asarray(rho)
    return complex(np.vdot(od, rd))
