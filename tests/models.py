"""Model cases built twice: once for libpicuda (picuda) and once for the oracle."""
import numpy as np

import picuda
from oracle import pi_oracle as O

KIND_NAMES = {0: "H", 1: "LJ", 2: "CJ"}


def to_oracle(model: "picuda.PIModel") -> "O.PIModel":
    b = O.PIBasis(model.basis.N, 2, sectors=model.basis.sectors)
    terms = [O.Term(KIND_NAMES[t.kind], t.operator, t.rate, t.hbar) for t in model.terms]
    return O.PIModel(b, terms)


def driven_c1(N=8):
    """Driven qubits, H = Omega Jx, local decay 0.5 (the N=8 CPU-runnable configuration)."""
    return picuda.Models.driven_qubits(N, drive=1.0, emission=0.5, pumping=0.0)


def ensemble_c2(N=120):
    """H = 0.3 Jz + 1.2 Jx, local decay 0.2, local dephasing 0.1, collective decay 0.05/N."""
    s = picuda.spin_matrices(2)
    return picuda.qubit_ensemble_model(N, hamiltonian=0.3 * s["jz"] + 1.2 * s["jx"], emission=0.2,
                                       dephasing=0.1, collective_emission=0.05 / N)


def btc_c3(N=200, omega_over_kappa=1.0):
    """Boundary-time-crystal-like model on all sectors: H = Omega Jx, collective decay 1/N,
    local dephasing 0.01, Omega = omega_over_kappa * kappa."""
    s = picuda.spin_matrices(2)
    kappa = 1.0 / N
    return picuda.qubit_ensemble_model(N, hamiltonian=omega_over_kappa * kappa * s["jx"],
                                       collective_emission=kappa, dephasing=0.01)


def general(N=6, seed=0, sectors=None):
    """Random complex one-body operators for every supported term kind."""
    rng = np.random.default_rng(seed)
    b = picuda.PIBasis(N, 2, sectors=sectors)
    h = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    h = (h + h.conj().T) / 2
    L1 = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    L2 = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    L3 = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    return picuda.PIModel(b, [picuda.CollectiveHamiltonian(h, rate=0.7, hbar=1.3),
                              picuda.LocalJump(L1, rate=0.3), picuda.CollectiveJump(L2, rate=0.2),
                              picuda.LocalJump(L3, rate=0.11),
                              picuda.LocalHamiltonian(0.5 * (h + h.T.conj()), rate=0.4)])


def random_state_vector(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)


def scan_model(N, omega, gdown, gphi):
    """Parameter-scan family: H = Omega Jx, local decay gdown, local dephasing gphi,
    collective decay 1/N on J-."""
    s = picuda.spin_matrices(2)
    return picuda.qubit_ensemble_model(N, hamiltonian=omega * s["jx"], emission=gdown, dephasing=gphi,
                                       collective_emission=1.0 / N)


def scan_draws(count, seed=0, nmin=20, nmax=160):
    """Seeded draws (N, Omega, gdown, gphi): N ~ U{nmin..nmax}, Omega ~ U[0.2, 2],
    gdown ~ U[0.05, 0.5], gphi ~ U[0, 0.2]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        N = int(rng.integers(nmin, nmax + 1))
        out.append((N, float(rng.uniform(0.2, 2.0)), float(rng.uniform(0.05, 0.5)), float(rng.uniform(0.0, 0.2))))
    return out
