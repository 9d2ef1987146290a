"""Full 2^N Hilbert-space Lindbladian (TEST INFRASTRUCTURE ONLY).

An oracle independent of the PI representation, the analogue of the reference's dense
Schur reference test (test/test_dense_schur_reference.jl): it builds the Liouvillian of
N <= 6 qubits directly on (C^2)^(x N) from the same terms (terms.jl:108-153: Hamiltonian
-(i/hbar) rate [sum_i H_i, rho], LocalJump rate sum_i D[L_i], CollectiveJump
rate D[sum_i L_i], with D[L] rho = L rho L' - {L'L, rho}/2) and propagates with a dense
matrix exponential, so PI results can be compared on collective observables.
Local basis order (|g>, |e>) as in spin.jl:13-36.
"""
import numpy as np
import scipy.linalg as sla


def site_op(X, i, N):
    out = np.array([[1.0 + 0j]])
    for k in range(N):
        out = np.kron(out, X if k == i else np.eye(2))
    return out


def collective(X, N):
    return sum(site_op(X, i, N) for i in range(N))


def dissipator(L):
    d = L.shape[0]
    I = np.eye(d)
    LL = L.conj().T @ L
    return np.kron(L.conj(), L) - 0.5 * (np.kron(I, LL) + np.kron(LL.T, I))


def liouvillian(N, terms):
    """terms: list of (kind, 2x2 operator, rate, hbar) with kind in {"H", "LJ", "CJ"}."""
    d = 2 ** N
    I = np.eye(d)
    L = np.zeros((d * d, d * d), dtype=np.complex128)
    for kind, op, rate, hbar in terms:
        op = np.asarray(op, dtype=np.complex128)
        if kind == "H":
            H = (rate / hbar) * collective(op, N)
            L += -1j * (np.kron(I, H) - np.kron(H.T, I))
        elif kind == "CJ":
            L += rate * dissipator(collective(op, N))
        elif kind == "LJ":
            for i in range(N):
                L += rate * dissipator(site_op(op, i, N))
        else:
            raise ValueError(kind)
    return L


def product_state(N, psi):
    v = np.array([1.0 + 0j])
    for _ in range(N):
        v = np.kron(v, np.asarray(psi, dtype=np.complex128))
    return np.outer(v, v.conj())


def evolve_expectations(N, terms, rho0, times, observables):
    L = liouvillian(N, terms)
    d = 2 ** N
    r0 = rho0.reshape(-1, order="F")
    out = {k: [] for k in observables}
    for t in times:
        r = (sla.expm(t * L) @ r0).reshape((d, d), order="F")
        for k, O in observables.items():
            out[k].append(np.trace(O @ r))
    return {k: np.array(v) for k, v in out.items()}
