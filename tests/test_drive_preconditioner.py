"""The drive preconditioner's host construction (pi_precond_drive_export, no GPU).

Per Schur sector the library takes the Hamiltonian block H_s from its own lowered stencil
(row-shift terms and the diagonal of the centre term) and the loss diagonal from the centre
term's real part, and diagonalises H_s with its own tridiagonal QL.  The tables must match
the oracle's sector blocks: U orthonormal with H_s U = U diag(h) (h up to the constant that
the lowering's split of the diagonal leaves open), c_s = -2 x the mean of the loss diagonal,
and q_i = (U^T Q_s U)_ii floored at -c_s / 4.
A numpy restatement of the preconditioner built from the tables must make GMRES(50) converge
on a strongly driven model where the unpreconditioned method stalls."""
import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from tests import models as M


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    picuda.load_library()


MODELS = {
    "scan_N20_strong": lambda: M.scan_model(20, 1.5, 0.1, 0.05),
    "ensemble_c2_N14": lambda: M.ensemble_c2(14),
    "driven_c1_N9": lambda: M.driven_c1(9),
    "btc_N16": lambda: M.btc_c3(16, 1.0),
    "scan_N41_odd": lambda: M.scan_model(41, 0.7, 0.3, 0.0),
}


@pytest.mark.parametrize("name", sorted(MODELS))
def test_tables_diagonalise_the_sector_hamiltonians(name):
    model = MODELS[name]()
    tables = picuda.drive_preconditioner_tables(model)
    plan = O.Plan(M.to_oracle(model))
    assert len(tables) == len(model.basis.dims)
    for s, t in enumerate(tables):
        n = model.basis.dims[s]
        U, h = t["U"], t["h"]
        assert U.shape == (n, n) and h.shape == (n,)
        assert np.abs(U.T @ U - np.eye(n)).max() <= 1e-12 * max(n, 1)
        H = plan.ham[s].toarray() if plan.ham is not None else np.zeros((n, n))
        assert np.abs(H.imag).max() == 0.0 and np.abs(H - H.T).max() <= 1e-13
        ref = np.linalg.eigvalsh(H.real)
        shift = ref.mean() - h.mean()  # the lowering's split of the diagonal is open up to a constant
        scale = max(np.abs(H).max(), 1.0)
        assert np.abs(np.sort(h + shift) - ref).max() <= 1e-12 * scale * n
        assert np.abs(H.real @ U - U * (h + shift)[None, :]).max() <= 1e-11 * scale * n
        Q = plan.loss[s].toarray() if plan.loss is not None else np.zeros((n, n))
        assert np.abs(Q - np.diag(np.diag(Q))).max() <= 1e-13 * max(np.abs(Q).max(), 1.0)
        want = -2.0 * float(np.mean(np.diag(Q).real))
        assert t["c"] == pytest.approx(min(want, -1e-6), rel=1e-12, abs=1e-14)
        # the loss each eigenmode sees, (U^T Q U)_ii, floored at half the mean loss
        qmode = np.einsum("ai,a,ai->i", U, np.diag(Q).real, U)
        assert np.abs(t["q"] - np.maximum(qmode, -0.25 * t["c"])).max() <= 1e-12 * max(np.abs(Q).max(), 1.0)


def test_tridiagonal_ql_on_a_large_collective_block():
    """The QL solver on the largest block of N = 120 qubits driven by Jx alone: a 121 x 121
    tridiagonal matrix whose eigenvalues are exactly -60 .. 60 (the magnetic numbers)."""
    model = picuda.qubit_ensemble_model(120, hamiltonian=picuda.spin_matrices(2)["jx"], emission=0.1)
    tables = picuda.drive_preconditioner_tables(model)
    top = tables[0]
    assert top["U"].shape == (121, 121)
    h = np.sort(top["h"])
    assert np.abs((h - h.mean()) - np.arange(-60, 61)).max() <= 1e-9


def _normal_part(model, tables, s_op):
    plan = O.Plan(M.to_oracle(model))
    n = len(plan)
    t = np.zeros(n, dtype=np.complex128)
    t[plan.trace_idx] = plan.trace_val
    v = t / np.vdot(t, t)
    b = model.basis

    def D(r):
        z = np.empty_like(r)
        for sec, tab in enumerate(tables):
            o, m = b.offsets[sec], b.dims[sec]
            U, h, q = tab["U"], tab["h"], tab["q"]
            d = (-0.5 * (q[:, None] + q[None, :]) - 1j * (h[:, None] - h[None, :])) / s_op
            R = r[o:o + m * m].reshape((m, m), order="F")
            z[o:o + m * m] = (U @ ((U.T @ R @ U) / d) @ U.T).reshape(-1, order="F")
        return z

    Dv = D(v)
    den = 1 + np.vdot(t, Dv)

    def P(r):
        z = D(r)
        return z - Dv * (np.vdot(t, z) / den)

    def B(z):
        return O.apply(plan, z) / s_op + v * np.vdot(t, z)

    return P, B, v


def _gmres_left(B, b, M, m=50, tol=1e-10, maxiter=1500):
    n = len(b)
    x = M(b)
    it = 0
    bn = np.linalg.norm(b)
    while it < maxiter:
        r = b - B(x)
        if np.linalg.norm(r) <= tol * bn:
            return it, True
        z = M(r)
        beta = np.linalg.norm(z)
        V = np.zeros((n, m + 1), dtype=np.complex128)
        H = np.zeros((m + 1, m), dtype=np.complex128)
        V[:, 0] = z / beta
        k = 0
        for j in range(m):
            w = M(B(V[:, j]))
            for _ in range(2):
                hh = V[:, :j + 1].conj().T @ w
                H[:j + 1, j] += hh
                w = w - V[:, :j + 1] @ hh
            H[j + 1, j] = np.linalg.norm(w)
            k, it = j + 1, it + 1
            if H[j + 1, j] == 0:
                break
            V[:, j + 1] = w / H[j + 1, j]
        e1 = np.zeros(k + 1, dtype=np.complex128)
        e1[0] = beta
        x = x + V[:, :k] @ np.linalg.lstsq(H[:k + 1, :k], e1, rcond=None)[0]
    return it, False


def test_tables_precondition_a_strongly_driven_steady_state():
    """Strong drive (Omega = 1.5 against loss 0.1, dephasing 0.05): the drive part applied
    twice per step (as the library's GMRES does) converges in a few restarts; the level
    sweep's charge-keeping part cannot, the drive changes the charge."""
    model = M.scan_model(16, 1.5, 0.1, 0.05)
    tables = picuda.drive_preconditioner_tables(model)
    plan = O.Plan(M.to_oracle(model))
    s_op = O.estimated_operator_scale(lambda z: O.apply(plan, z), len(plan))
    P, B, v = _normal_part(model, tables, s_op)

    def twice(r):
        z = P(r)
        return z + P(r - B(z))

    it, ok = _gmres_left(B, v, twice)
    assert ok and it <= 200, it
