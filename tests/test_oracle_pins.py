"""Pins the CPU oracle to the reference's own known answers (no GPU).

Every check below restates a test of PermutationalInvariantDynamics.jl (file:line given)
or an analytic law those tests use, so the oracle that the CUDA library is compared with
is itself anchored to the reference's behaviour.
"""
import math
from pathlib import Path

import numpy as np
import pytest
import scipy.linalg as sla

from oracle import fullspace as F
from oracle import pi_oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_partition_dimension_identities():
    """test/test_combinatorics.jl:1-14."""
    for N in range(0, 9):
        for d in range(1, 5):
            ps = O.partitions(N, d)
            assert all(sum(p) == N for p in ps)
            assert sum(O.unitary_group_dimension(p) ** 2 for p in ps) == O.commutant_dimension(N, d)
            for p in ps:
                assert len(O.gt_patterns(p)) == O.unitary_group_dimension(p)
    assert O.symmetric_group_dimension((3, 1)) == 3
    assert O.unitary_group_dimension((3, 1)) == 3
    # descending lexicographic sector order (partitions.jl:29-46)
    assert O.partitions(4, 2) == [(4, 0), (3, 1), (2, 2)]


def test_cg_orthogonality():
    """test/test_cgc.jl:6-20: the one-box CG matrix C satisfies C C^H = I."""
    for d in (2, 3):
        for N in range(1, 6):
            for mu in O.partitions(N - 1, d):
                mus = O.gt_patterns(mu)
                lambdas = []
                for r in range(1, d + 1):
                    lam = tuple(mu[i] + (1 if i == r - 1 else 0) for i in range(d))
                    if all(lam[i] >= lam[i + 1] for i in range(d - 1)) and lam not in lambdas:
                        lambdas.append(lam)
                states = [w for lam in lambdas for w in O.gt_patterns(lam)]
                C = np.zeros((len(states), d * len(mus)))
                for a, w in enumerate(states):
                    for q, wm in enumerate(mus):
                        for j in range(d):
                            C[a, q + j * len(mus)] = O.cgc(wm, j, w, d)
                assert np.allclose(C @ C.T, np.eye(len(states)), atol=2e-13)


def _occupation_block(b, X):
    """test/test_collective_fastpaths.jl:6-35: bosonic occupation action in the symmetric sector."""
    s = b.index[(b.N, 0)]
    occ = [O.content(p, 2) for p in b.patterns[s]]
    look = {o: i for i, o in enumerate(occ)}
    n = len(occ)
    E = np.zeros((n, n), dtype=np.complex128)
    for c, o in enumerate(occ):
        for l in range(2):
            E[c, c] += o[l] * X[l, l]
        for sl in range(2):
            if o[sl] == 0:
                continue
            for tl in range(2):
                if tl == sl:
                    continue
                t = list(o)
                t[tl] += 1
                t[sl] -= 1
                E[look[tuple(t)], c] += math.sqrt((o[tl] + 1) * o[sl]) * X[tl, sl]
    return E


def test_symmetric_sector_collective_block():
    """test/test_collective_fastpaths.jl:63-80 (qubit case)."""
    X = np.array([[0.2 + 0.1j, 0.7 - 0.3j], [-0.4 + 0.2j, -0.5 + 0.6j]])
    for N in (1, 4, 7):
        b = O.PIBasis(N, 2)
        g = O.OneBodyGeometry(b)
        B = O.collective_sparse_block(g, b.index[(N, 0)], X).toarray()
        assert np.allclose(B, _occupation_block(b, X), atol=2e-13, rtol=2e-13)


def test_single_sector_generator_is_commutator_plus_dissipator():
    """test/test_collective_fastpaths.jl:98-128: L = r_h C(H) + r_j D(K) on one sector."""
    rng = np.random.default_rng(0x51C011EC)
    N = 4
    b = O.PIBasis(N, 2, sectors=[(N, 0)])
    h = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    h = (h + h.conj().T) / 2
    j = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    plan = O.Plan(O.PIModel(b, [O.CollectiveHamiltonian(h, rate=0.17), O.CollectiveJump(j, rate=0.23)]))
    lh, lj = _occupation_block(b, h), _occupation_block(b, j)
    dense = 0.17 * O.commutator_superoperator(lh) + 0.23 * O.dissipator_superoperator(lj)
    assert np.allclose(O.materialize(plan), dense, atol=3e-12, rtol=3e-12)


def _general_model(N, seed):
    rng = np.random.default_rng(seed)
    h = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    h = (h + h.conj().T) / 2
    Ls = [rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2)) for _ in range(3)]
    return O.PIModel(O.PIBasis(N, 2), [O.CollectiveHamiltonian(h, rate=0.7), O.LocalJump(Ls[0], 0.3),
                                      O.CollectiveJump(Ls[1], 0.2), O.LocalJump(Ls[2], 0.11)])


def test_trace_and_hermiticity_preservation():
    """test/test_liouvillian_properties.jl:145-185: t^H L = 0 and L maps Hermitian to Hermitian."""
    model = _general_model(6, 3)
    plan = O.Plan(model)
    L = O.materialize(plan)
    t = np.zeros(len(plan), dtype=np.complex128)
    t[plan.trace_idx] = plan.trace_val
    assert np.abs(t.conj() @ L).max() <= 1e-12 * np.abs(L).max()
    rng = np.random.default_rng(5)
    b = plan.basis
    x = np.zeros(len(plan), dtype=np.complex128)
    for s, n in enumerate(b.dims):
        A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        x[b.offsets[s]:b.offsets[s + 1]] = (A + A.conj().T).reshape(-1, order="F")
    y = L @ x
    for s, n in enumerate(b.dims):
        Y = y[b.offsets[s]:b.offsets[s + 1]].reshape((n, n), order="F")
        assert np.allclose(Y, Y.conj().T, atol=1e-12)


def test_independent_dephasing_coherence():
    """test/test_published_models.jl:432-438 with examples/paper_models.jl:79-86."""
    sz = np.array([[1, 0], [0, -1]], dtype=np.complex128)
    sx = np.array([[0, 1], [1, 0]], dtype=np.complex128) / 2
    for N in (1, 3, 5):
        b = O.PIBasis(N, 2)
        plan = O.Plan(O.PIModel(b, [O.LocalJump(sz, rate=0.4 / 2)]))
        L = O.materialize(plan)
        rho = O.iid_pure_state(b, np.array([1, 1]) / math.sqrt(2))
        S = O.collective_operator(b, sx)
        for t in (0.0, 0.2, 0.8):
            v = O.expectation(S, sla.expm(t * L) @ rho).real
            assert v == pytest.approx(N / 2 * math.exp(-0.4 * t), abs=2e-10)


def test_local_pump_decay_product_steady_state():
    """test/test_published_models.jl:439-441 (exact product state up/(down+up))."""
    sm = np.array([[0, 1], [0, 0]], dtype=np.complex128)
    b = O.PIBasis(4, 2)
    plan = O.Plan(O.PIModel(b, [O.LocalJump(sm, 1.0), O.LocalJump(sm.conj().T, 0.3)]))
    x, _ = O.krylov_steady_state(plan)
    exc = O.collective_operator(b, np.array([[0, 0], [0, 1]]))
    assert O.expectation(exc, x).real == pytest.approx(4 * 0.3 / 1.3, abs=2e-9)


def test_cooperative_fluorescence_exact_state():
    """test/test_published_models.jl:471-474 with paper_models.jl:131-137 (Morrison-Parkins)."""
    N, Omega, gamma = 4, 0.2, 0.12
    b = O.PIBasis(N, 2, sectors=[(N, 0)])
    sx = np.array([[0, 1], [1, 0]], dtype=np.complex128)
    sm = np.array([[0, 1], [0, 0]], dtype=np.complex128)
    plan = O.Plan(O.PIModel(b, [O.CollectiveHamiltonian(sx / 2, rate=Omega),
                                O.CollectiveJump(sm, rate=2 * gamma / N)]))
    x, _ = O.krylov_steady_state(plan)
    g = O.OneBodyGeometry(b)
    Jm = O.collective_sparse_block(g, 0, sm).toarray()
    a = Omega * N / (2 * gamma)
    A = Jm + 1j * a * np.eye(N + 1)
    R = np.linalg.inv(A) @ np.linalg.inv(A).conj().T
    R = (R + R.conj().T) / 2
    R /= np.trace(R)
    assert np.allclose(x, R.reshape(-1, order="F"), atol=3e-10)


def test_collective_decay_initial_derivative():
    """benchmark/comparison/README.md:26-45 (the matched_collective track): on the symmetric
    irrep, L = gamma D[J-] with gamma = 0.37 acting on |N/2,N/2><N/2,N/2| for N = 4..64 gives
    a trace-zero Hermitian derivative with |L rho|_F = sqrt(2) gamma N whose only nonzero
    eigenvalues are +gamma N and -gamma N."""
    sm = np.array([[0, 1], [0, 0]], dtype=np.complex128)
    gamma = 0.37
    for N in (4, 8, 16, 32, 64):
        b = O.PIBasis(N, 2, sectors=[(N, 0)])
        plan = O.Plan(O.PIModel(b, [O.CollectiveJump(sm, rate=gamma)]))
        y = O.apply(plan, O.computational_product_state(b, 2))
        assert abs(O.trace(plan, y)) <= 1e-12
        assert abs(np.linalg.norm(y) - math.sqrt(2) * gamma * N) <= 1e-12 * N
        Y = y.reshape(N + 1, N + 1, order="F")
        assert np.abs(Y - Y.conj().T).max() <= 1e-14 * N
        ev = np.linalg.eigvalsh((Y + Y.conj().T) / 2)
        nonzero = np.sort(ev[np.abs(ev) > 1e-10])
        assert np.allclose(nonzero, [-gamma * N, gamma * N], atol=1e-12 * N, rtol=0)


def test_collective_local_radiation_expectations():
    """test/test_published_models.jl:446-457 (Zhang-Zhang-Molmer fluxes of Dicke states)."""
    b = O.PIBasis(4, 2)
    sm = O.spin_matrices(2)["jm"]
    g = O.OneBodyGeometry(b)
    Jm = O.collective_operator(b, sm, g)
    exc = O.collective_operator(b, sm.conj().T @ sm, g)
    # J+J- in PI coordinates: blockwise product of the stored blocks divided by sqrt(f)
    JpJm = np.zeros(len(b), dtype=np.complex128)
    for s, p in enumerate(b.sectors):
        n, o = b.dims[s], b.offsets[s]
        K = Jm[o:o + n * n].reshape((n, n), order="F") / math.sqrt(O.symmetric_group_dimension(p))
        JpJm[o:o + n * n] = math.sqrt(O.symmetric_group_dimension(p)) * (K.conj().T @ K).reshape(-1, order="F")
    fully = O.iid_pure_state(b, np.array([0, 1]))
    ground = O.iid_pure_state(b, np.array([1, 0]))
    assert O.expectation(0.3 * JpJm, fully).real == pytest.approx(0.3 * 4, abs=2e-13)
    assert O.expectation(0.7 * exc, fully).real == pytest.approx(0.7 * 4, abs=2e-13)
    assert O.expectation(JpJm, ground) == 0
    assert O.expectation(exc, ground) == 0


def test_balanced_gain_loss_spectrum():
    """test/test_published_models.jl:598-616 (Nakanishi-Sasamoto exact spectrum)."""
    N, g, kappa = 5, 1.3, 0.4
    s = O.spin_matrices(2)
    S = N / 2
    b = O.PIBasis(N, 2, sectors=[(N, 0)])
    plan = O.Plan(O.PIModel(b, [O.CollectiveHamiltonian(s["jx"], rate=g),
                                O.CollectiveJump(s["jy"] + 1j * s["jz"], rate=2 * kappa / S),
                                O.CollectiveJump(s["jy"] - 1j * s["jz"], rate=2 * kappa / S)]))
    numerical = list(np.linalg.eigvals(O.materialize(plan)))
    remaining = [1j * g * q - (4 * kappa / N) * (abs(q) + l * (1 + l + 2 * abs(q)))
                 for q in range(-N, N + 1) for l in range(0, N - abs(q) + 1)]
    worst = 0.0
    for z in numerical:
        j = int(np.argmin(np.abs(np.array(remaining) - z)))
        worst = max(worst, abs(remaining[j] - z))
        remaining.pop(j)
    assert not remaining and worst < 2e-10


def test_full_hilbert_space_observables():
    """The PI expv/exp trajectory matches a 2^N Lindbladian on collective observables
    (analogue of test/test_dense_schur_reference.jl)."""
    N = 4
    s = O.spin_matrices(2)
    terms = [("H", 0.3 * s["jz"] + 1.2 * s["jx"], 1.0, 1.0), ("LJ", s["jm"], 0.2, 1.0), ("LJ", s["jz"], 0.1, 1.0),
             ("CJ", s["jm"], 0.05 / N, 1.0)]
    b = O.PIBasis(N, 2)
    plan = O.Plan(O.PIModel(b, [O.Term(k, op, r, h) for k, op, r, h in terms]))
    rho0 = O.computational_product_state(b, 2)
    obs = {"Jz": s["jz"], "JpJm_local": s["jp"] @ s["jm"]}
    ts = [0.0, 0.3, 1.1, 2.5]
    full = F.evolve_expectations(N, terms, F.product_state(N, [0, 1]),
                                 ts, {k: F.collective(v, N) for k, v in obs.items()})
    L = O.materialize(plan)
    for k, v in obs.items():
        op = O.collective_operator(b, v)
        pi = np.array([O.expectation(op, sla.expm(t * L) @ rho0) for t in ts])
        assert np.allclose(pi, full[k], atol=1e-11)


def test_gmres_and_expv_restatements():
    """test/test_krylov.jl:2-16 (GMRES vs direct) and test_krylov_extensions.jl:273-281."""
    plan = O.Plan(_general_model(4, 9))
    L = O.materialize(plan)
    x, info = O.krylov_steady_state(plan)
    assert np.linalg.norm(L @ x) / info["operator_scale"] <= 1e-10 + 1e-8 * max(np.linalg.norm(x), 1)
    b0 = O.iid_pure_state(plan.basis, np.array([0.6, 0.8j]))
    y, _ = O.krylov_expv(lambda v: L @ v, b0, 1.7)
    assert np.allclose(y, sla.expm(1.7 * L) @ b0, atol=3e-9)


def test_golden_fixtures_reproduce():
    g = np.load(GOLDEN / "driven_qubits_N8.npz")
    plan = O.Plan(O.driven_qubits(8, drive=1.0, emission=0.5, pumping=0.0))
    assert np.array_equal(np.array(plan.basis.offsets), g["offsets"])
    assert np.allclose(O.apply(plan, g["x"]), g["Lx"], atol=1e-14, rtol=0)
    ss, _ = O.krylov_steady_state(plan, operator_scale=float(g["steady_operator_scale"]))
    assert np.allclose(ss, g["steady"], atol=1e-12)
    for line in (GOLDEN / "multiplicities.txt").read_text().splitlines():
        if line.startswith("#"):
            continue
        N, k, f = line.split()
        if int(N) <= 120:
            assert O.symmetric_group_dimension((int(N) - int(k), int(k))) == int(f)


def test_threaded_c_baseline_matches_numpy_oracle():
    from oracle import cpu_baseline
    for model in (_general_model(7, 1), O.driven_qubits(12, drive=1.0, emission=0.5, pumping=0.1)):
        plan = O.Plan(model)
        ta = cpu_baseline.ThreadedApply(plan)
        rng = np.random.default_rng(3)
        x = rng.standard_normal(len(plan)) + 1j * rng.standard_normal(len(plan))
        ref = O.apply(plan, x)
        for threads in (1, 3):
            assert np.abs(ta(x, threads=threads) - ref).max() <= 1e-13 * np.abs(ref).max()


def test_rk4_restatement_matches_exponential():
    """test/test_evolution.jl:1-20: RK4 with 400 steps equals exp(tL) rho to 2e-12 for
    N=2 local decay, and chained evolutions (0,t) then (t,2t) equal exp(2tL) rho to 3e-12."""
    b = O.PIBasis(2, 2)
    plan = O.Plan(O.qubit_ensemble_model(b, emission=1.0))
    L = O.materialize(plan)
    rho = O.iid_pure_state(b, np.array([0.0, 1.0], dtype=np.complex128))
    t = 0.7
    A = lambda v: O.apply(plan, v)
    out = O.evolve_rk4(A, rho, (0.0, t), steps=400)
    assert np.allclose(out, sla.expm(t * L) @ rho, atol=2e-12, rtol=0)
    assert abs(O.trace(plan, out) - 1) <= 2e-12
    out2 = O.evolve_rk4(A, out, (t, 2 * t), steps=400)
    assert np.allclose(out2, sla.expm(2 * t * L) @ rho, atol=3e-12, rtol=0)
    with pytest.raises(ValueError):
        O.evolve_rk4(A, rho, (0.0, t), steps=0)


def test_rk4_dynamics_grid_and_expv_agreement():
    """test/test_highlevel.jl:33-60: saveat 0.05 with 40 steps per interval equals one
    160-step evolution to 2e-11; expv at tight tolerance agrees to 2e-9; repeated saved
    times give identical states."""
    b = O.PIBasis(3, 2)
    plan = O.Plan(O.qubit_ensemble_model(b, emission=0.4))
    rho0 = O.iid_pure_state(b, np.array([0.0, 1.0], dtype=np.complex128))
    sol = O.solve_dynamics_rk4(plan, rho0, (0.0, 0.2), saveat=0.05, steps_per_interval=40)
    assert len(sol["t"]) == 5
    one = O.evolve_rk4(lambda v: O.apply(plan, v), rho0, (0.0, 0.2), steps=160)
    assert np.allclose(sol["states"][-1], one, atol=2e-11, rtol=0)
    ex = O.solve_dynamics_expv(plan, rho0, (0.0, 0.2), saveat=sol["t"], krylovdim=12, atol=1e-12,
                               rtol=1e-10)
    for a, c in zip(sol["states"], ex["states"]):
        assert np.allclose(a, c, atol=2e-9, rtol=0)
    rep = O.solve_dynamics_rk4(plan, rho0, (0.0, 0.2), saveat=[0.0, 0.1, 0.1, 0.2])
    assert np.array_equal(rep["states"][1], rep["states"][2])


def test_arnoldi_spectrum_restatement_matches_dense_spectrum():
    """test/test_krylov.jl:131-136: with krylovdim = dim the Arnoldi Ritz values equal the
    dense spectrum's leading values to 2e-10, residual estimates < 2e-10, and
    |L V - V diag(values)| < 2e-9."""
    plan = O.Plan(_general_model(3, 2))
    L = O.materialize(plan)
    n = L.shape[0]
    dense = np.linalg.eigvals(L)
    dense = dense[O.ritz_order(dense, "LR")]
    arn = O.krylov_liouvillian_spectrum(lambda v: L @ v, n, nev=4, krylovdim=n, vectors=True)
    # conjugate pairs tie in real part, so compare the leading values as sets
    canon = lambda v: v[np.lexsort((np.round(v.imag, 8), np.round(v.real, 8)))]
    assert np.allclose(canon(arn["values"]), canon(dense[:4]), atol=2e-10, rtol=0)
    assert arn["residuals"].max() < 2e-10
    Vv = arn["vectors"]
    assert np.linalg.norm(L @ Vv - Vv * arn["values"][None, :]) < 2e-9
    with pytest.raises(ValueError):
        O.krylov_liouvillian_spectrum(lambda v: L @ v, n, nev=0)
    # duality: <y, L x> = <L^H y, x> and the trace functional is a left null vector
    rng = np.random.default_rng(3)
    x, y = rng.standard_normal(n) + 1j * rng.standard_normal(n), rng.standard_normal(n) + 1j * rng.standard_normal(n)
    LH = O.adjoint_matrix(plan)
    assert abs(np.vdot(y, L @ x) - np.vdot(LH @ y, x)) <= 1e-12 * np.linalg.norm(L) * np.linalg.norm(x) * np.linalg.norm(y)
    t = np.zeros(n, dtype=np.complex128)
    t[plan.trace_idx] = plan.trace_val
    assert np.abs(LH @ t).max() <= 1e-12 * np.abs(L).max()
