"""Adjoint apply (apply_adjoint!) and Arnoldi spectra (krylov_liouvillian_spectrum) on the
GPU against the oracle's conjugate transpose, dense spectrum and Arnoldi restatement."""
import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from tests import models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


CASES = [("driven8", lambda: M.driven_c1(8)), ("general6", lambda: M.general(6, seed=4)),
         ("restricted7", lambda: M.general(7, 5, sectors=[(7, 0), (5, 2)])),
         ("pump_decay6", lambda: picuda.Models.local_pump_decay(6, down=1.0, up=0.3))]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_adjoint_apply_matches_oracle(torch_cuda, name, make):
    torch = torch_cuda
    model = make()
    c = picuda.compile(model)
    LH = O.adjoint_matrix(O.Plan(M.to_oracle(model)))
    X = np.stack([M.random_state_vector(len(model.basis), s) for s in range(3)])
    xd = torch.from_numpy(X).cuda()
    yd = torch.empty_like(xd)
    picuda.apply_adjoint_(yd[0], c, xd[0])
    picuda.apply_adjoint_(yd, c, xd)  # three columns: the batched kernels on the adjoint plan
    torch.cuda.synchronize()
    Y = yd.cpu().numpy()
    for j in range(3):
        ref = LH @ X[j]
        assert np.abs(Y[j] - ref).max() <= 1e-12 * np.abs(ref).max(), (name, j)


def test_adjoint_duality_and_trace_at_scale(torch_cuda):
    """<y, L x> = <L^H y, x> and L^H t = 0 for the trace functional t
    (test_liouvillian_properties.jl:139-168) at N = 60."""
    torch = torch_cuda
    model = M.ensemble_c2(60)
    c = picuda.compile(model)
    n = len(model.basis)
    x = torch.from_numpy(M.random_state_vector(n, 1)).cuda()
    y = torch.from_numpy(M.random_state_vector(n, 2)).cuda()
    Lx, LHy = torch.empty_like(x), torch.empty_like(y)
    picuda.apply_(Lx, c, x)
    picuda.apply_adjoint_(LHy, c, y)
    lhs = complex(torch.vdot(y, Lx).item())
    rhs = complex(torch.vdot(LHy, x).item())
    assert abs(lhs - rhs) <= 1e-12 * float(torch.linalg.norm(Lx)) * float(torch.linalg.norm(y))
    idx, val = c.library_trace_functional()
    t = np.zeros(n, dtype=np.complex128)
    t[idx] = val
    td = torch.from_numpy(t).cuda()
    out = torch.empty_like(td)
    picuda.apply_adjoint_(out, c, td)
    # t holds sqrt(f) (up to ~1e8 at N = 60): measure against |t| times the operator's scale
    op_scale = float(LHy.abs().max()) / float(y.abs().max())
    assert float(out.abs().max()) <= 1e-12 * float(np.abs(t).max()) * op_scale


@pytest.mark.parametrize("N", [4, 6])
def test_spectrum_matches_dense_with_full_krylov_space(torch_cuda, N):
    """test/test_krylov.jl:131-136 on the GPU."""
    model = M.general(N, seed=2)
    plan = O.Plan(M.to_oracle(model))
    L = O.materialize(plan)
    n = L.shape[0]
    dense = np.linalg.eigvals(L)
    dense = dense[O.ritz_order(dense, "LR")]
    arn = picuda.krylov_liouvillian_spectrum(model, nev=4, krylovdim=n, vectors=True,
                                             rng=np.random.default_rng(7))
    canon = lambda v: v[np.lexsort((np.round(v.imag, 8), np.round(v.real, 8)))]
    assert np.allclose(canon(arn["values"]), canon(dense[:4]), atol=2e-10, rtol=0)
    assert arn["residuals"].max() < 2e-10 and arn["converged"].all()
    Vv = arn["vectors"]
    assert np.linalg.norm(L @ Vv - Vv * arn["values"][None, :]) < 2e-9


def test_spectrum_agrees_with_oracle_arnoldi_and_rejects_bad_input(torch_cuda):
    """Same initial vector, partial Krylov space: the converged leading Ritz values agree
    with the oracle's restatement; argument errors follow krylov.jl:920-933."""
    model = M.driven_c1(8)
    oplan = O.Plan(M.to_oracle(model))
    n = len(model.basis)
    v0 = M.random_state_vector(n, 11)
    kw = dict(nev=3, krylovdim=60, initial_vector=v0, require_convergence=False)
    ref = O.krylov_liouvillian_spectrum(lambda v: O.apply(oplan, v), n, **kw)
    got = picuda.krylov_liouvillian_spectrum(model, **kw)
    assert got["iterations"] == ref["iterations"] == 60
    for v, r in zip(got["values"], got["residuals"]):
        if r <= 1e-9:
            assert np.min(np.abs(ref["values"] - v)) <= 1e-8 * max(1.0, abs(v))
    with pytest.raises(picuda.PiArgumentError):
        picuda.krylov_liouvillian_spectrum(model, nev=0)
    with pytest.raises(picuda.PiArgumentError):
        picuda.krylov_liouvillian_spectrum(model, which="XX")
    with pytest.raises(picuda.PiArgumentError):
        picuda.krylov_liouvillian_spectrum(model, initial_vector=np.zeros(n))


# ---- thick-restarted harmonic Arnoldi (harmonic_arnoldi_spectrum, krylov.jl:1378-1551) ----

SM = np.array([[0, 1], [0, 0]], dtype=np.complex128)


@pytest.mark.parametrize("name,make", [("driven8", lambda: M.driven_c1(8)), ("general6", lambda: M.general(6, seed=4))])
def test_harmonic_spectrum_matches_oracle(torch_cuda, name, make):
    """Restarted harmonic Arnoldi (krylovdim 30 < dim) on the device: the values nearest zero
    agree with the oracle's restatement from the same initial vector and with the dense
    spectrum, every residual is below atol + rtol * scale, and the returned Ritz vectors
    satisfy |L x - lambda x| within that tolerance under the oracle's operator."""
    model = make()
    L = O.materialize(O.Plan(M.to_oracle(model)))
    n = L.shape[0]
    v0 = M.random_state_vector(n, 11)
    kw = dict(nev=3, krylovdim=30, maxrestarts=100, initial_vector=v0, vectors=True)
    ref = O.harmonic_arnoldi_spectrum(lambda v: L @ v, n, **kw)
    got = picuda.harmonic_arnoldi_spectrum(model, **kw)
    tol = got["residual_tolerance"]
    assert got["algorithm"] == "harmonic" and got["ritz_extraction"] == "harmonic"
    assert got["converged"].all() and (got["residuals"] <= tol).all()
    assert abs(got["restarts"] - ref["restarts"]) <= 1, (got["restarts"], ref["restarts"])
    assert np.allclose(got["values"], ref["values"], atol=10 * tol, rtol=0), (got["values"], ref["values"])
    dense = np.linalg.eigvals(L)
    for v in got["values"]:
        assert np.abs(dense - v).min() <= 10 * tol + 1e-9
    X = got["vectors"]
    assert X.shape == (n, 3)
    resid = np.linalg.norm(L @ X - X * got["values"][None, :], axis=0)
    assert (resid <= 1.01 * tol + 1e-12).all(), (resid, tol)


def test_harmonic_spectrum_complete_space_and_continuation(torch_cuda):
    """test/test_krylov.jl:154-165 on the device: three qubits with local (0.7) and
    collective (0.2) decay, nev=3, krylovdim=dim, atol=1e-9, rtol=1e-7 -- residuals below
    2e-7 and the stationary value within 3 residuals (+ eps * scale) of the dense one.  The
    Ritz vectors then seed a second solve as an initial subspace (the spectral scan's
    continuation), which retains all three and returns the same values."""
    model = picuda.PIModel(picuda.PIBasis(3, 2), [picuda.LocalJump(SM, rate=0.7), picuda.CollectiveJump(SM, rate=0.2)])
    L = O.materialize(O.Plan(M.to_oracle(model)))
    n = L.shape[0]
    dense = np.linalg.eigvals(L)
    dense = dense[O.ritz_order(dense, "LR")]
    h = picuda.harmonic_arnoldi_spectrum(model, nev=3, krylovdim=n, initial_vector=M.random_state_vector(n, 10),
                                         vectors=True, atol=1e-9, rtol=1e-7)
    assert h["residuals"].max() < 2e-7
    assert h["search_space_exhausted"] and h["ritz_extraction"] == "rayleigh_ritz"
    i = int(np.argmin(np.abs(h["values"] - dense[0])))
    floor = np.finfo(float).eps * max(1.0, h["residual_scale"])
    assert abs(h["values"][i] - dense[0]) <= 3 * h["residuals"][i] + floor
    again = picuda.harmonic_arnoldi_spectrum(model, nev=3, krylovdim=n, initial_subspace=h["vectors"],
                                             atol=1e-9, rtol=1e-7)
    assert again["initial_retained_dimension"] == 3
    assert np.allclose(np.sort_complex(again["values"]), np.sort_complex(h["values"]), atol=1e-6, rtol=0)
    with pytest.raises(picuda.PiArgumentError, match="symmetry projectors"):
        picuda.harmonic_arnoldi_spectrum(model, projector=np.eye(n))
    with pytest.raises(picuda.PiArgumentError):
        picuda.harmonic_arnoldi_spectrum(model, nev=n + 1)
    with pytest.raises(picuda.PiArgumentError, match="zero component"):
        picuda.harmonic_arnoldi_spectrum(model, nev=2, initial_vector=np.zeros(n))


def test_harmonic_spectral_scan_continuation(torch_cuda):
    """test/test_compiled_families.jl:170-188: a near-zero spectral scan of a one-qubit family
    (decay 1.0, pumping p) with HarmonicArnoldiAlgorithm(nev=2, krylovdim=4, thickdim=2,
    maxrestarts=4) warm-starts the second point from both Ritz vectors of the first and
    keeps the restart seed as a matrix."""
    spin = picuda.spin_matrices()
    fam = picuda.compile_family(picuda.PIModel(picuda.PIBasis(1, 2), [picuda.LocalJump(spin["jm"], rate=1.0),
                                                                      picuda.LocalJump(spin["jp"], rate=0.2)]))
    alg = picuda.HarmonicArnoldiAlgorithm(nev=2, krylovdim=4, thickdim=2, maxrestarts=4)
    plan = picuda.ParameterScanPlan([0.2, 0.25], fam, rate_builder=lambda p: (1.0, p), task="spectrum",
                                    algorithm=alg, spectrum_target="near_zero", nev=2, save_vectors=False,
                                    solver_options=dict(require_convergence=False))
    res = picuda.parameter_scan(plan, on_error="throw")
    assert [p.status for p in res] == ["success", "success"]
    assert res.points[1].warm_started
    assert res.points[1].diagnostics["solver"]["initial_retained_dimension"] == 2
    assert isinstance(res.restart_seed, np.ndarray) and res.restart_seed.shape == (4, 2)
    # the slowest modes of decay 1 and pumping p: 0 and -(1 + p)/2
    for p, pt in zip([0.2, 0.25], res.points):
        vals = pt.output["values"]
        assert abs(vals[0]) <= 1e-9
        assert abs(vals[1] + (1 + p) / 2) <= 1e-9


def test_liouvillian_gap_from_device_arnoldi(torch_cuda):
    """test/test_krylov.jl:145-152 on the device: method=:krylov, nev=4, krylovdim=dim gives
    the dense gap (spectra.jl:289-308 on the oracle's matrix) to 2e-10 with the stationary
    count certified; the driven N=8 system's gap agrees with its dense gap as well."""
    model = picuda.PIModel(picuda.PIBasis(3, 2), [picuda.LocalJump(SM, rate=0.7), picuda.CollectiveJump(SM, rate=0.2)])
    for m in (model, M.driven_c1(8)):
        L = O.materialize(O.Plan(M.to_oracle(m)))
        n = L.shape[0]
        vals = np.linalg.eigvals(L)
        tol = 1e-12 + 1e-10 * max(np.abs(vals).max(), 1.0)
        dense_gap = -max(v.real for v in vals if abs(v) > tol)
        info = picuda.pi_liouvillian_gap(m, method="krylov", nev=4, krylovdim=min(n, 120), return_info=True,
                                         initial_vector=M.random_state_vector(n, 3))
        assert abs(info["gap"] - dense_gap) <= 2e-10, (info["gap"], dense_gap)
        assert info["method"] == "arnoldi" and info["stationary_multiplicity_certified"]
    with pytest.raises(picuda.PiArgumentError):
        picuda.pi_liouvillian_gap(model, method="krylov", symmetry="auto")


def test_liouvillian_spectrum_high_level(torch_cuda):
    """liouvillian_spectrum (highlevel.jl:735-835) on the device: near zero it selects
    harmonic Arnoldi, otherwise Arnoldi; with the default krylovdim = dim of the three-qubit
    model both return the dense spectrum's selected values."""
    model = picuda.PIModel(picuda.PIBasis(3, 2), [picuda.LocalJump(SM, rate=0.7), picuda.CollectiveJump(SM, rate=0.2)])
    L = O.materialize(O.Plan(M.to_oracle(model)))
    n = L.shape[0]
    dense = np.linalg.eigvals(L)
    near = picuda.liouvillian_spectrum(model, target="near_zero", nev=3, return_info=True, vectors=True)
    assert near.info["selected_algorithm"] == "harmonic" and near.vectors.shape == (n, 3)
    for v in near.values:
        assert np.abs(dense - v).min() <= 1e-6
    assert abs(near.values[0]) <= 1e-9
    lr = picuda.liouvillian_spectrum(model, nev=3)
    ref = dense[np.argsort(-dense.real, kind="stable")][:3]
    assert np.allclose(np.sort_complex(lr), np.sort_complex(ref), atol=1e-6, rtol=0)


def test_implicitly_restarted_arnoldi_on_device(torch_cuda):
    """implicitly_restarted_arnoldi_spectrum (krylov.jl:996-1110) with the basis on the GPU:
    krylovdim 40 on the driven N=8 system (dim 165) needs restarts, and every projection spans
    more than one group of 32 basis vectors of the allocation-free multi-dot.  The values
    match the dense spectrum and the oracle's restatement run from the same initial vector,
    and the device Ritz vectors satisfy |L v - lambda v| within the reported residuals."""
    torch = torch_cuda
    model = M.driven_c1(8)
    oplan = O.Plan(M.to_oracle(model))
    L = O.materialize(oplan)
    n = L.shape[0]
    dense = np.linalg.eigvals(L)
    dense = dense[O.ritz_order(dense, "LR")]
    v0 = M.random_state_vector(n, 21)
    res = picuda.implicitly_restarted_arnoldi_spectrum(model, nev=4, krylovdim=40, which="LR", initial_vector=v0,
                                                       vectors=True, atol=1e-10, rtol=1e-8)
    ref = O.implicitly_restarted_arnoldi_spectrum(lambda v: L @ v, n, nev=4, krylovdim=40, which="LR",
                                                  initial_vector=v0, atol=1e-10, rtol=1e-8, vectors=True)
    assert res["restarts"] >= 1
    assert res["converged"].all()
    # the last convergence test sits near its tolerance, so rounding may move it by a cycle
    assert abs(res["restarts"] - ref["restarts"]) <= 1
    assert np.allclose(res["values"], ref["values"], atol=1e-8, rtol=0)
    for v, rv in zip(res["values"], res["residuals"]):
        assert np.abs(dense - v).min() <= 3 * rv + 1e-9
    X = res["vectors"]
    assert X.shape == (n, 4)
    for j, lam in enumerate(res["values"]):
        x = X[:, j]
        r = np.linalg.norm(L @ x - lam * x) / np.linalg.norm(x)
        # the Hessenberg estimate omits the rounding of the restarted basis: allow 1e-8 of
        # the operator scale on top of it
        assert r <= 10 * res["residuals"][j] + 1e-8 * res["residual_scale"], (j, r, res["residuals"][j])
    # the spectral entry points that select it
    lr = picuda.liouvillian_spectrum(model, nev=3, algorithm="iram", krylovdim=40)
    assert len(lr) == 3
    for v in lr:  # the third value is one of a conjugate pair of equal real part
        assert np.abs(dense[:4] - v).min() <= 1e-7
    vals = np.linalg.eigvals(L)
    tol = 1e-12 + 1e-10 * max(np.abs(vals).max(), 1.0)
    dense_gap = -max(v.real for v in vals if abs(v) > tol)
    info = picuda.pi_liouvillian_gap(model, method="iram", nev=4, krylovdim=40, return_info=True,
                                     initial_vector=M.random_state_vector(n, 3))
    assert abs(info["gap"] - dense_gap) <= 1e-7, (info["gap"], dense_gap)
