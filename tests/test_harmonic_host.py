"""Thick-restarted harmonic Arnoldi (harmonic_arnoldi_spectrum, krylov.jl:1378-1551) on the CPU.

Three layers, no GPU:
  * the oracle's restatement pinned to the reference's own known answers
    (test/test_krylov.jl:154-214);
  * the library's algorithm (picuda.backend._harmonic_arnoldi) run over a numpy vector
    space that stands in for the device one, against the oracle on the same operator and
    starting vectors -- the same host logic the GPU path drives through pi_apply_f64,
    pi_mdot_f64_noalloc and pi_combine_f64;
  * argument checks and the algorithm record (HarmonicArnoldiAlgorithm, highlevel.jl:126-150).
"""
import ctypes as C

import numpy as np
import pytest

import picuda
from picuda import backend as B
from oracle import pi_oracle as O

SM = np.array([[0, 1], [0, 0]], dtype=np.complex128)


class NumpySpace:
    """The vector operations of the device Krylov space over numpy rows."""

    def __init__(self, A):
        self.A = A
        self.n = A.shape[0]
        self.applications = 0

    def block(self, m):
        return np.zeros((m, self.n), dtype=np.complex128)

    def upload(self, v):
        return np.array(v, dtype=np.complex128)

    def copy(self, v):
        return v.copy()

    def download(self, rows):
        return rows.T.copy()

    def apply(self, dst, src):
        dst[:] = self.A @ src
        self.applications += 1

    def dots(self, M, k, q):
        return M[:k].conj() @ q

    def norm(self, q):
        return float(np.linalg.norm(q))

    def combine(self, M, k, Y):
        return (M[:k].T @ np.asarray(Y)).T.copy()

    def subtract(self, q, M, k, coef):
        q -= M[:k].T @ coef


def _host_harmonic(A, nev=6, krylovdim=None, thickdim=None, maxrestarts=20, target=0, initial_vector=None,
                   initial_subspace=None, atol=1e-10, rtol=1e-8, vectors=False, seed=0, require_convergence=True):
    n = A.shape[0]
    kd, td, t, v0, s0 = B._check_harmonic_arguments(n, nev, krylovdim, thickdim, maxrestarts, target,
                                                    initial_vector, initial_subspace, None)
    return B._harmonic_arnoldi(NumpySpace(A), n, nev, kd, td, maxrestarts, t, v0, s0, atol, rtol, vectors,
                               np.random.default_rng(seed), require_convergence)


def _pi_matrix():
    """test/test_krylov.jl:2-4: three qubits with local (0.7) and collective (0.2) decay."""
    model = O.PIModel(O.PIBasis(3, 2), [O.LocalJump(SM, 0.7), O.CollectiveJump(SM, 0.2)])
    return O.materialize(O.Plan(model))


def _nonnormal(n, seed):
    rng = np.random.default_rng(seed)
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    return A - 2.5 * np.eye(n)


def _seed(n, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


# ---- the oracle against the reference's known answers ---------------------------------

def test_oracle_harmonic_stationary_mode():
    """test/test_krylov.jl:154-165: nev=3, krylovdim=dim, atol=1e-9, rtol=1e-7 -> residuals
    below 2e-7 and the stationary value within 3 residuals (+ eps * scale) of the dense one."""
    L = _pi_matrix()
    n = L.shape[0]
    dense = np.linalg.eigvals(L)
    dense = dense[O.ritz_order(dense, "LR")]
    h = O.harmonic_arnoldi_spectrum(lambda v: L @ v, n, nev=3, krylovdim=n, initial_vector=_seed(n, 10),
                                    vectors=True, atol=1e-9, rtol=1e-7)
    assert h["residuals"].max() < 2e-7
    i = int(np.argmin(np.abs(h["values"] - dense[0])))
    floor = np.finfo(float).eps * max(1.0, h["residual_scale"])
    assert abs(h["values"][i] - dense[0]) <= 3 * h["residuals"][i] + floor
    assert h["algorithm"] == "harmonic"


def test_oracle_harmonic_complete_space_uses_rayleigh_ritz():
    """test/test_krylov.jl:170-192: the nonnormal 4 x 4 operator whose harmonic pencil is
    singular at zero.  The reference restricts it to a two-dimensional symmetry sector; with
    no projector the whole space is the range, and once it is spanned the extraction is
    Rayleigh-Ritz with the same two values nearest zero, 0 and -0.7."""
    L = np.zeros((4, 4), dtype=np.complex128)
    L[0, 3], L[3, 3], L[1, 1], L[2, 2] = 1, -0.7, -2, -3
    h = O.harmonic_arnoldi_spectrum(lambda v: L @ v, 4, nev=2, krylovdim=4, maxrestarts=0,
                                    initial_vector=np.array([1, 2, 3, 4], dtype=np.complex128), vectors=True,
                                    atol=1e-12, rtol=1e-10)
    assert np.allclose(h["values"], [0, -0.7], atol=1e-11, rtol=0)
    assert h["residuals"].max() < 1e-11
    X = h["vectors"]
    assert np.linalg.norm(L @ X - X * h["values"][None, :]) < 2e-11
    assert h["ritz_extraction"] == "rayleigh_ritz" and h["search_space_exhausted"]


def test_oracle_harmonic_restarts():
    """test/test_krylov.jl:209-214: krylovdim 8 with atol = rtol = 0 runs every restart."""
    L = _pi_matrix()
    n = L.shape[0]
    h = O.harmonic_arnoldi_spectrum(lambda v: L @ v, n, nev=2, krylovdim=8, initial_vector=_seed(n, 10),
                                    maxrestarts=2, require_convergence=False, atol=0, rtol=0)
    assert h["restarts"] == 2
    assert h["ritz_extraction"] == "harmonic" and not h["search_space_exhausted"]


def test_oracle_harmonic_restarted_converges_to_nearest_eigenvalues():
    A = _nonnormal(60, 3)
    ev = np.linalg.eigvals(A)
    ev = ev[np.argsort(np.abs(ev))]
    h = O.harmonic_arnoldi_spectrum(lambda v: A @ v, 60, nev=3, krylovdim=20, maxrestarts=200,
                                    initial_vector=_seed(60, 1))
    assert h["restarts"] > 0
    assert np.allclose(h["values"], ev[:3], atol=1e-7, rtol=0)


# ---- the library's algorithm over a numpy vector space against the oracle ---------------

# Value tolerance per case: two converged runs agree to about the residual tolerance times
# the eigenvalues' condition; the restarted PI case holds the nonnormal pair -0.65 / -0.7
# (condition ~1e2 at a residual tolerance of 3e-8).
@pytest.mark.parametrize("case,vtol", [("pi_full", 1e-9), ("pi_restarted", 1e-5), ("nonnormal", 1e-8),
                                       ("target", 1e-8)])
def test_library_harmonic_matches_oracle(case, vtol):
    if case == "pi_full":
        A, kw = _pi_matrix(), dict(nev=3, atol=1e-9, rtol=1e-7)
        kw["krylovdim"] = A.shape[0]
    elif case == "pi_restarted":
        A, kw = _pi_matrix(), dict(nev=3, krylovdim=10, maxrestarts=100)
    elif case == "nonnormal":
        A, kw = _nonnormal(60, 3), dict(nev=3, krylovdim=20, maxrestarts=200)
    else:
        A, kw = _nonnormal(50, 5), dict(nev=4, krylovdim=24, target=-2.0 + 0.5j, maxrestarts=200)
    n = A.shape[0]
    v0 = _seed(n, 11)
    ref = O.harmonic_arnoldi_spectrum(lambda v: A @ v, n, initial_vector=v0, vectors=True, **kw)
    got = _host_harmonic(A, initial_vector=v0, vectors=True, **kw)
    assert got["restarts"] == ref["restarts"]
    assert got["ritz_extraction"] == ref["ritz_extraction"]
    assert got["iterations"] == ref["iterations"]
    assert np.allclose(got["values"], ref["values"], atol=vtol, rtol=0)
    # each value is an eigenvalue (the PI case's -0.65 is a defective double eigenvalue with
    # one eigenvector, so the values nearest zero are 0, -0.65 and -0.7)
    dense = np.linalg.eigvals(A)
    for v in got["values"]:
        assert np.abs(dense - v).min() <= max(vtol, 10 * got["residual_tolerance"])
    assert (got["residuals"] <= got["residual_tolerance"]).all()
    X = got["vectors"]
    resid = np.linalg.norm(A @ X - X * got["values"][None, :], axis=0)
    assert (resid <= 1.01 * got["residual_tolerance"] + 1e-12).all()


def test_library_harmonic_subspace_continuation():
    """A converged set of Ritz vectors as initial_subspace (the spectral scan's continuation,
    scans.jl:983-1000, 1020-1025) converges in the first cycle with the same values."""
    A = _nonnormal(60, 3)
    first = _host_harmonic(A, nev=3, krylovdim=20, maxrestarts=200, initial_vector=_seed(60, 1), vectors=True)
    again = _host_harmonic(A, nev=3, krylovdim=20, maxrestarts=200, initial_subspace=first["vectors"])
    assert again["initial_retained_dimension"] == 3
    assert again["restarts"] <= first["restarts"]
    assert np.allclose(again["values"], first["values"], atol=1e-7, rtol=0)
    ref = O.harmonic_arnoldi_spectrum(lambda v: A @ v, 60, nev=3, krylovdim=20, maxrestarts=200,
                                      initial_subspace=first["vectors"])
    assert np.allclose(again["values"], ref["values"], atol=1e-9, rtol=0)


def test_library_harmonic_not_converged():
    A = _nonnormal(60, 3)
    with pytest.raises(picuda.PiArgumentError, match="did not converge in 1 restarts"):
        _host_harmonic(A, nev=3, krylovdim=8, maxrestarts=1, initial_vector=_seed(60, 1), atol=0, rtol=0)
    out = _host_harmonic(A, nev=3, krylovdim=8, maxrestarts=1, initial_vector=_seed(60, 1), atol=0, rtol=0,
                         require_convergence=False, vectors=True)
    assert out["restarts"] == 1 and not out["converged"].any()
    assert out["vectors"].shape == (60, 3)
    assert [r["cycle"] for r in out["restart_history"]] == [0, 1]


# ---- argument checks -----------------------------------------------------------------------

def test_harmonic_argument_checks():
    chk = B._check_harmonic_arguments
    with pytest.raises(picuda.PiArgumentError, match="symmetry projectors"):
        chk(10, 2, None, None, 20, 0, None, None, np.eye(10))
    with pytest.raises(picuda.PiArgumentError, match="nev must lie"):
        chk(10, 0, None, None, 20, 0, None, None, None)
    with pytest.raises(picuda.PiArgumentError, match="nev must lie"):
        chk(10, 11, None, None, 20, 0, None, None, None)
    with pytest.raises(picuda.PiArgumentError, match="maxrestarts"):
        chk(10, 2, None, None, -1, 0, None, None, None)
    with pytest.raises(picuda.PiArgumentError, match="finite"):
        chk(10, 2, None, None, 20, complex(np.inf, 0), None, None, None)
    with pytest.raises(picuda.PiArgumentError, match="mutually exclusive"):
        chk(10, 2, None, None, 20, 0, np.ones(10), np.ones((10, 1)), None)
    with pytest.raises(picuda.PiDimensionMismatch):
        chk(10, 2, None, None, 20, 0, np.ones(9), None, None)
    with pytest.raises(picuda.PiDimensionMismatch):
        chk(10, 2, None, None, 20, 0, None, np.ones((9, 2)), None)
    with pytest.raises(picuda.PiArgumentError, match="zero columns"):
        chk(10, 2, None, None, 20, 0, None, np.ones((10, 0)), None)
    with pytest.raises(picuda.PiArgumentError, match="up to 128"):
        chk(1000, 2, 129, None, 20, 0, None, None, None)
    assert chk(1000, 6, None, None, 20, 0, None, None, None)[:2] == (30, 12)
    assert chk(10, 2, None, None, 20, 0, None, None, None)[:2] == (30, 4)
    with pytest.raises(picuda.PiArgumentError, match="zero component"):
        _host_harmonic(np.eye(5, dtype=np.complex128), nev=1, initial_vector=np.zeros(5))
    with pytest.raises(picuda.PiArgumentError, match="no independent component"):
        _host_harmonic(np.eye(5, dtype=np.complex128), nev=1, initial_subspace=np.zeros((5, 2)))


def test_harmonic_algorithm_record():
    a = picuda.HarmonicArnoldiAlgorithm()
    assert (a.nev, a.krylovdim, a.thickdim, a.maxrestarts) == (6, 30, 12, 20)
    a = picuda.HarmonicArnoldiAlgorithm(nev=12)
    assert (a.krylovdim, a.thickdim) == (42, 24)
    with pytest.raises(picuda.PiArgumentError, match="Bool"):
        picuda.HarmonicArnoldiAlgorithm(nev=True)
    with pytest.raises(picuda.PiArgumentError, match="at least 0"):
        picuda.HarmonicArnoldiAlgorithm(maxrestarts=-1)
    with pytest.raises(picuda.PiArgumentError, match="at least 1"):
        picuda.HarmonicArnoldiAlgorithm(krylovdim=0)


def test_near_zero_spectral_scan_host_logic(monkeypatch):
    """The spectral scan's harmonic branch (scans.jl:974-1053) with the device solve replaced
    by the library's algorithm over a numpy space: test/test_compiled_families.jl:170-188's
    one-qubit family (decay 1.0, pumping p) warm-starts the second point from both Ritz
    vectors of the first and keeps the restart seed as a matrix."""
    import types
    from picuda import scans as S
    from tests import models as M
    spin = picuda.spin_matrices()
    fam = picuda.compile_family(picuda.PIModel(picuda.PIBasis(1, 2), [picuda.LocalJump(spin["jm"], rate=1.0),
                                                                      picuda.LocalJump(spin["jp"], rate=0.2)]))
    seen = []

    def compile_point(plan, parameter, index):
        made = plan.model_builder(parameter, index)
        model = S._family_model(made.family, S._family_rates(made.family, made.rates))
        return types.SimpleNamespace(basis=model.basis, matrix=O.materialize(O.Plan(M.to_oracle(model))))

    def solve(compiled, nev=6, krylovdim=None, thickdim=None, maxrestarts=20, target=0, initial_vector=None,
              initial_subspace=None, atol=1e-10, rtol=1e-8, vectors=False, rng=None, require_convergence=True):
        n = len(compiled.basis)
        kd, td, t, v0, s0 = B._check_harmonic_arguments(n, nev, krylovdim, thickdim, maxrestarts, target,
                                                        initial_vector, initial_subspace, None)
        seen.append(dict(nev=nev, krylovdim=kd, thickdim=td, maxrestarts=maxrestarts, warm=s0 is not None))
        return B._harmonic_arnoldi(NumpySpace(compiled.matrix), n, nev, kd, td, maxrestarts, t, v0, s0, atol, rtol,
                                   vectors, rng, require_convergence)

    monkeypatch.setattr(S, "_compile_point", compile_point)
    monkeypatch.setattr(B, "harmonic_arnoldi_spectrum", solve)
    alg = picuda.HarmonicArnoldiAlgorithm(nev=2, krylovdim=4, thickdim=2, maxrestarts=4)
    plan = picuda.ParameterScanPlan([0.2, 0.25], fam, rate_builder=lambda p: (1.0, p), task="spectrum",
                                    algorithm=alg, spectrum_target="near_zero", nev=2, save_vectors=False,
                                    solver_options=dict(require_convergence=False))
    res = picuda.parameter_scan(plan, on_error="throw")
    assert [p.status for p in res] == ["success", "success"]
    assert seen == [dict(nev=2, krylovdim=4, thickdim=2, maxrestarts=4, warm=False),
                    dict(nev=2, krylovdim=4, thickdim=2, maxrestarts=4, warm=True)]
    assert res.points[1].warm_started and not res.points[0].warm_started
    assert res.points[1].diagnostics["solver"]["initial_retained_dimension"] == 2
    assert res.points[1].diagnostics["method"] == "harmonic"
    assert isinstance(res.restart_seed, np.ndarray) and res.restart_seed.shape == (4, 2)
    for p, pt in zip([0.2, 0.25], res.points):
        vals = pt.output["values"]
        assert pt.output["vectors"] is None
        assert abs(vals[0]) <= 1e-9
        assert abs(vals[1] + (1 + p) / 2) <= 1e-9


# ---- the Liouvillian gap (pi_liouvillian_gap, spectra.jl:262-470) ------------------------

def _dense_gap(L, atol=1e-12, rtol=1e-10):
    """spectra.jl:289-308 on the dense spectrum (the reference's default method=:dense)."""
    vals = np.linalg.eigvals(L)
    tol = atol + rtol * max(np.abs(vals).max(), 1.0)
    return -max(v.real for v in vals if abs(v) > tol)


def test_gap_info_known_values():
    """spectra.jl:289-308: the oscillatory counterexample of test/test_krylov.jl:324-330
    (gap 0.1 from -0.1+100i, not the -1 mode), the stationary-count and stability rules."""
    info = B._liouvillian_gap_info([0, -0.1 + 100j, -1], 1e-12, 1e-10, True)
    assert abs(info["gap"] - 0.1) < 1e-15 and info["oscillation_frequency"] == 100.0
    assert info["stationary_multiplicity"] == 1 and info["unique_stationary_mode"] and info["stable"]
    assert info["decay_eigenvalue"] == -0.1 + 100j
    with pytest.raises(picuda.PiArgumentError, match="no stationary eigenvalue"):
        B._liouvillian_gap_info([-1.0, -2.0], 1e-12, 1e-10, True)
    with pytest.raises(picuda.PiArgumentError, match="unstable"):
        B._liouvillian_gap_info([0.0, 0.5, -1.0], 1e-12, 1e-10, True)
    info = B._liouvillian_gap_info([0.0, 0.5, -1.0], 1e-12, 1e-10, False)
    assert not info["stable"] and info["gap"] == -0.5
    info = B._liouvillian_gap_info([0.0, 1e-13], 1e-12, 1e-10, True)
    assert info["gap"] == float("inf") and info["decay_eigenvalue"] is None
    assert info["stationary_multiplicity"] == 2 and not info["unique_stationary_mode"]


def test_gap_from_arnoldi_host_logic(monkeypatch):
    """test/test_krylov.jl:145-152 with the device Arnoldi replaced by the oracle's
    restatement: method=:krylov, nev=4, krylovdim=dim gives the dense gap to 2e-10 with the
    stationary count certified; a symmetry with method=:krylov is rejected."""
    L = _pi_matrix()
    n = L.shape[0]

    def spectrum(x, nev=6, krylovdim=None, which="LR", initial_vector=None, atol=1e-10, rtol=1e-8, vectors=False,
                 rng=None, require_convergence=True):
        assert x == "model" and which == "LR"
        return O.krylov_liouvillian_spectrum(lambda v: L @ v, n, nev=nev, krylovdim=krylovdim, which=which,
                                             initial_vector=initial_vector, atol=atol, rtol=rtol,
                                             require_convergence=require_convergence)

    monkeypatch.setattr(B, "krylov_liouvillian_spectrum", spectrum)
    info = picuda.pi_liouvillian_gap("model", method="krylov", nev=4, krylovdim=n, return_info=True)
    assert abs(info["gap"] - _dense_gap(L)) <= 2e-10
    assert info["method"] == "arnoldi" and info["stationary_multiplicity_certified"]
    assert info["scope"] == "global" and info["selection"] == "largest_real" and info["dimension"] == n
    assert picuda.pi_liouvillian_gap("model", nev=4, krylovdim=n) == info["gap"]
    with pytest.raises(picuda.PiArgumentError, match="symmetry"):
        picuda.pi_liouvillian_gap("model", method="krylov", symmetry="auto")
    with pytest.raises(picuda.PiArgumentError, match="cannot certify"):
        picuda.pi_liouvillian_gap("model", method="harmonic")
    with pytest.raises(picuda.PiArgumentError, match="method=:krylov"):
        picuda.pi_liouvillian_gap("model", method="dense")


# ---- the high-level spectral command (liouvillian_spectrum, highlevel.jl:735-835) ---------

def test_liouvillian_spectrum_dispatch(monkeypatch):
    """Automatic selection (highlevel.jl:735-746): harmonic Arnoldi near zero, Arnoldi
    otherwise; an explicit Arnoldi request near zero orders by smallest modulus; the
    HarmonicArnoldiAlgorithm record fixes nev and the Krylov sizes.  The device solvers are
    replaced by the oracle's Arnoldi and the library's harmonic algorithm over numpy."""
    import types
    L = _nonnormal(40, 7)  # a nonnormal matrix stands in for a compiled plan
    n = L.shape[0]
    calls = []

    def arnoldi(compiled, nev=6, krylovdim=None, which="LR", initial_vector=None, atol=1e-10, rtol=1e-8,
                vectors=False, rng=None, require_convergence=True):
        calls.append(("arnoldi", which, nev, krylovdim))
        return O.krylov_liouvillian_spectrum(lambda v: L @ v, n, nev=nev, krylovdim=krylovdim, which=which,
                                             atol=atol, rtol=rtol, vectors=vectors, rng=rng,
                                             require_convergence=require_convergence)

    def harmonic(compiled, nev=6, krylovdim=None, thickdim=None, maxrestarts=20, target=0, initial_vector=None,
                 initial_subspace=None, atol=1e-10, rtol=1e-8, vectors=False, rng=None, require_convergence=True):
        calls.append(("harmonic", nev, krylovdim, thickdim, maxrestarts))
        kd, td, t, v0, s0 = B._check_harmonic_arguments(n, nev, krylovdim, thickdim, maxrestarts, target,
                                                        initial_vector, initial_subspace, None)
        return B._harmonic_arnoldi(NumpySpace(L), n, nev, kd, td, maxrestarts, t, v0, s0, atol, rtol, vectors, rng,
                                   require_convergence)

    monkeypatch.setattr(B, "_as_compiled", lambda x: types.SimpleNamespace(basis=range(n)))
    monkeypatch.setattr(B, "krylov_liouvillian_spectrum", arnoldi)
    monkeypatch.setattr(B, "harmonic_arnoldi_spectrum", harmonic)
    dense = np.linalg.eigvals(L)

    near = picuda.liouvillian_spectrum("plan", target="near_zero", nev=3, maxrestarts=200, return_info=True)
    assert calls[-1] == ("harmonic", 3, 20, None, 200)
    assert isinstance(near, picuda.SpectrumResult) and near.vectors is None
    assert near.info["selected_algorithm"] == "harmonic" and near.info["requested_algorithm"] == "auto"
    nearest = dense[np.argsort(np.abs(dense), kind="stable")][:3]
    assert np.allclose(np.sort_complex(near.values), np.sort_complex(nearest), atol=1e-7, rtol=0)

    lr = picuda.liouvillian_spectrum("plan", nev=2, krylovdim=n)
    assert calls[-1] == ("arnoldi", "LR", 2, n)
    assert np.allclose(lr, dense[np.argsort(-dense.real, kind="stable")][:2], atol=1e-9, rtol=0)
    lm = picuda.liouvillian_spectrum("plan", target="largest_magnitude", nev=2, krylovdim=n, vectors=True)
    assert calls[-1] == ("arnoldi", "LM", 2, n)
    assert set(lm) == {"values", "vectors"} and lm["vectors"].shape == (n, 2)
    picuda.liouvillian_spectrum("plan", target="near_zero", algorithm="arnoldi", nev=2, krylovdim=n)
    assert calls[-1] == ("arnoldi", "SM", 2, n)
    alg = picuda.HarmonicArnoldiAlgorithm(nev=2, krylovdim=12, maxrestarts=300)
    out = picuda.liouvillian_spectrum("plan", nev=5, algorithm=alg)
    assert calls[-1] == ("harmonic", 2, 12, 4, 300) and out.shape == (2,)

    with pytest.raises(picuda.PiArgumentError, match="target must be"):
        picuda.liouvillian_spectrum("plan", target="smallest")
    with pytest.raises(picuda.PiArgumentError, match="unsupported spectrum algorithm"):
        picuda.liouvillian_spectrum("plan", algorithm="dense")
    with pytest.raises(picuda.PiArgumentError, match="Bool"):
        picuda.liouvillian_spectrum("plan", nev=True)
    with pytest.raises(picuda.PiArgumentError, match="positive"):
        picuda.liouvillian_spectrum("plan", nev=0)
    with pytest.raises(picuda.PiArgumentError, match="exceeds the source dimension"):
        picuda.liouvillian_spectrum("plan", algorithm=picuda.HarmonicArnoldiAlgorithm(nev=n + 1))


def test_arnoldi_spectral_scan_continuation_host_logic(monkeypatch):
    """The spectral scan's Arnoldi branch (scans.jl:983-1041) with the device process
    replaced by the oracle's restatement: the second point starts from v_1 + sum_c v_c / c
    of the first point's Ritz vectors, normalised, and the restart seed is that vector."""
    import types
    from picuda import scans as S
    from tests import models as M
    spin = picuda.spin_matrices()
    fam = picuda.compile_family(picuda.PIModel(picuda.PIBasis(3, 2), [picuda.LocalJump(spin["jm"], rate=1.0),
                                                                      picuda.LocalJump(spin["jp"], rate=0.2)]))
    seeds = []

    def compile_point(plan, parameter, index):
        made = plan.model_builder(parameter, index)
        model = S._family_model(made.family, S._family_rates(made.family, made.rates))
        return types.SimpleNamespace(basis=model.basis, matrix=O.materialize(O.Plan(M.to_oracle(model))))

    def arnoldi(compiled, nev=6, krylovdim=None, which="LR", initial_vector=None, atol=1e-10, rtol=1e-8,
                vectors=False, rng=None, require_convergence=True):
        seeds.append(None if initial_vector is None else np.array(initial_vector))
        n = len(compiled.basis)
        return O.krylov_liouvillian_spectrum(lambda v: compiled.matrix @ v, n, nev=nev, krylovdim=krylovdim,
                                             which=which, initial_vector=initial_vector, atol=atol, rtol=rtol,
                                             vectors=vectors, rng=rng, require_convergence=require_convergence)

    monkeypatch.setattr(S, "_compile_point", compile_point)
    monkeypatch.setattr(B, "krylov_liouvillian_spectrum", arnoldi)
    plan = picuda.ParameterScanPlan([0.2, 0.3], fam, rate_builder=lambda p: (1.0, p), task="spectrum", nev=3,
                                    save_vectors=True, solver_options={"krylovdim": 20})
    res = picuda.parameter_scan(plan, on_error="throw")
    assert [p.warm_started for p in res] == [False, True]
    assert seeds[0] is None
    expected = S._arnoldi_continuation(res.points[0].output["vectors"])
    assert np.array_equal(seeds[1], expected)
    assert np.array_equal(res.restart_seed, S._arnoldi_continuation(res.points[1].output["vectors"]))
    assert res.points[1].diagnostics["method"] == "arnoldi"


# ---- implicitly restarted Arnoldi (krylov.jl:996-1110) -------------------------------------

class TorchCpuSpace(NumpySpace):
    """The device space's tensor semantics on CPU torch tensors: rows of complex128 tensors,
    in-place row updates and Python-scalar arithmetic as on the GPU; the reductions and
    combinations follow the C-ABI layouts (coefficients k x c column-major)."""

    def __init__(self, A):
        super().__init__(A)
        self.torch = pytest.importorskip("torch")
        self.At = self.torch.from_numpy(A)

    def block(self, m):
        return self.torch.zeros((m, self.n), dtype=self.torch.complex128)

    def upload(self, v):
        return self.torch.from_numpy(np.ascontiguousarray(v, dtype=np.complex128)).clone()

    def copy(self, v):
        return v.clone()

    def download(self, rows):
        return rows.numpy().T.copy()

    def apply(self, dst, src):
        assert dst.is_contiguous() and src.is_contiguous() and dst.shape == src.shape == (self.n,)
        dst.copy_(self.At @ src)

    def dots(self, M, k, q):
        assert q.is_contiguous() and M[0].is_contiguous()
        return (M[:k].conj() @ q).numpy()

    def norm(self, q):
        return float(self.torch.linalg.vector_norm(q))

    def combine(self, M, k, Y):
        Yc = np.ascontiguousarray(np.asarray(Y, dtype=np.complex128).T)  # the layout the C-ABI receives
        coef = self.torch.from_numpy(Yc.reshape(-1)).reshape(Yc.shape[0], k)
        return (coef @ M[:k]).contiguous()

    def subtract(self, q, M, k, coef):
        q.sub_(self.torch.from_numpy(np.ascontiguousarray(coef, dtype=np.complex128)) @ M[:k])


def _host_iram(space, n, nev=6, krylovdim=None, retained_dimension=None, maxrestarts=20, which="LR", target=None,
               initial_vector=None, atol=1e-10, rtol=1e-8, vectors=False, require_convergence=True):
    kd = max(30, 3 * nev + 6) if krylovdim is None else krylovdim
    rd = max(nev, min(2 * nev, kd - 1)) if retained_dimension is None else retained_dimension
    return B._iram(space, n, nev, kd, rd, maxrestarts, which, None if target is None else complex(target),
                   initial_vector, atol, rtol, vectors, np.random.default_rng(0), require_convergence)


def test_oracle_iram_known_answers():
    """test/test_krylov.jl:219-234: nev=2, krylovdim=10, retained_dimension=5,
    maxrestarts=30, atol=1e-9, rtol=1e-7 reaches the two largest-real values within 2e-7
    after at least one restart with |L X - X diag(values)| < 3e-7, and the gap from them
    equals the dense gap within 2e-7."""
    L = _pi_matrix()
    n = L.shape[0]
    dense = np.linalg.eigvals(L)
    dense = dense[O.ritz_order(dense, "LR")]
    r = O.implicitly_restarted_arnoldi_spectrum(lambda v: L @ v, n, nev=2, krylovdim=10, retained_dimension=5,
                                                maxrestarts=30, initial_vector=_seed(n, 112), vectors=True,
                                                atol=1e-9, rtol=1e-7)
    assert r["algorithm"] == "implicit_qr_arnoldi" and r["restarts"] > 0
    assert np.allclose(r["values"], dense[:2], atol=2e-7, rtol=0)
    X = r["vectors"]
    assert np.linalg.norm(L @ X - X * r["values"][None, :]) < 3e-7
    gap = B._liouvillian_gap_info(r["values"], 1e-9, 1e-7, True)["gap"]
    assert abs(gap - _dense_gap(L)) <= 2e-7


@pytest.mark.parametrize("space_kind", ["numpy", "torch"])
@pytest.mark.parametrize("case", ["pi", "nonnormal_LR", "nonnormal_LM", "target"])
def test_library_iram_matches_oracle(space_kind, case):
    if case == "pi":
        A, kw = _pi_matrix(), dict(nev=2, krylovdim=10, retained_dimension=5, maxrestarts=30, atol=1e-9, rtol=1e-7)
    elif case == "nonnormal_LR":
        A, kw = _nonnormal(60, 3), dict(nev=3, krylovdim=20, maxrestarts=200)
    elif case == "nonnormal_LM":
        A, kw = _nonnormal(60, 4), dict(nev=3, krylovdim=20, maxrestarts=200, which="LM")
    else:
        A, kw = _nonnormal(50, 5), dict(nev=3, krylovdim=20, maxrestarts=300, target=-2.0 + 0.5j)
    n = A.shape[0]
    v0 = _seed(n, 9)
    ref = O.implicitly_restarted_arnoldi_spectrum(lambda v: A @ v, n, initial_vector=v0, vectors=True, **kw)
    space = NumpySpace(A) if space_kind == "numpy" else TorchCpuSpace(A)
    got = _host_iram(space, n, initial_vector=v0, vectors=True, **kw)
    assert got["converged"].all() and got["restarts"] == ref["restarts"]
    assert got["iterations"] == ref["iterations"]
    tol = got["residual_tolerance"]
    assert np.allclose(got["values"], ref["values"], atol=max(1e-8, 10 * tol), rtol=0)
    X = got["vectors"]
    resid = np.linalg.norm(A @ X - X * got["values"][None, :], axis=0)
    assert (resid <= 10 * tol).all(), (resid, tol)


@pytest.mark.parametrize("space_kind", ["numpy", "torch"])
def test_library_harmonic_over_torch_semantics(space_kind):
    """The harmonic algorithm over the torch-tensor stand-in gives the numpy space's values."""
    A = _nonnormal(60, 3)
    v0 = _seed(60, 1)
    n = 60
    kd, td, t, vv, s0 = B._check_harmonic_arguments(n, 3, 20, None, 200, 0, v0, None, None)
    space = NumpySpace(A) if space_kind == "numpy" else TorchCpuSpace(A)
    got = B._harmonic_arnoldi(space, n, 3, kd, td, 200, t, vv, s0, 1e-10, 1e-8, True, np.random.default_rng(0), True)
    ref = O.harmonic_arnoldi_spectrum(lambda v: A @ v, n, nev=3, krylovdim=20, maxrestarts=200, initial_vector=v0)
    assert np.allclose(got["values"], ref["values"], atol=1e-8, rtol=0)
    assert got["vectors"].shape == (60, 3)


def test_library_iram_not_converged_and_checks():
    A = _nonnormal(60, 3)
    with pytest.raises(picuda.PiArgumentError, match="did not converge in 1 restarts"):
        _host_iram(NumpySpace(A), 60, nev=3, krylovdim=8, maxrestarts=1, initial_vector=_seed(60, 1), atol=0, rtol=0)
    out = _host_iram(NumpySpace(A), 60, nev=3, krylovdim=8, maxrestarts=1, initial_vector=_seed(60, 1), atol=0,
                     rtol=0, vectors=True, require_convergence=False)
    assert out["restarts"] == 1 and out["vectors"].shape == (60, 3)
    with pytest.raises(picuda.PiArgumentError, match="nonzero"):
        _host_iram(NumpySpace(A), 60, nev=3, initial_vector=np.zeros(60))


def test_iram_gap_and_spectrum_dispatch(monkeypatch):
    """test/test_krylov.jl:219-234 through pi_liouvillian_gap(method=:iram) and
    liouvillian_spectrum(algorithm=:iram), with the device process replaced by the library's
    algorithm over numpy: the gap equals the dense gap within 2e-7 and the values are the
    two largest-real eigenvalues."""
    import types
    L = _pi_matrix()
    n = L.shape[0]
    calls = []

    def iram(compiled, nev=6, krylovdim=None, retained_dimension=None, maxrestarts=20, which="LR", target=None,
             initial_vector=None, atol=1e-10, rtol=1e-8, vectors=False, rng=None, require_convergence=True):
        calls.append((nev, krylovdim, retained_dimension, maxrestarts, which))
        return _host_iram(NumpySpace(L), n, nev=nev, krylovdim=krylovdim, retained_dimension=retained_dimension,
                          maxrestarts=maxrestarts, which=which, target=target, initial_vector=initial_vector,
                          atol=atol, rtol=rtol, vectors=vectors, require_convergence=require_convergence)

    monkeypatch.setattr(B, "implicitly_restarted_arnoldi_spectrum", iram)
    monkeypatch.setattr(B, "_as_compiled", lambda x: types.SimpleNamespace(basis=range(n)))
    info = picuda.pi_liouvillian_gap("model", method="iram", nev=2, krylovdim=10, retained_dimension=5,
                                     maxrestarts=30, return_info=True, initial_vector=_seed(n, 112), atol=1e-9,
                                     rtol=1e-7)
    assert calls[-1] == (2, 10, 5, 30, "LR")
    assert abs(info["gap"] - _dense_gap(L)) <= 2e-7
    assert info["method"] == "iram" and info["selection"] == "largest_real"
    picuda.pi_liouvillian_gap("model", method="implicit_qr", nev=2, krylovdim=10, initial_vector=_seed(n, 112),
                              atol=1e-9, rtol=1e-7)
    assert calls[-1] == (2, 10, 4, 20, "LR")
    res = picuda.liouvillian_spectrum("model", nev=2, algorithm="iram", krylovdim=10, retained_dimension=5,
                                      maxrestarts=30, initial_vector=_seed(n, 112), atol=1e-9, rtol=1e-7,
                                      return_info=True)
    assert calls[-1] == (2, 10, 5, 30, "LR")
    dense = np.linalg.eigvals(L)
    assert np.allclose(res.values, dense[O.ritz_order(dense, "LR")][:2], atol=2e-7, rtol=0)
    assert res.info["selected_algorithm"] == "iram"


def test_iram_spectral_scan_host_logic(monkeypatch):
    """A spectral scan with algorithm=:iram runs implicitly restarted Arnoldi per point and
    continues like Arnoldi, from the weighted combination of the previous Ritz vectors."""
    import types
    from picuda import scans as S
    from tests import models as M
    spin = picuda.spin_matrices()
    fam = picuda.compile_family(picuda.PIModel(picuda.PIBasis(3, 2), [picuda.LocalJump(spin["jm"], rate=1.0),
                                                                      picuda.LocalJump(spin["jp"], rate=0.2)]))
    seeds = []

    def compile_point(plan, parameter, index):
        made = plan.model_builder(parameter, index)
        model = S._family_model(made.family, S._family_rates(made.family, made.rates))
        return types.SimpleNamespace(basis=model.basis, matrix=O.materialize(O.Plan(M.to_oracle(model))))

    def iram(compiled, nev=6, krylovdim=None, retained_dimension=None, maxrestarts=20, which="LR", target=None,
             initial_vector=None, atol=1e-10, rtol=1e-8, vectors=False, rng=None, require_convergence=True):
        seeds.append(None if initial_vector is None else np.array(initial_vector))
        n = len(compiled.basis)
        v0 = initial_vector if initial_vector is not None else _seed(n, 5)
        return _host_iram(NumpySpace(compiled.matrix), n, nev=nev, krylovdim=krylovdim, maxrestarts=maxrestarts,
                          which=which, initial_vector=v0, atol=atol, rtol=rtol, vectors=vectors,
                          require_convergence=require_convergence)

    monkeypatch.setattr(S, "_compile_point", compile_point)
    monkeypatch.setattr(B, "implicitly_restarted_arnoldi_spectrum", iram)
    plan = picuda.ParameterScanPlan([0.2, 0.3], fam, rate_builder=lambda p: (1.0, p), task="spectrum", nev=2,
                                    algorithm="iram", save_vectors=True,
                                    solver_options={"krylovdim": 12, "maxrestarts": 50})
    res = picuda.parameter_scan(plan, on_error="throw")
    assert [p.status for p in res] == ["success", "success"]
    assert [p.warm_started for p in res] == [False, True]
    assert np.array_equal(seeds[1], S._arnoldi_continuation(res.points[0].output["vectors"]))
    assert res.points[1].diagnostics["method"] == "iram"
    for p, pt in zip([0.2, 0.3], res.points):
        L = compile_point(plan, p, 0).matrix
        dense = np.linalg.eigvals(L)
        assert np.allclose(pt.output["values"], dense[O.ritz_order(dense, "LR")][:2], atol=1e-6, rtol=0)


# ---- the device vector space's C-ABI marshalling, against a host model of the two calls ----

class _HostLib:
    """pi_mdot_f64_noalloc and pi_combine_f64 as include/picuda.h specifies them, computed
    on host memory: V holds nv (or k) vectors of n complex at leading dimension ldv, h and
    out receive the results, coef is k x ncols complex column-major."""

    @staticmethod
    def _view(ptr, count):
        address = ptr.value if isinstance(ptr, C.c_void_p) else C.cast(ptr, C.c_void_p).value
        return np.ctypeslib.as_array((C.c_double * (2 * count)).from_address(address)).view(np.complex128)

    def __init__(self):
        self.mdot_sizes = []

    def pi_mdot_f64_noalloc(self, V, ldv, nv, w, n, h, stream):
        assert 1 <= nv <= 32 and ldv >= n
        self.mdot_sizes.append(nv)
        Vm = self._view(V, ldv * nv).reshape(nv, ldv)[:, :n]
        self._view(h, nv)[:] = Vm.conj() @ self._view(w, n)
        return 0

    def pi_combine_f64(self, plan, V, ldv, k, coef, ncols, out, ldo):
        assert 1 <= k <= 128
        n = ldv
        Vm = self._view(V, ldv * k).reshape(k, ldv)[:, :n]
        cm = self._view(coef, k * ncols).reshape(ncols, k)  # column c holds coef[0..k) of output c
        self._view(out, ldo * ncols).reshape(ncols, ldo)[:, :n] = cm @ Vm
        return 0


def _host_device_space(A, m, monkeypatch):
    """A _DeviceKrylovSpace whose tensors live on the host and whose library is _HostLib."""
    import types
    torch = pytest.importorskip("torch")

    class TorchHost:
        cuda = types.SimpleNamespace(synchronize=lambda: None,
                                     current_stream=lambda: types.SimpleNamespace(cuda_stream=0))

        def __getattr__(self, name):
            return getattr(torch, name)

        @staticmethod
        def empty(*shape, dtype=None, device=None):
            return torch.empty(*shape, dtype=dtype)

        @staticmethod
        def zeros(*shape, dtype=None, device=None):
            return torch.zeros(*shape, dtype=dtype)

    n = A.shape[0]
    At = torch.from_numpy(A)

    def apply(y, compiled, x):
        y.copy_(At @ x)

    monkeypatch.setattr(B, "apply_", apply)
    monkeypatch.setattr(B, "_torch", lambda: TorchHost())
    lib = _HostLib()
    monkeypatch.setattr(B._lib, "load", lambda: lib)
    space = B._DeviceKrylovSpace(types.SimpleNamespace(basis=range(n), handle=None), m)
    space.upload = lambda v: torch.from_numpy(np.ascontiguousarray(v, dtype=np.complex128)).clone()
    space.download = lambda rows: rows.numpy().T.copy()
    return space, lib


def test_device_space_marshalling_harmonic_and_iram(monkeypatch):
    """The device space's pointers, leading dimensions, 32-vector multi-dot groups and
    column-major coefficients, checked by running harmonic Arnoldi and implicitly restarted
    Arnoldi with krylovdim 40 (projections over more than 32 vectors) against the oracle."""
    A = _nonnormal(80, 6)
    n = 80
    v0 = _seed(n, 21)
    space, lib = _host_device_space(A, 41, monkeypatch)
    kd, td, t, vv, s0 = B._check_harmonic_arguments(n, 3, 40, None, 100, 0, v0, None, None)
    got = B._harmonic_arnoldi(space, n, 3, kd, td, 100, t, vv, s0, 1e-10, 1e-8, True, np.random.default_rng(0),
                              True)
    ref = O.harmonic_arnoldi_spectrum(lambda v: A @ v, n, nev=3, krylovdim=40, maxrestarts=100, initial_vector=v0)
    assert max(lib.mdot_sizes) == 32 and 8 in lib.mdot_sizes  # 40 = 32 + 8
    assert got["restarts"] == ref["restarts"]
    assert np.allclose(got["values"], ref["values"], atol=1e-8, rtol=0)
    X = got["vectors"]
    assert (np.linalg.norm(A @ X - X * got["values"][None, :], axis=0) <= 1.01 * got["residual_tolerance"]).all()
    space, lib = _host_device_space(A, 41, monkeypatch)
    got = B._iram(space, n, 3, 40, 6, 100, "LR", None, v0, 1e-10, 1e-8, True, np.random.default_rng(0), True)
    ref = O.implicitly_restarted_arnoldi_spectrum(lambda v: A @ v, n, nev=3, krylovdim=40, retained_dimension=6,
                                                  maxrestarts=100, initial_vector=v0)
    assert max(lib.mdot_sizes) == 32 and 9 in lib.mdot_sizes  # the 41-vector block
    assert got["restarts"] == ref["restarts"]
    assert np.allclose(got["values"], ref["values"], atol=1e-8, rtol=0)
