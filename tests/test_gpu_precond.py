"""The level-sweep preconditioner on the GPU and the preconditioned steady-state GMRES.

- pi_precond_apply against the numpy sweep of the exported tables (FP32 sweeps in population
  coordinates: 2e-5 relative; FP64 sweeps in reference coordinates: 1e-12);
- preconditioned stationary states (left preconditioning as in krylov.jl:732-787), FP64 and
  mixed with FP64 refinement, against the exact steady state of the oracle's dense L and the
  oracle's own GMRES solve;
- the N = 200 boundary-time-crystal-like configuration (H = Omega Jx, Omega in
  {0.5, 1, 2} kappa, collective decay kappa = 1/N, local dephasing 0.01, dim 1,373,701): FP64
  and mixed reach a normalized residual of 1e-10 in population coordinates with the trace
  fixed, and agree with each other."""
import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from tests import models as M
from tests.level_sweep_eval import sweep

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("coords,tol", [("population", 2e-5), ("reference", 1e-12)])
@pytest.mark.parametrize("make", [lambda: M.btc_c3(12, 1.0), lambda: M.ensemble_c2(40)], ids=["btc12", "ens40"])
def test_device_sweep_matches_tables(torch_cuda, make, coords, tol):
    torch = torch_cuda
    model = make()
    c = picuda.compile(model)
    P = picuda.level_preconditioner(c, coords=coords, operator_scale=0.9)
    assert P.info["fp64"] == (1 if coords == "reference" else 0)
    T = picuda.level_preconditioner_tables(model, coords=coords, operator_scale=0.9)
    n = len(model.basis)
    for seed in range(2):
        r = M.random_state_vector(n, seed)
        rd = torch.from_numpy(r).cuda()
        zd = torch.empty_like(rd)
        P.apply(zd, rd)
        torch.cuda.synchronize()
        z = zd.cpu().numpy()
        ref = sweep(T, r, 0.9)
        assert np.abs(z - ref).max() <= tol * np.abs(ref).max(), (coords, np.abs(z - ref).max() / np.abs(ref).max())
    # repeated applies are bitwise equal (fixed order everywhere)
    z2 = torch.empty_like(rd)
    P.apply(z2, rd)
    torch.cuda.synchronize()
    assert torch.equal(z2, zd)


def exact_steady_state(model):
    """Null vector of the oracle's dense L with trace one (reference coordinates)."""
    oplan = O.Plan(M.to_oracle(model))
    L = O.materialize(oplan)
    n = L.shape[0]
    t = np.zeros(n)
    t[oplan.trace_idx] = np.real(oplan.trace_val)
    A = np.vstack([L, t[None, :]])
    rhs = np.zeros(n + 1, dtype=np.complex128)
    rhs[-1] = 1.0
    x, *_ = np.linalg.lstsq(A, rhs, rcond=None)
    return x, oplan


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("coords", ["population", "reference"])
@pytest.mark.parametrize("make", [lambda: M.btc_c3(10, 2.0), lambda: M.driven_c1(8), lambda: M.ensemble_c2(9)],
                         ids=["btc10", "driven8", "ens9"])
def test_preconditioned_steady_state_matches_exact(torch_cuda, make, coords, precision):
    model = make()
    c = picuda.compile(model)
    x_ref, oplan = exact_steady_state(model)
    P = picuda.level_preconditioner(c, coords=coords)
    alg = picuda.GMRESAlgorithm(krylovdim=30, maxiter=500, preconditioner=P, precision=precision)
    res = picuda.stationary_state(c, algorithm=alg, return_info=True, atol=1e-12, rtol=1e-12)
    assert res.info["converged"] and res.info["preconditioned"]
    x = res.state.data
    assert np.abs(x - x_ref).max() <= 1e-9 * np.abs(x_ref).max(), np.abs(x - x_ref).max()
    assert abs(O.trace(oplan, x) - 1) <= 1e-10
    # fewer operator applications than the unpreconditioned reference method needs
    try:
        plain = picuda.stationary_state(c, algorithm=picuda.GMRESAlgorithm(krylovdim=30, maxiter=3000),
                                        return_info=True, atol=1e-12, rtol=1e-12, coords=coords)
        plain_iterations = plain.info["iterations"]
    except picuda.PiNotConverged:
        plain_iterations = 3000
    assert res.info["iterations"] <= plain_iterations


def test_preconditioned_matches_oracle_gmres_c1(torch_cuda):
    """The driven N=8 configuration: the oracle's reference GMRES steady state and the
    preconditioned device solve agree to the solver tolerance."""
    model = M.driven_c1(8)
    oplan = O.Plan(M.to_oracle(model))
    x_o, _ = O.krylov_steady_state(oplan, atol=1e-12, rtol=1e-12, maxiter=5000)
    c = picuda.compile(model)
    P = picuda.level_preconditioner(c)
    res = picuda.stationary_state(c, algorithm=picuda.GMRESAlgorithm(preconditioner=P), return_info=True,
                                  atol=1e-12, rtol=1e-12)
    assert np.abs(res.state.data - x_o).max() <= 1e-8 * np.abs(x_o).max()


def test_preconditioner_argument_checks(torch_cuda):
    c1 = picuda.compile(M.btc_c3(8, 1.0))
    c2 = picuda.compile(M.btc_c3(8, 1.0))
    P = picuda.level_preconditioner(c1)
    with pytest.raises(picuda.PiArgumentError):
        picuda.stationary_state(c2, algorithm=picuda.GMRESAlgorithm(preconditioner=P))
    with pytest.raises(picuda.PiArgumentError, match="inconsistent"):
        picuda.stationary_state(c1, algorithm=picuda.GMRESAlgorithm(preconditioner=P),
                                operator_scale=2.0 * P.operator_scale)
    with pytest.raises(picuda.PiArgumentError):
        picuda.level_preconditioner(picuda.compile(picuda.Models.local_pump_decay(5, down=1.0, up=0.3)))
    with pytest.raises(picuda.PiArgumentError):
        picuda.stationary_state_batch([c1], algorithm=picuda.GMRESAlgorithm(preconditioner=P))


C3_TOL = 5e-11  # atol = rtol: normalized residual and trace error <= 1e-10 for |z| <= 1


@pytest.fixture(scope="module")
def c3_solutions(torch_cuda):
    out = {}
    for w in (0.5, 1.0, 2.0):
        c = picuda.compile(M.btc_c3(200, w))
        P = picuda.level_preconditioner(c, coords="population")
        for prec in ("fp64", "mixed"):
            alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=2000, preconditioner=P, precision=prec)
            res = picuda.stationary_state(c, algorithm=alg, return_info=True, atol=C3_TOL, rtol=C3_TOL)
            out[(w, prec)] = (res, c)
    return out


@pytest.mark.parametrize("w", [0.5, 1.0, 2.0])
def test_c3_steady_state_n200(torch_cuda, c3_solutions, w):
    r64, c = c3_solutions[(w, "fp64")]
    r32, _ = c3_solutions[(w, "mixed")]
    for r in (r64, r32):
        assert r.info["converged"]
        assert r.info["normalized_residual"] <= 1e-10
        assert r.info["trace_error"] <= 1e-10
        assert r.info["coords"] == "population"
    # population coordinates z = sqrt(f) x: compare where the entries are populations
    s = c.sector_scales()
    b = c.basis
    scale = np.concatenate([np.full(n * n, s[i]) for i, n in enumerate(b.dims)])
    z64, z32 = r64.state.data * scale, r32.state.data * scale
    dev = np.abs(z32 - z64).max() / np.abs(z64).max()
    assert dev <= 1e-8, dev
    # populations are real, nonnegative to the solver tolerance and sum to one
    idx, _ = c.library_trace_functional()
    pops = z64[idx]
    assert abs(pops.sum() - 1) <= 1e-10
    assert pops.real.min() >= -1e-9 and np.abs(pops.imag).max() <= 1e-9
