"""The drive preconditioner on the GPU: its application against a numpy restatement built
from the host tables, and preconditioned steady states of strongly driven models (where the
reference's unpreconditioned GMRES and the level sweep stall) against the oracle."""
import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from picuda import _lib
from tests import models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _border(model):
    plan = O.Plan(M.to_oracle(model))
    n = len(plan)
    t = np.zeros(n, dtype=np.complex128)
    t[plan.trace_idx] = plan.trace_val
    return plan, t, t / np.vdot(t, t)


def test_apply_matches_numpy_restatement(torch_cuda):
    """z = M^-1 r in reference coordinates: block-diagonal normal-part solves plus the trace
    border by Sherman-Morrison; FP64 vectors are mapped in FP64 arithmetic."""
    torch = torch_cuda
    model = M.scan_model(37, 1.3, 0.2, 0.05)
    c = picuda.compile(model)
    P = picuda.drive_preconditioner(c, coords="reference", operator_scale=17.0)
    assert P.info["kind"] == _lib.PI_PRECOND_DRIVE and P.operator_scale == 17.0
    assert P.info["max_asymmetry"] <= 1e-12 and P.info["max_nonhermitian"] <= 1e-12
    tables = picuda.drive_preconditioner_tables(model)
    plan, t, v = _border(model)
    b = model.basis
    rng = np.random.default_rng(5)
    r = rng.standard_normal(len(b)) + 1j * rng.standard_normal(len(b))

    def dmat(tab):
        h, q = tab["h"], tab["q"]
        return (-0.5 * (q[:, None] + q[None, :]) - 1j * (h[:, None] - h[None, :])) / 17.0

    def D(x):
        z = np.empty_like(x)
        for sec, tab in enumerate(tables):
            o, m = b.offsets[sec], b.dims[sec]
            R = x[o:o + m * m].reshape((m, m), order="F")
            z[o:o + m * m] = (tab["U"] @ ((tab["U"].T @ R @ tab["U"]) / dmat(tab)) @ tab["U"].T).reshape(-1, order="F")
        return z

    Dv = D(v)
    ref = D(r)
    ref = ref - Dv * (np.vdot(t, ref) / (1 + np.vdot(t, Dv)))
    z = torch.zeros(len(b), dtype=torch.complex128, device="cuda")
    P.apply(z, torch.from_numpy(r).cuda())
    got = z.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()
    # M z = r: the preconditioner inverts its own operator, U [(U^T X U) * d] U^T + v t^H X
    Bz = np.empty_like(got)
    for sec, tab in enumerate(tables):
        o, m = b.offsets[sec], b.dims[sec]
        U = tab["U"]
        X = got[o:o + m * m].reshape((m, m), order="F")
        Bz[o:o + m * m] = (U @ ((U.T @ X @ U) * dmat(tab)) @ U.T).reshape(-1, order="F")
    Bz = Bz + v * np.vdot(t, got)
    assert np.abs(Bz - r).max() <= 1e-10 * np.abs(r).max()


def _check_against_oracle(model, x, tol):
    plan, t, _ = _border(model)
    res = O.apply(plan, x)
    s = O.estimated_operator_scale(lambda z: O.apply(plan, z), len(plan))
    assert np.linalg.norm(res) / s <= tol * max(np.linalg.norm(x), 1.0)
    assert abs(np.vdot(t, x) - 1) <= 1e-8  # the solve's trace tolerance, atol + rtol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_drive_preconditioned_steady_state_of_a_strongly_driven_model(torch_cuda, precision):
    """Omega = 1.7 against loss 0.06 and dephasing 0.02 at N = 40: the unpreconditioned method
    does not reach 1e-10 in 3000 steps; with the drive part it converges in a few restarts.
    The state's residual and trace are checked with the oracle's apply."""
    model = M.scan_model(40, 1.7, 0.06, 0.02)
    c = picuda.compile(model)
    P = picuda.drive_preconditioner(c, coords="population")
    alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=1500, precision=precision, preconditioner=P)
    res = picuda.stationary_state(c, algorithm=alg, return_info=True)
    info = res.info
    assert info["converged"], info
    assert info["iterations"] <= 600
    _check_against_oracle(model, res.state.data, 1e-8)


def test_matches_dense_oracle_steady_state(torch_cuda):
    """A strongly driven model small enough for a dense solve of the oracle's bordered system."""
    model = M.scan_model(12, 1.6, 0.1, 0.05)
    plan, t, v = _border(model)
    L = O.materialize(plan)
    n = len(plan)
    s = O.estimated_operator_scale(lambda z: O.apply(plan, z), n)
    x_ref = np.linalg.solve(L / s + np.outer(v, t.conj()), v)
    c = picuda.compile(model)
    P = picuda.drive_preconditioner(c, coords="reference", operator_scale=s)
    alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=1000, precision="fp64", preconditioner=P)
    # tight tolerances: the state error is the residual tolerance times the conditioning
    res = picuda.stationary_state(c, algorithm=alg, return_info=True, atol=1e-14, rtol=1e-12)
    assert res.info["converged"]
    assert np.abs(res.state.data - x_ref).max() <= 1e-9 * np.abs(x_ref).max()


@pytest.mark.parametrize("case,want_stage", [("strong", 1), ("weak", 0)])
def test_adaptive_ladder_moves_only_when_the_level_sweep_stalls(torch_cuda, case, want_stage):
    """Level sweep first; the strongly driven model moves to the drive part after one slow
    cycle, the weakly driven BTC-like model (the level sweep's regime) never moves."""
    model = M.scan_model(40, 1.5, 0.1, 0.05) if case == "strong" else M.btc_c3(40, 1.0)
    c = picuda.compile(model)
    lev = picuda.level_preconditioner(c, coords="population")
    drv = picuda.drive_preconditioner(c, coords="population", operator_scale=lev.operator_scale)
    alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=3000, precision="mixed", preconditioner=lev,
                                drive_preconditioner=drv)
    res = picuda.stationary_state(c, algorithm=alg, return_info=True)
    info = res.info
    assert info["converged"], info
    if want_stage:
        assert info["preconditioner_stage"] >= want_stage
    else:
        assert info["preconditioner_stage"] == 0
    _check_against_oracle(model, res.state.data, 1e-8)


def test_argument_errors(torch_cuda):
    m = M.scan_model(10, 1.0, 0.2, 0.1)
    c = picuda.compile(m)
    c2 = picuda.compile(M.scan_model(10, 0.5, 0.2, 0.1))
    lev = picuda.level_preconditioner(c, coords="population")
    drv = picuda.drive_preconditioner(c, coords="population", operator_scale=lev.operator_scale)
    with pytest.raises(picuda.PiArgumentError):
        picuda.GMRESAlgorithm(drive_preconditioner=drv)  # needs a level preconditioner beside it
    with pytest.raises(picuda.PiArgumentError):
        picuda.GMRESAlgorithm(preconditioner=drv, drive_preconditioner=drv)
    other = picuda.drive_preconditioner(c2, coords="population", operator_scale=lev.operator_scale)
    with pytest.raises(picuda.PiArgumentError):
        picuda.stationary_state(c, algorithm=picuda.GMRESAlgorithm(preconditioner=lev, drive_preconditioner=other))
    mismatched = picuda.drive_preconditioner(c, coords="population", operator_scale=2 * lev.operator_scale)
    with pytest.raises(picuda.PiArgumentError, match="operator scales"):
        picuda.stationary_state(c, algorithm=picuda.GMRESAlgorithm(preconditioner=lev,
                                                                   drive_preconditioner=mismatched))
    with pytest.raises(picuda.PiArgumentError):
        picuda.drive_preconditioner(c, coords="nowhere")
    # the batched engine runs unpreconditioned
    with pytest.raises(picuda.PiError):
        picuda.stationary_state_batch([c], algorithm=picuda.GMRESAlgorithm(preconditioner=lev,
                                                                           drive_preconditioner=drv))
