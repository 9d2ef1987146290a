"""Parameter scans and compiled families on the GPU (scans.jl, compiled_families.jl): the
batched execution against one stationary_state per point, serial continuation, outputs."""
import numpy as np
import pytest

import picuda
from tests import models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_family_scan_batched_matches_single_solves(torch_cuda):
    proto = M.scan_model(10, 1.0, 0.2, 0.05)  # terms: H, emission, dephasing, collective emission
    fam = picuda.compile_family(proto, rate_indices=[0, 1])
    grid = [(om, gd) for om in (0.4, 1.3) for gd in (0.1, 0.35, 0.6)]
    alg = picuda.GMRESAlgorithm(maxiter=3000)  # weakly damped points need more than the default 500
    plan = picuda.ParameterScanPlan(grid, fam, continuation=False, algorithm=alg,
                                    diagnostic=lambda st, p, i: float(np.abs(st.data).max()))
    res = picuda.parameter_scan(plan, execution="batched")
    assert len(res) == len(grid) and res.restart_index == len(grid)
    for pt, rates in zip(res, grid):
        assert pt.status == "success" and pt.converged and pt.parameter == rates
        assert pt.trace_error <= 1e-10 + 1e-8
        ref = picuda.stationary_state(picuda.specialize(fam, rates), algorithm=alg)
        # both solves stop at normalized residual 1e-8; their states differ by up to the
        # conditioning times that, ~1e-7 here
        assert _rel(pt.output.data, ref.data) <= 1e-6
        assert pt.diagnostics["user"] == pytest.approx(float(np.abs(pt.output.data).max()))
        assert pt.diagnostics["dimension"] == len(proto.basis)


def test_builder_scan_uneven_dimensions_and_serial_continuation(torch_cuda):
    params = [(8, 0.9), (13, 1.4), (10, 0.6), (10, 0.65)]
    build = lambda p, i: M.scan_model(p[0], p[1], 0.25, 0.05)
    alg = picuda.GMRESAlgorithm(maxiter=3000)
    batched = picuda.parameter_scan(picuda.ParameterScanPlan(params, build, continuation=False, algorithm=alg),
                                    execution="batched")
    serial = picuda.parameter_scan(picuda.ParameterScanPlan(params, build, continuation=True, algorithm=alg))
    assert [p.warm_started for p in serial] == [False, False, False, True]  # dims must match to warm-start
    assert serial.restart_seed is not None
    for a, b in zip(batched, serial):
        assert a.status == b.status == "success"
        assert _rel(a.output.data, b.output.data) <= 1e-6
    quiet = picuda.parameter_scan(picuda.ParameterScanPlan(params[:2], build, continuation=False, algorithm=alg,
                                                           save_outputs=False), execution="batched")
    assert all(p.output is None and p.status == "success" for p in quiet)


def test_scan_records_nonconverged_points(torch_cuda):
    """A point the solver cannot bring to tolerance within maxiter is a failed record."""
    build = lambda p: M.scan_model(12, p, 0.2, 0.05)
    plan = picuda.ParameterScanPlan([0.5, 1.5], build, continuation=False,
                                    algorithm=picuda.GMRESAlgorithm(krylovdim=4, maxiter=8))
    res = picuda.parameter_scan(plan, execution="batched", on_error="record")
    assert all(p.status == "failed" and p.error_type == "PiNotConverged" for p in res)
    with pytest.raises(picuda.PiNotConverged):
        picuda.parameter_scan(plan, execution="batched", on_error="throw")


def test_spectral_family_scan(torch_cuda):
    """task=:spectrum: each point's leading Ritz values equal a direct Arnoldi spectrum of the
    specialized model; serial continuation warm-starts from the previous leading vector."""
    proto = M.scan_model(6, 1.0, 0.2, 0.05)
    fam = picuda.compile_family(proto, rate_indices=[0])
    grid = [0.5, 0.8, 1.1]
    n = len(proto.basis)
    plan = picuda.ParameterScanPlan(grid, fam, task="spectrum", nev=3, continuation=True, save_vectors=True,
                                    solver_options={"krylovdim": n})
    res = picuda.parameter_scan(plan)
    assert [p.warm_started for p in res] == [False, True, True]
    for pt, om in zip(res, grid):
        assert pt.status == "success" and pt.converged
        direct = picuda.krylov_liouvillian_spectrum(picuda.specialize(fam, om), nev=3, krylovdim=n)
        canon = lambda v: v[np.lexsort((np.round(v.imag, 8), np.round(v.real, 8)))]
        assert np.allclose(canon(pt.output["values"]), canon(direct["values"]), atol=1e-9, rtol=0)
        assert pt.output["vectors"].shape == (n, 3)
