"""Batched multi-instance engine (pi_expv_batch, pi_dynamics_batch, pi_steady_state_batch)
against the single-instance entry points and the oracle."""
import ctypes as C

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


def _mixed_set():
    """Instances of uneven dimension and different term structure."""
    return [M.driven_c1(8), M.ensemble_c2(12), M.scan_model(17, 1.3, 0.2, 0.05), M.general(6, 3),
            M.scan_model(9, 0.4, 0.45, 0.15)]


def _excited(model):
    return picuda.computational_product_state(model.basis, 2).data


def test_expv_batch_fp64_matches_single_instance(torch_cuda):
    models = _mixed_set()
    states = [_excited(m) for m in models]
    ts = [0.7, 0.3, 1.1, 0.5, 2.0]
    got, infos = picuda.krylov_expv_batch(models, states, ts, return_info=True)
    for m, b, t, y, info in zip(models, states, ts, got, infos):
        ref, rinfo = picuda.krylov_expv(m, b, t, return_info=True)
        assert info["converged"]
        assert info["reached_time"] == pytest.approx(t)
        # same controller, same factorizations; only reduction order differs
        assert info["accepted_steps"] == rinfo["accepted_steps"]
        assert info["arnoldi_factorizations"] == rinfo["arnoldi_factorizations"]
        assert np.abs(y - ref).max() <= 1e-11 * max(np.abs(ref).max(), 1.0)


def test_expv_batch_matches_oracle(torch_cuda):
    models = [M.driven_c1(8), M.general(5, 9)]
    states = [_excited(models[0]), picuda.iid_pure_state(models[1].basis, np.array([0.6, 0.8j])).data]
    got = picuda.krylov_expv_batch(models, states, [1.5, 0.9])
    for m, b, t, y in zip(models, states, [1.5, 0.9], got):
        oplan = O.Plan(M.to_oracle(m))
        ref, _ = O.krylov_expv(lambda z: O.apply(oplan, z), b, t)
        assert np.abs(y - ref).max() <= 1e-9 * max(np.abs(ref).max(), 1.0)


def test_expv_batch_mixed_error_vs_fp64(torch_cuda):
    models = _mixed_set()
    states = [_excited(m) for m in models]
    ts = [0.7, 0.3, 1.1, 0.5, 2.0]
    y64 = picuda.krylov_expv_batch(models, states, ts)
    ymx = picuda.krylov_expv_batch(models, states, ts, algorithm=picuda.ExpvAlgorithm(precision="mixed"))
    for a, b in zip(ymx, y64):
        # FP32 applies and basis, FP64 orthogonalisation and state: ~FP32 rounding per step
        assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max()


def test_expv_batch_negative_and_zero_time(torch_cuda):
    models = [M.driven_c1(6), M.driven_c1(7)]
    states = [_excited(m) for m in models]
    got, infos = picuda.krylov_expv_batch(models, states, [0.0, -0.2], return_info=True)
    assert np.array_equal(got[0], states[0])
    ref = picuda.krylov_expv(models[1], states[1], -0.2)
    assert np.abs(got[1] - ref).max() <= 1e-11 * np.abs(ref).max()
    assert infos[1]["reached_time"] == pytest.approx(-0.2)


EXC = np.array([[0, 0], [0, 1]])
JZ = np.diag([0.5, -0.5])


def test_dynamics_batch_matches_single_solve_dynamics(torch_cuda):
    models = [M.driven_c1(8), M.ensemble_c2(10), M.scan_model(14, 1.7, 0.1, 0.02)]
    rho0s = [picuda.computational_product_state(m.basis, 2 if i != 1 else 1) for i, m in enumerate(models)]
    obs = {"exc": EXC, "jz": JZ}
    results, finals = picuda.solve_dynamics_batch(models, rho0s, (0.0, 1.0), saveat=0.1, observables=obs)
    for m, r0, res, fin in zip(models, rho0s, results, finals):
        ref = picuda.solve_dynamics(m, r0, (0.0, 1.0), algorithm="expv", saveat=0.1, save_states=False, observables=obs)
        assert res.t == ref.t
        for k in obs:
            assert np.abs(res.values[k] - ref.values[k]).max() <= 1e-10 * max(np.abs(ref.values[k]).max(), 1.0)
        single = picuda.krylov_expv(m, r0.data, 0.0)  # state unchanged at t = 0
        assert np.array_equal(single, r0.data)


def test_dynamics_batch_zero_length_intervals(torch_cuda):
    m = M.driven_c1(6)
    rho0 = picuda.computational_product_state(m.basis, 2)
    res, fin = picuda.solve_dynamics_batch([m], [rho0], (0.0, 0.4), saveat=[[0.0, 0.0, 0.2, 0.2, 0.4]],
                                           observables={"exc": np.array([[0, 0], [0, 1]])})
    v = res[0].values["exc"]
    assert v[0] == v[1] and v[2] == v[3]
    ref = picuda.solve_dynamics(m, rho0, (0.0, 0.4), algorithm="expv", saveat=[0.0, 0.0, 0.2, 0.2, 0.4], save_states=False,
                                observables={"exc": np.array([[0, 0], [0, 1]])})
    assert np.abs(v - ref.values["exc"]).max() <= 1e-10 * np.abs(ref.values["exc"]).max()


def test_batch_result_same_alone_and_in_mix(torch_cuda):
    """An instance's arithmetic does not depend on its batch companions: bitwise equal."""
    target = M.scan_model(15, 0.9, 0.3, 0.1)
    others = [M.driven_c1(8), M.ensemble_c2(20), M.scan_model(11, 1.9, 0.06, 0.0)]
    mix = others[:2] + [target] + others[2:]
    for prec in ("fp64", "mixed"):
        alg = picuda.ExpvAlgorithm(precision=prec)
        ra, fa = picuda.solve_dynamics_batch([target], [_excited(target)], (0.0, 0.5), algorithm=alg,
                                             saveat=0.05, observables={"exc": EXC})
        rm, fm = picuda.solve_dynamics_batch(mix, [_excited(m) for m in mix], (0.0, 0.5), algorithm=alg,
                                             saveat=0.05, observables={"exc": EXC})
        assert np.array_equal(fa[0], fm[2]), prec
        assert np.array_equal(ra[0].values["exc"], rm[2].values["exc"]), prec


def test_steady_state_batch_fp64_matches_single(torch_cuda):
    models = [M.driven_c1(8), picuda.Models.local_pump_decay(5, down=1.0, up=0.3), M.scan_model(10, 0.8, 0.4, 0.1)]
    states, infos = picuda.stationary_state_batch(models, algorithm=picuda.GMRESAlgorithm(krylovdim=50, maxiter=3000),
                                                  return_info=True)
    for m, s, info in zip(models, states, infos):
        assert info["converged"], info
        ref = picuda.stationary_state(m, algorithm=picuda.GMRESAlgorithm(krylovdim=50, maxiter=3000))
        assert np.abs(s.data - ref.data).max() <= 1e-7 * np.abs(ref.data).max()


def test_steady_state_batch_matches_oracle_direct_solve(torch_cuda):
    m = M.driven_c1(8)
    oplan = O.Plan(M.to_oracle(m))
    x_ref, info_ref = O.krylov_steady_state(oplan)
    states, infos = picuda.stationary_state_batch([m], return_info=True,
                                                  operator_scale=info_ref["operator_scale"])
    assert infos[0]["converged"]
    assert np.abs(states[0].data - x_ref).max() <= 1e-8 * np.abs(x_ref).max()


def test_steady_state_batch_mixed(torch_cuda):
    models = [M.driven_c1(8), M.driven_c1(12), M.scan_model(12, 0.5, 0.45, 0.2)]
    alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=5000)
    s64 = picuda.stationary_state_batch(models, algorithm=alg)
    smx, infos = picuda.stationary_state_batch(
        models, algorithm=picuda.GMRESAlgorithm(krylovdim=50, maxiter=5000, precision="mixed"), return_info=True)
    for a, b, info in zip(smx, s64, infos):
        assert info["converged"] and info["refinements"] >= 1
        assert info["normalized_residual"] <= 1e-10 + 1e-8 * max(np.linalg.norm(a.data), 1.0)
        assert np.abs(a.data - b.data).max() <= 1e-6 * np.abs(b.data).max()


def test_batch_argument_errors(torch_cuda):
    torch = torch_cuda
    m = M.driven_c1(5)
    c = picuda.compile(m)
    x = torch.zeros(len(m.basis), dtype=torch.complex128, device="cuda")
    lib = picuda.load_library()
    plans = (C.c_void_p * 2)(c.handle, c.handle)
    xs = (C.c_void_p * 2)(x.data_ptr(), x.data_ptr())
    o = picuda.ExpvAlgorithm().opts()
    ts = np.array([0.1, 0.1])
    rc = lib.pi_expv_batch(2, plans, xs, _lib.dptr(ts), C.byref(o), None)
    assert rc == _lib.PI_ERR_INVALID_ARGUMENT and "share" in _lib.last_error()
    o.krylovdim = 121
    xs2 = (C.c_void_p * 1)(x.data_ptr())
    rc = lib.pi_expv_batch(1, plans, xs2, _lib.dptr(ts), C.byref(o), None)
    assert rc == _lib.PI_ERR_INVALID_ARGUMENT and "krylovdim" in _lib.last_error()


def test_steady_state_batch_reports_nonconverged_instance(torch_cuda):
    """A scan keeps going when one point does not converge: its info says so."""
    models = [M.driven_c1(8), M.driven_c1(10)]
    states, infos = picuda.stationary_state_batch(models, algorithm=picuda.GMRESAlgorithm(maxiter=3),
                                                  return_info=True, raise_on_failure=False)
    assert not infos[0]["converged"] and infos[0]["iterations"] == 3
    assert not infos[1]["converged"]
    with pytest.raises(picuda.PiNotConverged):
        picuda.stationary_state_batch(models, algorithm=picuda.GMRESAlgorithm(maxiter=3))
