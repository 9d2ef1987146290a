"""Mixed-precision results against the FP64 oracle, not only against the GPU's own FP64 path.

- C1 (driven qubits N=8): expv dynamics observables and the steady state, mixed and FP64,
  against the oracle fixtures of tests/golden/driven_qubits_N8.npz;
- C2 at N=40: four saved intervals of expv dynamics, mixed and FP64, against the oracle run
  here;
- C2 at N=120 (the large time-evolution configuration): twenty saved intervals of expv and of
  the reference's default fixed-step RK4 (64 steps per interval), mixed and FP64, against
  the oracle's FP64 expv observables of tests/golden/ensemble_c2_N120_expv.npz.

Tolerances (relative to the largest |value|): FP64 1e-9 (the oracle's own expv tolerance is
1e-10 absolute, 1e-8 relative per step); mixed 1e-6 (FP32 applies, FP64 orthogonalisation)."""
from pathlib import Path

import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from tests import models as M

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
TOL = {"fp64": 1e-9, "mixed": 1e-6}


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c1_dynamics_and_steady_state_vs_oracle(torch_cuda, precision):
    g = np.load(GOLDEN / "driven_qubits_N8.npz")
    model = M.driven_c1(8)
    c = picuda.compile(model)
    s = picuda.spin_matrices(2)
    rho0 = picuda.computational_product_state(model.basis, 2)
    res = picuda.solve_dynamics(c, rho0, (0.0, 4.0), saveat=0.1, save_states=False,
                                algorithm=picuda.ExpvAlgorithm(krylovdim=30, precision=precision),
                                observables={"excited": s["jp"] @ s["jm"], "Jz": s["jz"]})
    for k in ("excited", "Jz"):
        assert _rel(res.values[k], g[k]) <= TOL[precision], (precision, k, _rel(res.values[k], g[k]))
    ss = picuda.stationary_state(c, algorithm=picuda.GMRESAlgorithm(precision=precision), return_info=True,
                                 operator_scale=float(g["steady_operator_scale"]))
    # both solves stop at the reference's tolerances (atol 1e-10, rtol 1e-8 on the residual)
    assert _rel(ss.state.data, g["steady"]) <= 1e-6, _rel(ss.state.data, g["steady"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c2_n40_dynamics_vs_oracle(torch_cuda, precision):
    model = M.ensemble_c2(40)
    oplan = O.Plan(M.to_oracle(model))
    ob = oplan.basis
    s = picuda.spin_matrices(2)
    so = O.spin_matrices(2)
    ref = O.solve_dynamics_expv(oplan, O.computational_product_state(ob, 2), (0.0, 0.2), saveat=0.05,
                                observables={"Jz": O.collective_operator(ob, so["jz"])}, save_states=False)
    c = picuda.compile(model)
    res = picuda.solve_dynamics(c, picuda.computational_product_state(model.basis, 2), (0.0, 0.2), saveat=0.05,
                                save_states=False, algorithm=picuda.ExpvAlgorithm(krylovdim=30, precision=precision),
                                observables={"Jz": s["jz"]})
    assert _rel(res.values["Jz"], ref["values"]["Jz"]) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("algorithm", ["expv", "rk4"])
def test_c2_n120_dynamics_vs_oracle(torch_cuda, algorithm, precision):
    g = np.load(GOLDEN / "ensemble_c2_N120_expv.npz")
    model = M.ensemble_c2(120)
    c = picuda.compile(model)
    s = picuda.spin_matrices(2)
    obs = {"Jz": s["jz"], "JpJm": s["jp"] @ s["jm"]}
    rho0 = picuda.computational_product_state(model.basis, 2)
    tspan = (0.0, float(g["t"][-1]))
    if algorithm == "expv":
        res = picuda.solve_dynamics(c, rho0, tspan, saveat=0.05, save_states=False, observables=obs,
                                    algorithm=picuda.ExpvAlgorithm(krylovdim=30, precision=precision))
    else:
        res = picuda.solve_dynamics(c, rho0, tspan, saveat=0.05, save_states=False, observables=obs,
                                    steps_per_interval=64, precision=precision)
    assert np.allclose(res.t, g["t"])
    for k in obs:
        assert _rel(res.values[k], g[k]) <= TOL[precision], (algorithm, precision, k, _rel(res.values[k], g[k]))
