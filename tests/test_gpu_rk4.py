"""GPU fixed-step RK4 (evolve!, the default solve_dynamics algorithm) against the oracle's
restatement of evolution.jl:75-118 and the reference's own known answers."""
import numpy as np
import pytest
import scipy.linalg as sla

import picuda
from oracle import pi_oracle as O
from tests import models as M

pytestmark = pytest.mark.gpu

EXC = np.array([[0, 0], [0, 1]])


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.mark.parametrize("case", ["driven8", "general6", "c2_14"])
def test_rk4_fp64_matches_oracle(torch_cuda, case):
    """States and streamed observables of the FP64 RK4 path equal the oracle's RK4 to 1e-12
    relative (same stage sequence, same step size)."""
    model = {"driven8": lambda: M.driven_c1(8), "general6": lambda: M.general(6, seed=3),
             "c2_14": lambda: M.ensemble_c2(14)}[case]()
    oplan = O.Plan(M.to_oracle(model))
    rho0 = picuda.computational_product_state(model.basis, 2)
    s = picuda.spin_matrices(2)
    obs = {"exc": EXC, "jz": s["jz"]}
    oobs = {k: O.collective_operator(oplan.basis, v) for k, v in obs.items()}
    ref = O.solve_dynamics_rk4(oplan, rho0.data, (0.0, 0.6), saveat=0.2, observables=oobs, steps_per_interval=24)
    res = picuda.solve_dynamics(model, rho0, (0.0, 0.6), saveat=0.2, observables=obs, steps_per_interval=24)
    assert res.algorithm == "rk4"
    assert res.t == ref["t"]
    for a, b in zip(res.states, ref["states"]):
        assert _rel(a.data, b) <= 1e-12
    for k in obs:
        assert _rel(res.values[k], ref["values"][k]) <= 1e-12
    stream = picuda.solve_dynamics(model, rho0, (0.0, 0.6), saveat=0.2, observables=obs, save_states=False,
                                   steps_per_interval=24)
    for k in obs:
        assert _rel(stream.values[k], ref["values"][k]) <= 1e-12


def test_rk4_known_answer_exponential(torch_cuda):
    """test/test_evolution.jl:1-20 on the GPU: 400 steps equal exp(tL) rho to 2e-12, the
    chained in-place evolution (t, 2t) equals exp(2tL) rho to 3e-12, trace stays 1."""
    torch = torch_cuda
    b = picuda.PIBasis(2, 2)
    model = picuda.PIModel(b, [picuda.LocalJump(np.array([[0, 1], [0, 0]], dtype=complex))])
    oplan = O.Plan(M.to_oracle(model))
    L = O.materialize(oplan)
    rho = picuda.iid_pure_state(b, np.array([0, 1], dtype=complex))
    rho0 = rho.data.copy()
    t = 0.7
    out = picuda.time_evolve(model, rho, (0.0, t), steps=400)
    assert np.abs(out.data - sla.expm(t * L) @ rho.data).max() <= 2e-12
    assert abs(O.trace(oplan, out.data) - 1) <= 2e-12
    assert np.array_equal(rho.data, rho0)
    compiled = picuda.compile(model)
    d = torch.from_numpy(rho.data.copy()).cuda()
    src = torch.from_numpy(rho.data.copy()).cuda()
    picuda.evolve_(d, compiled, src, (0.0, t), steps=400)
    picuda.evolve_(d, compiled, d, (t, 2 * t), steps=400)
    assert np.abs(d.cpu().numpy() - sla.expm(2 * t * L) @ rho.data).max() <= 3e-12
    # partially overlapping storage and non-positive step counts are rejected (evolution.jl:82-84)
    buf = torch.zeros(2 * len(b), dtype=torch.complex128, device="cuda")
    with pytest.raises(picuda.PiArgumentError):
        picuda.evolve_(buf[1:1 + len(b)], compiled, buf[:len(b)], (0.0, 0.01), steps=1)
    with pytest.raises(picuda.PiArgumentError):
        picuda.evolve_(d, compiled, src, (0.0, 0.01), steps=0)


def test_rk4_grid_repeated_times_and_expv_agreement(torch_cuda):
    """test/test_highlevel.jl:33-60: saveat 0.05 with 40 steps per interval equals one
    160-step evolution to 2e-11; a tight expv agrees to 2e-9; repeated saved times give
    identical states; :auto selects RK4."""
    b = picuda.PIBasis(3, 2)
    model = picuda.PIModel(b, [picuda.LocalJump(np.array([[0, 1], [0, 0]], dtype=complex), rate=0.4)])
    rho0 = picuda.iid_pure_state(b, np.array([0, 1], dtype=complex))
    sol = picuda.solve_dynamics(model, rho0, (0.0, 0.2), saveat=0.05, steps_per_interval=40)
    assert len(sol) == 5 and sol.algorithm == "rk4"
    one = picuda.time_evolve(model, rho0, (0.0, 0.2), steps=160)
    assert np.abs(sol[-1].data - one.data).max() <= 2e-11
    ex = picuda.solve_dynamics(model, rho0, (0.0, 0.2), saveat=sol.t,
                               algorithm=picuda.ExpvAlgorithm(krylovdim=12, atol=1e-12, rtol=1e-10))
    assert ex.algorithm == "expv"
    for a, c in zip(sol.states, ex.states):
        assert np.abs(a.data - c.data).max() <= 2e-9
    rep = picuda.solve_dynamics(model, rho0, (0.0, 0.2), saveat=[0.0, 0.1, 0.1, 0.2])
    assert np.array_equal(rep[1].data, rep[2].data)
    rep_stream = picuda.solve_dynamics(model, rho0, (0.0, 0.2), saveat=[0.0, 0.1, 0.1, 0.2], save_states=False,
                                       observables={"exc": EXC})
    v = rep_stream.values["exc"]
    assert v[1] == v[2]
    for name in ("rk4", "adaptive_or_rk4", "dynamics", "auto"):
        assert picuda.solve_dynamics(model, rho0, (0.0, 0.1), algorithm=name).algorithm == "rk4"
    with pytest.raises(picuda.PiArgumentError):
        picuda.solve_dynamics(model, rho0, (0.0, 0.1), algorithm="euler")
    with pytest.raises(picuda.PiArgumentError):
        picuda.solve_dynamics(model, rho0, (0.0, 0.1), steps_per_interval=0)


def test_rk4_long_interval_graph_chunks(torch_cuda):
    """More steps per interval than one graph holds (main graph replayed plus a remainder
    graph) give the oracle's result."""
    model = M.scan_model(7, 1.3, 0.2, 0.05)
    oplan = O.Plan(M.to_oracle(model))
    rho0 = picuda.computational_product_state(model.basis, 2)
    ref = O.evolve_rk4(lambda v: O.apply(oplan, v), rho0.data, (0.0, 1.5), steps=203)
    out = picuda.time_evolve(model, rho0, (0.0, 1.5), steps=203)
    assert _rel(out.data, ref) <= 1e-12


@pytest.mark.parametrize("N", [12, 40])
def test_rk4_mixed_precision_vs_fp64(torch_cuda, N):
    """FP32 applies in population coordinates with an FP64 state and stage sum: observables
    within 1e-5 of the FP64 RK4 relative to their scale, trace within 1e-6."""
    model = M.ensemble_c2(N)
    rho0 = picuda.computational_product_state(model.basis, 2)
    s = picuda.spin_matrices(2)
    obs = {"Jz": s["jz"], "JpJm": s["jp"] @ s["jm"]}
    kw = dict(saveat=0.25, observables=obs, steps_per_interval=32)
    r64 = picuda.solve_dynamics(model, rho0, (0.0, 1.0), save_states=False, **kw)
    rmx = picuda.solve_dynamics(model, rho0, (0.0, 1.0), save_states=False, precision="mixed", **kw)
    for k in obs:
        assert _rel(rmx.values[k], r64.values[k]) <= 1e-5, k
    full = picuda.solve_dynamics(model, rho0, (0.0, 1.0), precision="mixed", **kw)
    oplan = O.Plan(M.to_oracle(model))
    for st in full.states:
        assert abs(O.trace(oplan, st.data) - 1) <= 1e-6
    for k in obs:
        assert _rel(full.values[k], rmx.values[k]) <= 1e-12


def test_checkpoint_resume_of_device_state(torch_cuda, tmp_path):
    """A device state saved mid-evolution (PIStateCheckpoint, :pid format) and loaded back
    resumes to exactly the uninterrupted result."""
    torch = torch_cuda
    model = M.driven_c1(8)
    c = picuda.compile(model)
    rho0 = picuda.computational_product_state(model.basis, 2)
    d = torch.from_numpy(rho0.data.copy()).cuda()
    picuda.evolve_(d, c, d, (0.0, 0.3), steps=30)
    picuda.save_checkpoint(tmp_path / "mid.pid", d, time=0.3, metadata={"steps": 30}, basis=model.basis)
    picuda.evolve_(d, c, d, (0.3, 0.6), steps=30)
    ck = picuda.load_checkpoint(tmp_path / "mid.pid")
    assert ck.time == 0.3 and ck.metadata == {"steps": "30"}
    r = torch.from_numpy(ck.state.data.copy()).cuda()
    picuda.evolve_(r, c, r, (ck.time, 0.6), steps=30)
    assert torch.equal(r, d)
