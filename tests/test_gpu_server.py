"""Continuous-batching server (pi_server_*): results against the batched/single entry points,
independence of a request's result from the requests it shares the engine with, and
memory-budget admission."""
import time

import numpy as np
import pytest

import picuda
from tests import models as M

pytestmark = pytest.mark.gpu

EXC = np.array([[0, 0], [0, 1]])


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _excited(m):
    return picuda.computational_product_state(m.basis, 2)


def test_server_dynamics_and_steady_match_direct_calls(torch_cuda):
    dyn = [M.scan_model(12, 1.1, 0.2, 0.05), M.driven_c1(8), M.ensemble_c2(16)]
    std = [M.driven_c1(8), picuda.Models.local_pump_decay(6, down=1.0, up=0.3)]
    with picuda.Server() as srv:
        tags = {}
        for i, m in enumerate(dyn):
            tags[srv.submit_dynamics(m, _excited(m), 0.4 + 0.1 * i, 0.05, observables={"exc": EXC})] = ("d", i)
        for i, m in enumerate(std):
            tags[srv.submit_steady(m, maxiter=3000)] = ("s", i)
        done = srv.drain()
    assert len(done) == len(tags)
    for c in done:
        kind, i = tags[c.tag]
        assert c.ok, c.message
        assert c.finish_time >= c.start_time >= c.submit_time
        if kind == "d":
            m = dyn[i]
            ref = picuda.solve_dynamics(m, _excited(m), (0.0, 0.4 + 0.1 * i), algorithm="expv", saveat=0.05, save_states=False,
                                        observables={"exc": EXC})
            assert c.times == ref.t
            assert np.abs(c.values["exc"] - ref.values["exc"]).max() <= 1e-10 * np.abs(ref.values["exc"]).max()
        else:
            ref = picuda.stationary_state(std[i], algorithm=picuda.GMRESAlgorithm(maxiter=3000))
            assert np.abs(c.state - ref.data).max() <= 1e-7 * np.abs(ref.data).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_server_result_same_alone_and_in_mix(torch_cuda, precision):
    """A request served alone and the same request arriving into a busy server give the
    same state and observables, bit for bit (tolerance 0)."""
    target = M.scan_model(18, 0.7, 0.25, 0.1)
    with picuda.Server(precision=precision) as srv:
        srv.submit_dynamics(target, _excited(target), 1.0, 0.05, observables={"exc": EXC}, tag=1)
        alone = srv.drain()[0]
    others = [M.scan_model(int(n), om, gd, gp) for n, om, gd, gp in M.scan_draws(6, seed=5, nmin=10, nmax=40)]
    with picuda.Server(precision=precision) as srv:
        for k, m in enumerate(others[:3]):
            srv.submit_dynamics(m, _excited(m), 0.5 + 0.25 * k, 0.05, tag=100 + k)
        srv.submit_steady(M.driven_c1(8), maxiter=2000, tag=200)
        time.sleep(0.05)  # the target arrives while the others are being served
        srv.submit_dynamics(target, _excited(target), 1.0, 0.05, observables={"exc": EXC}, tag=1)
        for k, m in enumerate(others[3:]):
            srv.submit_dynamics(m, _excited(m), 0.3, 0.05, tag=300 + k)
        done = {c.tag: c for c in srv.drain()}
    mixed = done[1]
    assert alone.ok and mixed.ok
    assert np.array_equal(alone.state, mixed.state)
    assert np.array_equal(alone.values["exc"], mixed.values["exc"])
    assert all(c.ok for c in done.values())


def test_server_memory_budget_serializes_admission(torch_cuda):
    models = [M.scan_model(30, 1.0, 0.2, 0.1) for _ in range(3)]
    dim = len(models[0].basis)
    one = 16 * dim * (30 + 3) + 2 * 16 * dim  # fp64 footprint of one dynamics request
    with picuda.Server(memory_budget=1.5 * one) as srv:
        for i, m in enumerate(models):
            srv.submit_dynamics(m, _excited(m), 0.2, 0.05, tag=i + 1)
        done = sorted(srv.drain(fetch_state=False), key=lambda c: c.tag)
        st = srv.stats()
    assert all(c.ok for c in done)
    for a, b in zip(done, done[1:]):
        assert b.start_time >= a.finish_time - 1e-3  # one at a time
    assert st["completed"] == 3 and st["active"] == 0 and st["bytes_in_use"] == 0


def test_server_rejects_oversized_request(torch_cuda):
    m = M.scan_model(20, 1.0, 0.2, 0.1)
    with picuda.Server(memory_budget=1e5) as srv:
        with pytest.raises(picuda.PiError):
            srv.submit_dynamics(m, _excited(m), 0.2, 0.05)


def test_server_mixed_close_to_fp64(torch_cuda):
    models = [M.scan_model(int(n), om, gd, gp) for n, om, gd, gp in M.scan_draws(4, seed=9, nmin=10, nmax=30)]
    res = {}
    for prec in ("fp64", "mixed"):
        with picuda.Server(precision=prec) as srv:
            for i, m in enumerate(models):
                srv.submit_dynamics(m, _excited(m), 1.0, 0.05, tag=i + 1)
            res[prec] = {c.tag: c.state for c in srv.drain()}
    for k in res["fp64"]:
        ref = res["fp64"][k]
        assert np.abs(res["mixed"][k] - ref).max() <= 2e-5 * np.abs(ref).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_server_preconditioned_steady_requests(torch_cuda, precision):
    """steady_solvers > 0: steady requests are solved beside the engine, preconditioned by the
    level sweep and the drive part (adaptive), while dynamics requests share the engine.  A
    strongly driven N = 40 request, which the unpreconditioned method does not bring to
    tolerance, converges; every steady state equals a direct preconditioned solve of the same
    model and stays the same alone and in the mix."""
    from oracle import pi_oracle as O
    std = [M.scan_model(40, 1.7, 0.06, 0.02), M.btc_c3(24, 1.0), M.driven_c1(8)]
    dyn = [M.scan_model(14, 1.1, 0.2, 0.05), M.ensemble_c2(16)]
    comp = [picuda.compile(m) for m in std]
    with picuda.Server(precision=precision, steady_solvers=2) as srv:
        tags = {}
        for i, m in enumerate(dyn):
            tags[srv.submit_dynamics(m, _excited(m), 0.5, 0.05, observables={"exc": EXC})] = ("d", i)
        for i, c in enumerate(comp):
            tags[srv.submit_steady(c)] = ("s", i)
        done = srv.drain()
    with picuda.Server(precision=precision, steady_solvers=1) as srv:
        alone = srv.submit_steady(comp[0])
        (a,) = srv.drain()
        assert a.tag == alone and a.ok, a.message
    assert len(done) == len(tags)
    for c in done:
        kind, i = tags[c.tag]
        assert c.ok, c.message
        if kind != "s":
            continue
        lev = picuda.level_preconditioner(comp[i], coords="population")
        drv = picuda.drive_preconditioner(comp[i], coords="population", operator_scale=lev.operator_scale)
        alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=2000, precision=precision, preconditioner=lev,
                                    drive_preconditioner=drv)
        ref = picuda.stationary_state(comp[i], algorithm=alg)
        assert np.array_equal(c.state, ref.data), i
        if i == 0:
            assert np.array_equal(c.state, a.state)
        plan = O.Plan(M.to_oracle(std[i]))
        t = np.zeros(len(plan), dtype=np.complex128)
        t[plan.trace_idx] = plan.trace_val
        s = O.estimated_operator_scale(lambda z: O.apply(plan, z), len(plan))
        assert np.linalg.norm(O.apply(plan, c.state)) / s <= 1e-8 * max(np.linalg.norm(c.state), 1.0)
        assert abs(np.vdot(t, c.state) - 1) <= 1e-8


def test_server_steady_pool_falls_back_to_the_reference_method(torch_cuda):
    """A model with decay and pump channels together has no level sweep (its charge-keeping
    gains point both ways) and no drive: the pool solves it unpreconditioned, the reference's
    method, bitwise as a direct GMRES(50) solve does."""
    model = picuda.Models.local_pump_decay(8, down=1.0, up=0.3)
    c = picuda.compile(model)
    with pytest.raises(picuda.PiError):
        picuda.level_preconditioner(c, coords="population")
    with picuda.Server(precision="fp64", steady_solvers=1) as srv:
        srv.submit_steady(c)
        (done,) = srv.drain()
    assert done.ok, done.message
    ref = picuda.stationary_state(c, algorithm=picuda.GMRESAlgorithm(krylovdim=50, maxiter=2000))
    assert np.array_equal(done.state, ref.data)
