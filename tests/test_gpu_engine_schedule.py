"""Step-apply schedules of the batched FP32 engine: one block per (instance, sector-tile)
item, or a persistent launch of k blocks per SM that prefetches each next tile's stage.
Every schedule computes every entry with the same arithmetic, so engine results must be
bitwise equal; the autotuner's record must name what it timed and what it picked."""
import numpy as np
import pytest

import picuda
from picuda import _lib
from tests import models as M

pytestmark = pytest.mark.gpu

EXC = np.array([[0, 0], [0, 1]])
JZ = np.diag([0.5, -0.5])


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture
def restore_schedule():
    yield
    picuda.set_engine_schedule("auto")


def _job_set():
    """Canonical plans of uneven size (about a thousand tiles: several per persistent block),
    a general-stencil plan (the persistent kernel's synchronous path) and a model smaller than
    the Krylov dimension (its cycles stop early, so its items are skipped mid-cycle)."""
    return [M.scan_model(120, 1.1, 0.2, 0.05), M.scan_model(64, 0.5, 0.4, 0.1), M.general(6, 3),
            M.driven_c1(3), M.scan_model(97, 1.7, 0.1, 0.15), M.ensemble_c2(33)]


def _run_dynamics(models):
    alg = picuda.ExpvAlgorithm(precision="mixed")
    rho0 = [picuda.computational_product_state(m.basis, 2) for m in models]
    return picuda.solve_dynamics_batch(models, rho0, (0.0, 0.3), algorithm=alg, saveat=0.1,
                                       observables={"exc": EXC, "jz": JZ})


@pytest.mark.parametrize("schedule", [1, 2, 3, "auto"])
def test_dynamics_bitwise_equal_across_schedules(torch_cuda, restore_schedule, schedule):
    models = _job_set()
    picuda.set_engine_schedule("per_tile")
    ref_res, ref_fin = _run_dynamics(models)
    assert picuda.engine_schedule_info()["schedule"] == "per_tile"
    picuda.set_engine_schedule(schedule)
    res, fin = _run_dynamics(models)
    info = picuda.engine_schedule_info()
    if schedule != "auto":
        assert info["schedule"] == min(schedule, info["resident_max"])
    for i in range(len(models)):
        assert np.array_equal(fin[i], ref_fin[i]), (schedule, i)
        for k in ("exc", "jz"):
            assert np.array_equal(res[i].values[k], ref_res[i].values[k]), (schedule, i, k)


def test_mixed_steady_state_bitwise_equal_across_schedules(torch_cuda, restore_schedule):
    """Bordered cycles in reference coordinates take the same two-stage path.  The N = 40
    instance stagnates unpreconditioned, so the solves stop at the iteration cap; whatever
    they return must be the same under both schedules."""
    models = [M.driven_c1(12), M.scan_model(40, 0.5, 0.45, 0.2), M.general(5, 9)]
    alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=400, precision="mixed")
    out = {}
    for schedule in ("per_tile", 1):
        picuda.set_engine_schedule(schedule)
        states, infos = picuda.stationary_state_batch(models, algorithm=alg, return_info=True,
                                                      raise_on_failure=False)
        out[schedule] = ([s.data for s in states], infos)
    for a, b, ia, ib in zip(out["per_tile"][0], out[1][0], out["per_tile"][1], out[1][1]):
        assert ia["converged"] == ib["converged"]
        assert ia["iterations"] == ib["iterations"]
        assert ia["normalized_residual"] == ib["normalized_residual"]
        assert np.array_equal(a, b)


def test_autotuner_times_candidates_and_caches_the_choice(torch_cuda, restore_schedule):
    picuda.set_engine_schedule("auto")
    before = picuda.engine_schedule_info()
    # a job-set shape no other test uses: a single large canonical instance
    _run_dynamics([M.scan_model(150, 0.9, 0.3, 0.1)])
    first = picuda.engine_schedule_info()
    assert first["choices"] > before["choices"]
    assert first["resident_max"] >= 1
    if first["tunings"] > before["tunings"]:  # timed now (not cached by an earlier run)
        cands = first["candidates_us"]
        assert "per_tile" in cands and "1" in cands
        assert all(t > 0 for t in cands.values())
        best = min(cands, key=cands.get)
        assert str(first["schedule"]) == best
    # the same shape again: the cached choice, no new timing
    _run_dynamics([M.scan_model(150, 0.9, 0.3, 0.1)])
    again = picuda.engine_schedule_info()
    assert again["tunings"] == first["tunings"]
    assert again["schedule"] == first["schedule"]
    assert again["candidates_us"] == {}


def test_schedule_argument_errors(torch_cuda, restore_schedule):
    with pytest.raises(picuda.PiArgumentError):
        picuda.set_engine_schedule(0.5)
    with pytest.raises(picuda.PiArgumentError):
        picuda.set_engine_schedule(0)
    lib = picuda.load_library()
    assert lib.pi_engine_set_apply_schedule(-2) == _lib.PI_ERR_INVALID_ARGUMENT
    assert "schedule" in _lib.last_error()
    assert lib.pi_engine_set_apply_schedule(65) == _lib.PI_ERR_INVALID_ARGUMENT
