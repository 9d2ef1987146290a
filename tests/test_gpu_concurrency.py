"""Several host threads on one compiled model: the default mode serializes their calls like
the reference's locked MatrixFreeLiouvillian (liouvillian.jl:35-60), so every thread gets the
result it would get alone; the "reject" mode raises PiBusy in a thread that finds the model in
use (the ThreadedLiouvillianWorkspace rule, threaded_apply.jl:575)."""
import threading
import time

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


def test_shared_plan_threads_wait_and_match_serial(torch_cuda):
    model = M.driven_c1(10)
    compiled = picuda.compile(model)
    rho0 = picuda.computational_product_state(model.basis, 2)
    ref_exp = picuda.krylov_expv(compiled, rho0, 0.7)
    ref_ss = picuda.stationary_state(compiled, return_info=True).state.data
    results, errors = {}, []

    def worker(k):
        try:
            torch_cuda.cuda.set_device(0)
            for rep in range(3):
                if k % 2 == 0:
                    results[(k, rep)] = ("expv", picuda.krylov_expv(compiled, rho0, 0.7))
                else:
                    results[(k, rep)] = ("ss", picuda.stationary_state(compiled, return_info=True).state.data)
        except Exception as err:  # pragma: no cover - reported below
            errors.append(repr(err))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    assert len(results) == 12
    for (k, rep), (kind, val) in results.items():
        ref = ref_exp if kind == "expv" else ref_ss
        # the same operations in the same order as alone: bitwise equal
        assert np.array_equal(val, ref), (k, rep, kind, np.abs(val - ref).max())


def test_reject_mode_raises_busy_while_in_use(torch_cuda):
    model = M.ensemble_c2(60)
    compiled = picuda.compile(model).set_concurrency("reject")
    rho0 = picuda.computational_product_state(model.basis, 2)
    picuda.krylov_expv(compiled, rho0, 0.05)  # warm: engine and graphs built
    running = threading.Event()
    done = threading.Event()

    def long_call():
        torch_cuda.cuda.set_device(0)
        running.set()
        try:
            while True:  # the probing thread may hold the model for a moment: try again
                try:
                    picuda.solve_dynamics(compiled, rho0, (0.0, 40.0), saveat=0.05, save_states=False,
                                          algorithm=picuda.ExpvAlgorithm(krylovdim=30),
                                          observables={"Jz": picuda.spin_matrices(2)["jz"]})
                    break
                except picuda.PiBusy:
                    time.sleep(0.001)
        finally:
            done.set()

    t = threading.Thread(target=long_call)
    t.start()
    running.wait()
    time.sleep(0.3)  # let the long call take the model (its 800 saved intervals run for seconds)
    busy = False
    deadline = time.time() + 30
    while not done.is_set() and time.time() < deadline:
        try:
            picuda.krylov_expv(compiled, rho0, 0.01)
        except picuda.PiBusy:
            busy = True
            break
        time.sleep(0.001)
    t.join()
    assert busy, "the call that overlapped the running solve should have raised PiBusy"
    # back to waiting: both calls complete
    compiled.set_concurrency("wait")
    out = picuda.krylov_expv(compiled, rho0, 0.01)
    assert np.isfinite(out).all()
