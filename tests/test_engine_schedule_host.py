"""Host-side behaviour of the engine schedule setting and the preconditioner options (no
device): argument validation in the Python layer and in the C ABI, and the schedule record
before any engine has chosen."""
import pytest

import picuda
from picuda import _lib


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    picuda.load_library()


@pytest.fixture
def restore():
    yield
    picuda.set_engine_schedule("auto")


def test_schedule_setting_validation(restore):
    for bad in (0, -3, 0.5, "persistent", True, None):
        with pytest.raises(picuda.PiArgumentError):
            picuda.set_engine_schedule(bad)
    lib = picuda.load_library()
    assert lib.pi_engine_set_apply_schedule(-2) == _lib.PI_ERR_INVALID_ARGUMENT
    assert lib.pi_engine_set_apply_schedule(65) == _lib.PI_ERR_INVALID_ARGUMENT
    for ok in ("auto", "per_tile", 1, 3, 64):
        picuda.set_engine_schedule(ok)
    assert lib.pi_engine_schedule_info(None) == _lib.PI_ERR_INVALID_ARGUMENT


def test_schedule_record_shape():
    info = picuda.engine_schedule_info()
    assert set(info) == {"choices", "tunings", "schedule", "items", "resident_max", "candidates_us"}
    assert info["tunings"] <= info["choices"]


def test_gmres_algorithm_rejects_misplaced_preconditioners():
    with pytest.raises(picuda.PiArgumentError):
        picuda.GMRESAlgorithm(preconditioner="level")
    with pytest.raises(picuda.PiArgumentError):
        picuda.GMRESAlgorithm(drive_preconditioner=object())


def test_drive_export_rejects_null_counts():
    lib = picuda.load_library()
    assert lib.pi_precond_drive_export(4, 2, 0, None, 0, None, None, None, None, None, None, None, None,
                                       None) == _lib.PI_ERR_INVALID_ARGUMENT


def test_c_abi_rejects_bad_preconditioner_arguments():
    lib = picuda.load_library()
    out = __import__("ctypes").c_void_p()
    assert lib.pi_precond_create_drive(None, 1, 0.0, __import__("ctypes").byref(out)) == _lib.PI_ERR_INVALID_ARGUMENT


def test_server_options_reject_out_of_range_solver_pools():
    import ctypes as C
    lib = picuda.load_library()
    o = _lib.pi_server_opts_t()
    lib.pi_server_default_opts(C.byref(o))
    assert o.steady_solvers == 0
    o.steady_solvers = -1
    h = C.c_void_p()
    assert lib.pi_server_create(C.byref(o), 0, C.byref(h)) == _lib.PI_ERR_INVALID_ARGUMENT
    o.steady_solvers = 65
    assert lib.pi_server_create(C.byref(o), 0, C.byref(h)) == _lib.PI_ERR_INVALID_ARGUMENT
