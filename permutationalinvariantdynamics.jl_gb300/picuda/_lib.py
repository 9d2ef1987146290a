"""ctypes binding of libpicuda.so (the C ABI declared in include/picuda.h).

The library is built in-tree (``lib/libpicuda.so`` beside this package).  There is no
CPU fallback: if the library is missing, importing the compute entry points raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_ROOT / "lib" / "libpicuda.so"

PI_OK = 0
PI_ERR_INVALID_ARGUMENT = -1
PI_ERR_DIMENSION = -2
PI_ERR_OUT_OF_MEMORY = -3
PI_ERR_NOT_CONVERGED = -4
PI_ERR_CUDA = -5
PI_ERR_UNSUPPORTED = -6
PI_ERR_NO_DEVICE = -7
PI_ERR_BUSY = -8

PI_CONCURRENCY_WAIT = 0
PI_CONCURRENCY_REJECT = 1

PI_TERM_HAMILTONIAN = 0
PI_TERM_LOCAL_JUMP = 1
PI_TERM_COLLECTIVE_JUMP = 2

PI_FP64 = 0
PI_FP32 = 1
PI_COORDS_REFERENCE = 0
PI_SCHEDULE_AUTO = 0
PI_PRECOND_LEVEL = 0
PI_PRECOND_DRIVE = 1
PI_SCHEDULE_PER_TILE = -1
PI_COORDS_POPULATION = 1


class PiError(RuntimeError):
    """Base error raised for a failing libpicuda call."""


class PiArgumentError(PiError, ValueError):
    """ArgumentError of the reference (invalid or unsupported input)."""


class PiDimensionMismatch(PiError, ValueError):
    """DimensionMismatch of the reference."""


class PiNotConverged(PiError):
    """Krylov solve that did not converge (krylov.jl:873, krylov_extensions.jl:1559-1561)."""


class PiBusy(PiError):
    """A compiled model in use by another host thread, with concurrency mode "reject"
    (the ThreadedLiouvillianWorkspace rule, threaded_apply.jl:575)."""


class pi_capability_t(C.Structure):
    _fields_ = [("functional", C.c_int), ("supports_matrixfree_pi", C.c_int),
                ("device_count", C.c_int), ("sm_count", C.c_int), ("cc_major", C.c_int),
                ("cc_minor", C.c_int), ("total_memory", C.c_size_t),
                ("device_name", C.c_char * 128)]


class pi_plan_info_t(C.Structure):
    _fields_ = [("N", C.c_int), ("nsectors", C.c_int), ("dim", C.c_longlong),
                ("max_block", C.c_int), ("max_terms", C.c_int),
                ("stencil_terms", C.c_longlong), ("device_bytes", C.c_size_t),
                ("batched_kernel", C.c_int)]


class pi_gmres_opts_t(C.Structure):
    _fields_ = [("krylovdim", C.c_int), ("maxiter", C.c_int), ("atol", C.c_double),
                ("rtol", C.c_double), ("operator_scale", C.c_double), ("precision", C.c_int),
                ("use_initial", C.c_int), ("max_refinements", C.c_int), ("coords", C.c_int),
                ("preconditioner", C.c_void_p), ("drive_preconditioner", C.c_void_p)]


class pi_precond_info_t(C.Structure):
    _fields_ = [("coords", C.c_int), ("fp64", C.c_int), ("operator_scale", C.c_double),
                ("regularization", C.c_double), ("chains", C.c_int), ("levels", C.c_int),
                ("entries", C.c_longlong), ("max_level", C.c_int), ("direction", C.c_int),
                ("singular", C.c_int), ("device_bytes", C.c_size_t), ("setup_seconds", C.c_double),
                ("kind", C.c_int), ("max_asymmetry", C.c_double), ("max_nonhermitian", C.c_double)]


class pi_schedule_info_t(C.Structure):
    _fields_ = [("choices", C.c_int), ("tunings", C.c_int), ("schedule", C.c_int), ("items", C.c_int),
                ("resident_max", C.c_int), ("ncand", C.c_int), ("cand", C.c_int * 8), ("cand_us", C.c_double * 8)]


class pi_precond_tables_t(C.Structure):
    _fields_ = [("chain_lev", C.POINTER(C.c_int)), ("lev_ent", C.POINTER(C.c_int)),
                ("elem", C.POINTER(C.c_int)), ("W", C.POINTER(C.c_double)), ("A", C.POINTER(C.c_double)),
                ("C", C.POINTER(C.c_double)), ("gsrc", C.POINTER(C.c_int)), ("G", C.POINTER(C.c_double)),
                ("t0", C.POINTER(C.c_double)), ("v0", C.POINTER(C.c_double)), ("w0", C.POINTER(C.c_double)),
                ("meta", C.c_int * 8), ("sm_coef", C.c_double * 2)]


class pi_gmres_info_t(C.Structure):
    _fields_ = [("converged", C.c_int), ("iterations", C.c_int), ("restarts", C.c_int),
                ("refinements", C.c_int), ("operator_applications", C.c_int),
                ("residual", C.c_double), ("normalized_residual", C.c_double),
                ("trace_error", C.c_double), ("operator_scale", C.c_double),
                ("linear_residual", C.c_double), ("preconditioner_stage", C.c_int)]


class pi_expv_opts_t(C.Structure):
    _fields_ = [("krylovdim", C.c_int), ("atol", C.c_double), ("rtol", C.c_double),
                ("initial_step", C.c_double), ("minimum_step", C.c_double),
                ("maximum_step", C.c_double), ("max_steps", C.c_int), ("safety", C.c_double),
                ("precision", C.c_int)]


class pi_expv_info_t(C.Structure):
    _fields_ = [("converged", C.c_int), ("reached_time", C.c_double),
                ("accepted_steps", C.c_int), ("rejected_steps", C.c_int),
                ("operator_applications", C.c_int), ("arnoldi_factorizations", C.c_int),
                ("trial_evaluations", C.c_int), ("estimated_error", C.c_double)]


class pi_rk4_opts_t(C.Structure):
    _fields_ = [("steps_per_interval", C.c_int), ("precision", C.c_int)]


class pi_rk4_info_t(C.Structure):
    _fields_ = [("steps", C.c_longlong), ("operator_applications", C.c_longlong),
                ("reached_time", C.c_double)]


class pi_arnoldi_info_t(C.Structure):
    _fields_ = [("steps", C.c_int), ("breakdown", C.c_int), ("operator_applications", C.c_int)]


class pi_dynamics_job_t(C.Structure):
    _fields_ = [("plan", C.c_void_p), ("state_dev", C.c_void_p), ("nt", C.c_int),
                ("times", C.POINTER(C.c_double)), ("nobs", C.c_int), ("obs_dev", C.c_void_p),
                ("values_host", C.POINTER(C.c_double))]


class pi_server_opts_t(C.Structure):
    _fields_ = [("krylovdim", C.c_int), ("precision", C.c_int), ("memory_budget", C.c_double),
                ("max_active", C.c_int), ("use_graphs", C.c_int), ("steady_solvers", C.c_int)]


PI_REQUEST_DYNAMICS = 0
PI_REQUEST_STEADY = 1


class pi_request_t(C.Structure):
    _fields_ = [("kind", C.c_int), ("plan", C.c_void_p), ("state_dev", C.c_void_p),
                ("t_final", C.c_double), ("dt", C.c_double), ("atol", C.c_double),
                ("rtol", C.c_double), ("maxiter", C.c_int), ("nobs", C.c_int),
                ("obs_dev", C.c_void_p), ("values_host", C.POINTER(C.c_double)),
                ("tag", C.c_ulonglong)]


class pi_completion_t(C.Structure):
    _fields_ = [("tag", C.c_ulonglong), ("kind", C.c_int), ("status", C.c_int),
                ("submit_time", C.c_double), ("start_time", C.c_double),
                ("finish_time", C.c_double), ("iterations", C.c_int),
                ("operator_applications", C.c_int), ("residual", C.c_double),
                ("trace_error", C.c_double), ("message", C.c_char * 160)]


class pi_server_stats_t(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("admitted", C.c_longlong),
                ("completed", C.c_longlong), ("queued", C.c_longlong), ("active", C.c_longlong),
                ("bytes_in_use", C.c_double), ("ticks", C.c_longlong), ("cycles", C.c_longlong),
                ("arnoldi_steps", C.c_longlong), ("elapsed", C.c_double)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_LL = C.POINTER(C.c_longlong)

# name -> (restype, argtypes); every function declared in include/picuda.h
PROTOTYPES = {
    "pi_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "pi_capability": (C.c_int, [C.POINTER(pi_capability_t)]),
    "pi_plan_create": (C.c_int, [C.c_int, C.c_int, C.c_int, _I, C.c_int, _I, _D, _D, _D,
                                 C.POINTER(_P)]),
    "pi_plan_destroy": (C.c_int, [_P]),
    "pi_plan_info": (C.c_int, [_P, C.POINTER(pi_plan_info_t)]),
    "pi_plan_set_concurrency": (C.c_int, [_P, C.c_int]),
    "pi_plan_sectors": (C.c_int, [_P, _I, _LL, _I]),
    "pi_plan_gt_patterns": (C.c_int, [_P, C.c_int, _I]),
    "pi_plan_trace_functional": (C.c_int, [_P, _LL, _D]),
    "pi_plan_sector_scales": (C.c_int, [_P, _D]),
    "pi_stencil_export": (C.c_int, [C.c_int, C.c_int, C.c_int, _I, C.c_int, _I, _D, _D, _D, _LL,
                                    _I, _D]),
    "pi_collective_block": (C.c_int, [C.c_int, C.c_int, _D, _D]),
    "pi_sector_multiplicity": (C.c_int, [C.c_int, C.c_int, _D, _D]),
    "pi_apply_f64": (C.c_int, [_P, _P, _P, C.c_int, C.c_longlong, _P]),
    "pi_apply_f32": (C.c_int, [_P, _P, _P, C.c_int, C.c_longlong, C.c_int, _P]),
    "pi_apply_f32_em": (C.c_int, [_P, _P, _P, C.c_int, C.c_longlong, C.c_int, _P]),
    "pi_apply_f32_em_tuning": (C.c_int, [_P, C.c_int, C.c_int, _I, _I, _D]),
    "pi_apply_f32_em_select": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int]),
    "pi_apply_host_f64": (C.c_int, [_P, _P, _P, C.c_int]),
    "pi_apply_host_f32": (C.c_int, [_P, _P, _P, C.c_int, C.c_int]),
    "pi_dot_f64": (C.c_int, [_P, _P, _P, _D]),
    "pi_mdot_f64_noalloc": (C.c_int, [_P, C.c_longlong, C.c_int, _P, C.c_longlong, _P, _P]),
    "pi_gmres_default_opts": (None, [C.POINTER(pi_gmres_opts_t)]),
    "pi_steady_state": (C.c_int, [_P, _P, C.POINTER(pi_gmres_opts_t), C.POINTER(pi_gmres_info_t)]),
    "pi_precond_create": (C.c_int, [_P, C.c_int, C.c_double, C.c_double, C.POINTER(_P)]),
    "pi_precond_create_drive": (C.c_int, [_P, C.c_int, C.c_double, C.POINTER(_P)]),
    "pi_precond_drive_export": (C.c_int, [C.c_int, C.c_int, C.c_int, _I, C.c_int, _I, _D, _D, _D, _LL, _D, _D, _D, _D]),
    "pi_precond_destroy": (C.c_int, [_P]),
    "pi_precond_info": (C.c_int, [_P, C.POINTER(pi_precond_info_t)]),
    "pi_precond_apply": (C.c_int, [_P, _P, _P, _P]),
    "pi_precond_export": (C.c_int, [C.c_int, C.c_int, C.c_int, _I, C.c_int, _I, _D, _D, _D, C.c_int,
                                    C.c_double, C.c_double, _LL, C.POINTER(pi_precond_tables_t)]),
    "pi_expv_default_opts": (None, [C.POINTER(pi_expv_opts_t)]),
    "pi_expv": (C.c_int, [_P, _P, C.c_double, C.POINTER(pi_expv_opts_t),
                          C.POINTER(pi_expv_info_t)]),
    "pi_solve_dynamics": (C.c_int, [_P, _P, C.c_int, _D, C.c_int, _P, _D,
                                    C.POINTER(pi_expv_opts_t), C.POINTER(pi_expv_info_t)]),
    "pi_plan_adjoint": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "pi_stencil_export_adjoint": (C.c_int, [C.c_int, C.c_int, C.c_int, _I, C.c_int, _I, _D, _D, _D, _LL,
                                            _I, _D]),
    "pi_arnoldi": (C.c_int, [_P, _P, C.c_int, _P, C.c_longlong, _D, C.POINTER(pi_arnoldi_info_t)]),
    "pi_combine_f64": (C.c_int, [_P, _P, C.c_longlong, C.c_int, _D, C.c_int, _P, C.c_longlong]),
    "pi_rk4_default_opts": (None, [C.POINTER(pi_rk4_opts_t)]),
    "pi_evolve": (C.c_int, [_P, _P, _P, C.c_double, C.c_double, C.POINTER(pi_rk4_opts_t),
                            C.POINTER(pi_rk4_info_t)]),
    "pi_solve_dynamics_rk4": (C.c_int, [_P, _P, C.c_int, _D, C.c_int, _P, _D,
                                        C.POINTER(pi_rk4_opts_t), C.POINTER(pi_rk4_info_t)]),
    "pi_expv_batch": (C.c_int, [C.c_int, C.POINTER(_P), C.POINTER(_P), _D,
                                C.POINTER(pi_expv_opts_t), C.POINTER(pi_expv_info_t)]),
    "pi_dynamics_batch": (C.c_int, [C.c_int, C.POINTER(pi_dynamics_job_t),
                                    C.POINTER(pi_expv_opts_t), C.POINTER(pi_expv_info_t)]),
    "pi_steady_state_batch": (C.c_int, [C.c_int, C.POINTER(_P), C.POINTER(_P),
                                        C.POINTER(pi_gmres_opts_t),
                                        C.POINTER(pi_gmres_info_t)]),
    "pi_engine_set_apply_schedule": (C.c_int, [C.c_int]),
    "pi_engine_schedule_info": (C.c_int, [C.POINTER(pi_schedule_info_t)]),
    "pi_server_default_opts": (None, [C.POINTER(pi_server_opts_t)]),
    "pi_server_create": (C.c_int, [C.POINTER(pi_server_opts_t), C.c_int, C.POINTER(_P)]),
    "pi_server_submit": (C.c_int, [_P, C.POINTER(pi_request_t)]),
    "pi_server_poll": (C.c_int, [_P, C.POINTER(pi_completion_t), C.c_int, _I, C.c_int]),
    "pi_server_stats": (C.c_int, [_P, C.POINTER(pi_server_stats_t)]),
    "pi_server_destroy": (C.c_int, [_P]),
}

_lib = None


def load(path: str | os.PathLike | None = None):
    """Loads libpicuda.so once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise PiError(f"libpicuda.so is not built ({p}); run __graft_entry__.build() or "
                      "python permutationalinvariantdynamics.jl_gb300/build_lib.py")
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().pi_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, what: str = "libpicuda call") -> None:
    if rc == PI_OK:
        return
    msg = f"{what}: {last_error()}"
    if rc in (PI_ERR_INVALID_ARGUMENT, PI_ERR_UNSUPPORTED):
        raise PiArgumentError(msg)
    if rc == PI_ERR_DIMENSION:
        raise PiDimensionMismatch(msg)
    if rc == PI_ERR_NOT_CONVERGED:
        raise PiNotConverged(msg)
    if rc == PI_ERR_BUSY:
        raise PiBusy(msg)
    raise PiError(f"{msg} (status {rc})")


def dptr(a):
    """ctypes double pointer of a contiguous numpy array."""
    return a.ctypes.data_as(_D)


def iptr(a):
    return a.ctypes.data_as(_I)


def llptr(a):
    return a.ctypes.data_as(_LL)
