"""The allocation-free multi-dot (pi_mdot_f64_noalloc) against the plan-owned dot.

pi_mdot_f64_noalloc serves callers that cannot allocate device memory when they reduce --
for example a Julia caller whose device memory belongs to its own pool, or a serving loop
that fixes its memory at start-up -- by keeping its partial sums in a static device array
of the library.  This file runs last so that a failure here cannot hide any other result.
"""
import ctypes as C

import numpy as np
import pytest

import picuda
from picuda import _lib
from tests import models as M

pytestmark = pytest.mark.gpu

# Same relative tolerance as the FP64 apply parity tests.
TOL = 1e-12


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _dot_existing(lib, compiled, a, b):
    out = np.zeros(2, dtype=np.float64)
    _lib.check(lib.pi_dot_f64(compiled.handle, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                              _lib.dptr(out)), "pi_dot_f64")
    return complex(out[0], out[1])


def test_noalloc_multidot_matches_plan_dot_twice(torch_cuda):
    torch = torch_cuda
    lib = picuda.load_library()
    compiled = picuda.compile(M.ensemble_c2(30))
    n = len(compiled.basis)
    nv = 7
    g = torch.Generator(device="cuda").manual_seed(7)
    for call in range(2):  # two calls in a row share the static scratch
        V = torch.randn((nv, n), dtype=torch.complex128, device="cuda", generator=g)
        w = torch.randn(n, dtype=torch.complex128, device="cuda", generator=g)
        h = torch.full((nv,), complex(np.nan, np.nan), dtype=torch.complex128, device="cuda")
        rc = lib.pi_mdot_f64_noalloc(C.c_void_p(V.data_ptr()), n, nv, C.c_void_p(w.data_ptr()), n,
                                     C.c_void_p(h.data_ptr()), None)
        _lib.check(rc, "pi_mdot_f64_noalloc")
        torch.cuda.synchronize()
        got = h.cpu().numpy()
        for i in range(nv):
            ref = _dot_existing(lib, compiled, V[i], w)
            assert abs(got[i] - ref) <= TOL * max(abs(ref), 1.0), (call, i, got[i], ref)


def test_noalloc_multidot_rejects_too_many_vectors(torch_cuda):
    torch = torch_cuda
    lib = picuda.load_library()
    V = torch.zeros((33, 16), dtype=torch.complex128, device="cuda")
    w = torch.zeros(16, dtype=torch.complex128, device="cuda")
    h = torch.zeros(33, dtype=torch.complex128, device="cuda")
    rc = lib.pi_mdot_f64_noalloc(C.c_void_p(V.data_ptr()), 16, 33, C.c_void_p(w.data_ptr()), 16,
                                 C.c_void_p(h.data_ptr()), None)
    assert rc == _lib.PI_ERR_INVALID_ARGUMENT
    assert "32" in _lib.last_error()
