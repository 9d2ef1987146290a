"""The allocation-free multi-dot (pi_mdot_f64_noalloc) against the plan-owned dot and numpy.

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


def _noalloc(lib, V, ldv, nv, w, n, h):
    rc = lib.pi_mdot_f64_noalloc(C.c_void_p(V.data_ptr()), ldv, nv, C.c_void_p(w.data_ptr()), n,
                                 C.c_void_p(h.data_ptr()), None)
    _lib.check(rc, "pi_mdot_f64_noalloc")


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
        _noalloc(lib, V, n, nv, w, n, h)
        torch.cuda.synchronize()
        got = h.cpu().numpy()
        for i in range(nv):
            ref = _dot_existing(lib, compiled, V[i], w)
            assert abs(got[i] - ref) <= TOL * max(abs(ref), 1.0), (call, i, got[i], ref)


# n = 200,003 with ldv > n: the partial-sum grid reaches the cap of 256 blocks shared by
# the 8-vector groups (gy = 4 groups of 8 at nv = 32, 2 at nv = 9 with a partly filled last
# group, 1 at nv = 1).
@pytest.mark.parametrize("nv", [1, 9, 32])
def test_noalloc_multidot_groups_and_leading_dimension(torch_cuda, nv):
    torch = torch_cuda
    lib = picuda.load_library()
    compiled = picuda.compile(M.ensemble_c2(30))
    n, ldv = 200_003, 200_003 + 37
    g = torch.Generator(device="cuda").manual_seed(100 + nv)
    for call in range(2):
        Vs = torch.randn((nv, ldv), dtype=torch.complex128, device="cuda", generator=g)
        w = torch.randn(n, dtype=torch.complex128, device="cuda", generator=g)
        h = torch.full((nv,), complex(np.nan, np.nan), dtype=torch.complex128, device="cuda")
        _noalloc(lib, Vs, ldv, nv, w, n, h)
        torch.cuda.synchronize()
        got = h.cpu().numpy()
        Vh = Vs.cpu().numpy()[:, :n]
        wh = w.cpu().numpy()
        ref = Vh.conj() @ wh
        bound = np.abs(Vh) @ np.abs(wh)  # sum |V_i||w|: the scale of the rounding error
        assert np.all(np.abs(got - ref) <= TOL * bound), (call, nv, np.max(np.abs(got - ref) / bound))
        # the existing entry point on the plan's dot: only defined for vectors of the plan's
        # length, so compare the first group of columns cut to a PI vector of that length
        npi = len(compiled.basis)
        for i in range(min(nv, 3)):
            a = Vs[i, :npi].contiguous()
            b = w[:npi].contiguous()
            h1 = torch.empty(1, dtype=torch.complex128, device="cuda")
            _noalloc(lib, a, npi, 1, b, npi, h1)
            torch.cuda.synchronize()
            ref1 = _dot_existing(lib, compiled, a, b)
            assert abs(h1.cpu().numpy()[0] - ref1) <= TOL * max(abs(ref1), 1.0)


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
