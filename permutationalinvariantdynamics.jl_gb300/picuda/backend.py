"""compile(model; backend=:cuda), apply!, solve_dynamics and stationary_state over libpicuda.

Mirrors the reference's high-level entry points (src/liouvillian.jl:4040-4098 compile,
:4165-4189 apply!/mul!, src/highlevel.jl:321-371 stationary_state, :559-733 solve_dynamics,
src/accelerators.jl:83-85 accelerator_capability) for the CUDA backend.  Every numerical
step runs in libpicuda on the GPU; device buffers come from torch (plumbing only).  There
is no CPU fallback: without the library or a GPU these functions raise.
"""
from __future__ import annotations

import ctypes as C
import threading
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import PiArgumentError, PiDimensionMismatch
from .core import PIModel, PIOperator, PIState, collective_operator

_DEFAULT_MEMORY_BUDGET = 512 * 1024 ** 2


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise _lib.PiError("the CUDA backend needs a CUDA device; no CPU fallback exists")
    return torch


@dataclass(frozen=True)
class AcceleratorCapability:
    """accelerators.jl:13-25 fields for backend :cuda."""
    backend: str
    extension_loaded: bool
    functional: bool
    supports_sparse_pi: bool
    supports_matrixfree_pi: bool
    rhs_kinds: tuple
    scalar_types: tuple
    index_type: str
    transfer_policy: str
    reason: str
    message: str
    device_name: str = ""
    sm_count: int = 0


def accelerator_capability(backend: str = "cuda") -> AcceleratorCapability:
    """Reports whether the CUDA backend is loaded and functional (accelerators.jl:83-85)."""
    if backend != "cuda":
        return AcceleratorCapability(backend, False, False, False, False, (), (), "Int", "unsupported",
                                     "unknown_backend",
                                     f"accelerator backend :{backend} is not registered")
    try:
        lib = _lib.load()
    except _lib.PiError as err:
        return AcceleratorCapability("cuda", False, False, False, False, ("vector", "matrix"),
                                     ("ComplexF64", "ComplexF32"), "Int32", "explicit_once",
                                     "extension_not_loaded", str(err))
    cap = _lib.pi_capability_t()
    rc = lib.pi_capability(C.byref(cap))
    functional = rc == _lib.PI_OK and bool(cap.functional)
    return AcceleratorCapability(
        "cuda", True, functional, False, functional, ("vector", "matrix"), ("ComplexF64", "ComplexF32"),
        "Int32", "explicit_once", "ready" if functional else "device_unavailable",
        "libpicuda matrix-free Schur-block backend" if functional else _lib.last_error(),
        cap.device_name.decode(errors="replace"), cap.sm_count)


def _term_arrays(model: PIModel):
    kinds = np.array([t.kind for t in model.terms], dtype=np.int32)
    ops = np.zeros((max(len(model.terms), 1), 8), dtype=np.float64)
    for i, t in enumerate(model.terms):
        ops[i] = t.operator.reshape(-1, order="F").view(np.float64)
    rates = np.array([t.rate for t in model.terms] or [0.0], dtype=np.float64)
    hbar = np.array([t.hbar for t in model.terms] or [1.0], dtype=np.float64)
    ks = np.array(model.basis.ks, dtype=np.int32)
    return kinds, np.ascontiguousarray(ops), rates, hbar, ks


def stencil_tables(model: PIModel, adjoint: bool = False):
    """Host-only export of the lowered stencil (pi_stencil_export, or the adjoint plan's with
    adjoint=True): (terms[n,8], coef[c])."""
    lib = _lib.load()
    fn = lib.pi_stencil_export_adjoint if adjoint else lib.pi_stencil_export
    kinds, ops, rates, hbar, ks = _term_arrays(model)
    counts = np.zeros(2, dtype=np.int64)
    args = (model.basis.N, model.basis.d, len(ks), _lib.iptr(ks), len(model.terms), _lib.iptr(kinds),
            _lib.dptr(ops), _lib.dptr(rates), _lib.dptr(hbar), _lib.llptr(counts))
    _lib.check(fn(*args, None, None), "pi_stencil_export")
    table = np.zeros((int(counts[0]), 8), dtype=np.int32)
    coef = np.zeros(int(counts[1]), dtype=np.complex128)
    _lib.check(fn(*args, _lib.iptr(table), _lib.dptr(coef.view(np.float64))), "pi_stencil_export")
    return table, coef


class CompiledPIModel:
    """A model lowered and uploaded once to the GPU (CompiledPIModel, liouvillian.jl:3495-3501)."""

    def __init__(self, model: PIModel, memory_budget=_DEFAULT_MEMORY_BUDGET):
        self.model = model
        self.basis = model.basis
        self.backend = "cuda"
        lib = _lib.load()
        kinds, ops, rates, hbar, ks = _term_arrays(model)
        handle = C.c_void_p()
        _lib.check(lib.pi_plan_create(model.basis.N, model.basis.d, len(ks), _lib.iptr(ks),
                                      len(model.terms), _lib.iptr(kinds), _lib.dptr(ops),
                                      _lib.dptr(rates), _lib.dptr(hbar), C.byref(handle)),
                   "compile(model; backend=:cuda)")
        self._handle = handle
        info = _lib.pi_plan_info_t()
        _lib.check(lib.pi_plan_info(handle, C.byref(info)), "pi_plan_info")
        self.info = {f: getattr(info, f) for f, _ in info._fields_}
        if len(self.basis) != info.dim:
            raise PiDimensionMismatch("library and host bases disagree")
        if memory_budget is not None and np.isfinite(memory_budget) and info.device_bytes > memory_budget:
            self.close()
            raise PiArgumentError("the prepared CUDA plan exceeds memory_budget")

    @property
    def handle(self):
        if self._handle is None:
            raise _lib.PiError("the compiled model has been closed")
        return self._handle

    def close(self):
        adj = self.__dict__.pop("_adjoint", None)
        if adj is not None:
            adj.close()
        if getattr(self, "_handle", None) is not None:
            _lib.load().pi_plan_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self.basis)

    @property
    def shape(self):
        n = len(self.basis)
        return (n, n)

    def isautonomous(self):
        return True

    def set_concurrency(self, mode: str = "wait"):
        """How concurrent calls on this compiled model from several host threads behave:
        "wait" (default) serializes them like the reference's locked MatrixFreeLiouvillian
        (liouvillian.jl:35-60); "reject" raises PiBusy in the later caller, the rule of the
        reference's per-task workspaces (threaded_apply.jl:575)."""
        modes = {"wait": _lib.PI_CONCURRENCY_WAIT, "reject": _lib.PI_CONCURRENCY_REJECT}
        if mode not in modes:
            raise PiArgumentError("mode must be 'wait' or 'reject'")
        _lib.check(_lib.load().pi_plan_set_concurrency(self.handle, modes[mode]), "set_concurrency")
        return self

    def adjoint(self):
        """The adjoint generator (pi_plan_adjoint), built on first use and kept with the model."""
        adj = getattr(self, "_adjoint", None)
        if adj is None:
            handle = C.c_void_p()
            _lib.check(_lib.load().pi_plan_adjoint(self.handle, C.byref(handle)), "apply_adjoint!")
            adj = CompiledPIModel.__new__(CompiledPIModel)
            adj.model, adj.basis, adj.backend, adj._handle = self.model, self.basis, "cuda", handle
            info = _lib.pi_plan_info_t()
            _lib.check(_lib.load().pi_plan_info(handle, C.byref(info)), "pi_plan_info")
            adj.info = {f: getattr(info, f) for f, _ in info._fields_}
            adj._primary = self  # keeps the forward plan alive while the adjoint is in use
            self._adjoint = adj
        return adj

    # -- basis maps straight from the library (bit-exact) --------------------------------
    def library_sectors(self):
        lib = _lib.load()
        S = self.info["nsectors"]
        ks = np.zeros(S, dtype=np.int32)
        offs = np.zeros(S, dtype=np.int64)
        dims = np.zeros(S, dtype=np.int32)
        _lib.check(lib.pi_plan_sectors(self.handle, _lib.iptr(ks), _lib.llptr(offs), _lib.iptr(dims)),
                   "pi_plan_sectors")
        return ks, offs, dims

    def library_patterns(self, sector):
        lib = _lib.load()
        n = self.basis.dims[sector]
        out = np.zeros(3 * n, dtype=np.int32)
        _lib.check(lib.pi_plan_gt_patterns(self.handle, sector, _lib.iptr(out)), "pi_plan_gt_patterns")
        return out.reshape(n, 3)

    def library_trace_functional(self):
        lib = _lib.load()
        nd = sum(self.basis.dims)
        idx = np.zeros(nd, dtype=np.int64)
        val = np.zeros(nd, dtype=np.float64)
        _lib.check(lib.pi_plan_trace_functional(self.handle, _lib.llptr(idx), _lib.dptr(val)),
                   "pi_plan_trace_functional")
        return idx, val

    def sector_scales(self):
        lib = _lib.load()
        out = np.zeros(self.info["nsectors"], dtype=np.float64)
        _lib.check(lib.pi_plan_sector_scales(self.handle, _lib.dptr(out)), "pi_plan_sector_scales")
        return out


def compile(model: PIModel, backend: str = "cuda", memory_budget=_DEFAULT_MEMORY_BUDGET):
    """compile(model; backend=:cuda) (liouvillian.jl:4040-4098)."""
    if backend != "cuda":
        raise PiArgumentError("this package implements backend=:cuda only")
    if not isinstance(model, PIModel):
        raise PiArgumentError("compile requires a PIModel")
    return CompiledPIModel(model, memory_budget)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def apply_(y, compiled: CompiledPIModel, x, t=0.0, p=None, precision="fp64", coords="reference"):
    """apply!(y, compiled, x, t, p) (liouvillian.jl:4165-4171).

    x, y: torch CUDA tensors (complex128 for fp64, complex64 for fp32) of shape (dim,) or
    (ncols, dim) -- device-resident, no transfers -- or numpy complex128 arrays (the
    host-buffer convenience path, fp64 only).  Aliasing of x and y is rejected.
    """
    if p is not None:
        raise PiArgumentError("the CUDA backend applies autonomous generators (parameters=nothing)")
    lib = _lib.load()
    n = len(compiled.basis)
    if isinstance(x, np.ndarray):
        if precision != "fp64":
            raise PiArgumentError("host-buffer apply is FP64")
        if x.dtype != np.complex128 or y.dtype != np.complex128:
            raise PiArgumentError("host buffers must be complex128")
        if x.shape != y.shape or x.shape[-1] != n:
            raise PiDimensionMismatch("Liouvillian vector has the wrong length")
        if np.shares_memory(x, y):
            raise PiArgumentError("source and destination must not share storage")
        xc = np.ascontiguousarray(x)
        ncols = 1 if x.ndim == 1 else x.shape[0]
        out = np.empty_like(xc) if not y.flags.c_contiguous else y
        _lib.check(lib.pi_apply_host_f64(compiled.handle, out.ctypes.data_as(C.c_void_p),
                                         xc.ctypes.data_as(C.c_void_p), ncols), "apply!")
        if out is not y:
            y[...] = out
        return y
    torch = _torch()
    if x.shape != y.shape or x.shape[-1] != n or not x.is_cuda or not y.is_cuda:
        raise PiDimensionMismatch("Liouvillian vector has the wrong length or is not on the GPU")
    if not (x.is_contiguous() and y.is_contiguous()):
        raise PiArgumentError("device vectors must be contiguous")
    ncols = 1 if x.dim() == 1 else x.shape[0]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if precision == "fp64":
        if x.dtype != torch.complex128 or y.dtype != torch.complex128:
            raise PiArgumentError("fp64 apply needs complex128 tensors")
        _lib.check(lib.pi_apply_f64(compiled.handle, _ptr(y), _ptr(x), ncols, n, stream), "apply!")
    elif precision == "fp32":
        if x.dtype != torch.complex64 or y.dtype != torch.complex64:
            raise PiArgumentError("fp32 apply needs complex64 tensors")
        cc = _lib.PI_COORDS_POPULATION if coords == "population" else _lib.PI_COORDS_REFERENCE
        _lib.check(lib.pi_apply_f32(compiled.handle, _ptr(y), _ptr(x), ncols, n, cc, stream), "apply!")
    else:
        raise PiArgumentError("precision must be 'fp64' or 'fp32'")
    return y


def apply_adjoint_(y, compiled: CompiledPIModel, x, t=0.0, p=None, precision="fp64", coords="reference"):
    """apply_adjoint!(y, compiled, x, t, p) (liouvillian.jl:4266, 3275-3324): y = L^H x with
    L^H the conjugate transpose of the PI-coordinate generator, through the adjoint plan.
    Same arguments and checks as apply_."""
    return apply_(y, compiled.adjoint(), x, t, p, precision=precision, coords=coords)


def krylov_liouvillian_spectrum(L, nev=6, krylovdim=None, which="LR", initial_vector=None, atol=1e-10,
                                rtol=1e-8, vectors=False, rng=None, require_convergence=True):
    """krylov_liouvillian_spectrum(L; nev, krylovdim=max(20, 2nev+4), which=:LR,
    initial_vector, atol, rtol, vectors, rng, require_convergence) (krylov.jl:914-962).

    The Arnoldi process runs on the GPU (pi_arnoldi); the projected eigenproblem, the Ritz
    ordering (:LR largest real part, :LM / :SM largest / smallest modulus, krylov.jl:893-898)
    and the residual estimates |H[k+1,k] y_k| with tolerance atol + rtol * max_j |H[:,j]|
    follow the reference on the host.  Returns a dict with the reference's info fields."""
    torch = _torch()
    compiled = _as_compiled(L)
    n = len(compiled.basis)
    if not (0 < nev <= n):
        raise PiArgumentError("nev must lie between 1 and the operator dimension")
    if which not in ("LR", "LM", "SM"):
        raise PiArgumentError("which must be :LR, :LM, or :SM")
    krylovdim = max(20, 2 * nev + 4) if krylovdim is None else int(krylovdim)
    m = min(n, max(krylovdim, nev + 1))
    if m > 127:
        raise PiArgumentError("the CUDA Arnoldi process supports krylov dimensions up to 127")
    if initial_vector is None:
        rng = rng if rng is not None else np.random.default_rng()
        q = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
    else:
        q = np.asarray(initial_vector, dtype=np.complex128)
        if q.shape != (n,):
            raise PiDimensionMismatch("initial_vector has wrong length")
    v0 = torch.from_numpy(np.ascontiguousarray(q)).cuda()
    V = torch.zeros((m + 1, n), dtype=torch.complex128, device="cuda")
    H = np.zeros((m, m + 1), dtype=np.complex128)  # column-major (m+1) x m
    info = _lib.pi_arnoldi_info_t()
    torch.cuda.synchronize()
    lib = _lib.load()
    _lib.check(lib.pi_arnoldi(compiled.handle, _ptr(v0), m, _ptr(V), n, _lib.dptr(H.view(np.float64)),
                              C.byref(info)), "krylov_liouvillian_spectrum")
    H = H.T  # (m+1) x m
    k = info.steps
    vals, Y = np.linalg.eig(H[:k, :k])
    key = {"LR": -vals.real, "LM": -np.abs(vals), "SM": np.abs(vals)}[which]
    order = np.argsort(key, kind="stable")[:min(nev, k)]
    vals, Y = vals[order], Y[:, order]
    residuals = np.abs(H[k, k - 1] * Y[-1, :])
    scale = max(max((np.linalg.norm(H[:k + 1, j]) for j in range(k)), default=0.0), np.finfo(float).tiny)
    tolerance = atol + rtol * scale
    converged = residuals <= tolerance
    if require_convergence and not np.all(converged):
        raise PiArgumentError(f"Arnoldi spectrum did not converge; maximum requested Ritz residual="
                              f"{residuals.max()}; increase krylovdim")
    out = dict(values=vals, residuals=residuals, converged=converged, iterations=k, krylov_dimension=m,
               dimension=n, which=which, residual_scale=scale, residual_tolerance=tolerance,
               workspace_reused=False, operator_applications=info.operator_applications)
    if vectors:
        Yc = np.ascontiguousarray(Y.T)  # ncols x k == k x ncols column-major
        vec = torch.zeros((len(order), n), dtype=torch.complex128, device="cuda")
        _lib.check(lib.pi_combine_f64(compiled.handle, _ptr(V), n, k, _lib.dptr(Yc.view(np.float64)), len(order),
                                      _ptr(vec), n), "krylov_liouvillian_spectrum")
        out["vectors"] = vec.cpu().numpy().T
    return out


# Vectors per pi_mdot_f64_noalloc call (the capacity of its static scratch) and the largest
# basis pi_combine_f64 combines.
_MDOT_VECTORS = 32
_COMBINE_VECTORS = 128
# Serialises the solves of this process that use pi_mdot_f64_noalloc's shared scratch; each
# solve has synchronised its last multi-dot before it releases the lock.
_NOALLOC_LOCK = threading.Lock()


class _DeviceKrylovSpace:
    """Vector storage and vector operations of the harmonic Arnoldi process on the GPU.

    A block of m vectors is an (m, dim) complex128 CUDA tensor, one vector per row.  L x runs
    through pi_apply_f64 and projections and norms through pi_mdot_f64_noalloc, both on
    torch's current stream; basis combinations run through pi_combine_f64, which works on
    the plan's own stream and returns after it finished, so the current stream is drained
    before each combination."""

    def __init__(self, compiled: CompiledPIModel, m: int):
        self.torch = _torch()
        self.compiled = compiled
        self.n = len(compiled.basis)
        self.lib = _lib.load()
        self.h = self.torch.empty(max(m, 1), dtype=self.torch.complex128, device="cuda")
        self.tmp = self.torch.empty(self.n, dtype=self.torch.complex128, device="cuda")

    def block(self, m):
        return self.torch.zeros((m, self.n), dtype=self.torch.complex128, device="cuda")

    def upload(self, v):
        return self.torch.from_numpy(np.ascontiguousarray(v, dtype=np.complex128)).cuda()

    def copy(self, v):
        return v.clone()

    def download(self, rows):
        """(dim, c) numpy array of the c rows."""
        return rows.cpu().numpy().T.copy()

    def apply(self, dst, src):
        apply_(dst, self.compiled, src)

    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def _mdot(self, M, k, q):
        for s in range(0, k, _MDOT_VECTORS):
            c = min(_MDOT_VECTORS, k - s)
            _lib.check(self.lib.pi_mdot_f64_noalloc(_ptr(M[s]), self.n, c, _ptr(q), self.n, _ptr(self.h[s:]),
                                                    self._stream()), "harmonic_arnoldi_spectrum")

    def dots(self, M, k, q):
        """conj(M[i]) . q for i < k, as a numpy vector."""
        self._mdot(M, k, q)
        return self.h[:k].cpu().numpy()

    def norm(self, q):
        _lib.check(self.lib.pi_mdot_f64_noalloc(_ptr(q), self.n, 1, _ptr(q), self.n, _ptr(self.h), self._stream()),
                   "harmonic_arnoldi_spectrum")
        return float(np.sqrt(max(self.h[0].item().real, 0.0)))

    def combine(self, M, k, Y):
        """Rows sum_i Y[i, c] M[i] for the columns c of the k x c matrix Y."""
        Yc = np.ascontiguousarray(np.asarray(Y, dtype=np.complex128).T)  # c x k row-major = k x c column-major
        out = self.torch.empty((Yc.shape[0], self.n), dtype=self.torch.complex128, device="cuda")
        self.torch.cuda.synchronize()
        _lib.check(self.lib.pi_combine_f64(self.compiled.handle, _ptr(M), self.n, k, _lib.dptr(Yc.view(np.float64)),
                                           Yc.shape[0], _ptr(out), self.n), "harmonic_arnoldi_spectrum")
        return out

    def subtract(self, q, M, k, coef):
        """q -= sum_i coef[i] M[i]."""
        c = np.ascontiguousarray(coef, dtype=np.complex128)
        self.torch.cuda.synchronize()
        _lib.check(self.lib.pi_combine_f64(self.compiled.handle, _ptr(M), self.n, k, _lib.dptr(c.view(np.float64)),
                                           1, _ptr(self.tmp), self.n), "harmonic_arnoldi_spectrum")
        q.sub_(self.tmp)


def _orthogonalize(space, q, V, k):
    """_orthogonalize! (krylov.jl:973-978): two Gram-Schmidt passes of q against the first
    k basis vectors; returns |q|.  The passes are classical (one multi-dot and one
    combination each) where the reference's are modified; two passes leave q orthogonal to
    working precision either way."""
    for _ in range(2):
        if k:
            space.subtract(q, V, k, space.dots(V, k, q))
    return space.norm(q)


def _orthonormalize_rows(space, R, ncols):
    """_orthonormalize_columns! (krylov.jl:980-995): two-pass Gram-Schmidt over the vectors,
    dropping those whose norm falls to sqrt(eps) of their initial norm; returns the count
    kept in the leading rows."""
    kept = 0
    threshold = np.sqrt(np.finfo(float).eps)
    for j in range(ncols):
        col = space.copy(R[j])
        initial = space.norm(col)
        for _ in range(2):
            if kept:
                space.subtract(col, R, kept, space.dots(R, kept, col))
        beta = space.norm(col)
        if beta <= threshold * max(initial, np.finfo(float).tiny):
            continue
        R[kept] = col / beta
        kept += 1
    return kept


def _harmonic_arnoldi(space, n, nev, krylovdim, thickdim, maxrestarts, target, initial_vector, initial_subspace,
                      atol, rtol, vectors, rng, require_convergence):
    """Thick-restarted harmonic Arnoldi without a projector (krylov.jl:1378-1551) over the
    vector operations of `space`.  The full space is the projector range, so the basis
    spanning it (k == dim) switches the extraction to ordinary Rayleigh-Ritz."""
    import scipy.linalg as sla
    eps = np.finfo(float).eps
    tiny = np.finfo(float).tiny
    m = min(n, max(krylovdim, nev + 2))
    keep = min(m - 1, max(thickdim, nev))
    breakfactor = np.sqrt(eps)

    def randn():
        return (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)

    V = space.block(m)
    LV = space.block(m)
    nkeep = 0
    if initial_subspace is not None:
        for column in range(min(initial_subspace.shape[1], keep)):
            q = space.upload(initial_subspace[:, column])
            seednorm = space.norm(q)
            beta = _orthogonalize(space, q, V, nkeep)
            if beta <= breakfactor * max(seednorm, seednorm * eps, tiny):
                continue
            V[nkeep] = q / beta
            nkeep += 1
        if nkeep == 0:
            raise PiArgumentError("initial_subspace has no independent component in the selected symmetry sector")
    else:
        q = space.upload(randn() if initial_vector is None else initial_vector)
        nq = space.norm(q)
        if not nq > breakfactor * max(nq, tiny):
            raise PiArgumentError("initial_vector has zero component in the selected symmetry sector")
        V[0] = q / nq
        nkeep = 1
    initial_retained = nkeep
    applications = 0
    history = []
    best = None
    X = None
    requested = complex(target)
    for cycle in range(maxrestarts + 1):
        k = nkeep
        # Images of the retained vectors are recomputed once per restart; the newest image
        # continues the Krylov sequence.
        for j in range(nkeep):
            space.apply(LV[j], V[j])
            applications += 1
        while k < m:
            q = space.copy(LV[k - 1])
            image_norm = space.norm(q)
            beta = _orthogonalize(space, q, V, k)
            if beta <= breakfactor * max(image_norm, tiny):
                q = space.upload(randn())
                seednorm = space.norm(q)
                beta = _orthogonalize(space, q, V, k)
                if beta <= breakfactor * max(seednorm, seednorm * eps, tiny):
                    break
            V[k] = q / beta
            k += 1
            space.apply(LV[k - 1], V[k - 1])
            applications += 1
        exhausted = k == n
        scale = max(max(space.norm(LV[j]) for j in range(k)), tiny)
        # At an exact eigenvalue (the stationary zero mode) the harmonic pencil is singular;
        # a shift of sqrt(eps) times the image scale makes it regular.
        sigma = complex(-max(np.sqrt(eps) * scale, atol)) if requested == 0 else requested
        A = np.empty((k, k), dtype=np.complex128)
        if exhausted:
            for j in range(k):
                A[:, j] = space.dots(V, k, LV[j])
            lam, Y = sla.eig(A)
        else:
            Z = LV[:k] - sigma * V[:k]
            B = np.empty((k, k), dtype=np.complex128)
            for j in range(k):
                A[:, j] = space.dots(Z, k, Z[j])
                B[:, j] = space.dots(Z, k, V[j])
            del Z
            mu, Y = sla.eig(A, B)
            lam = sigma + mu
        finite = np.flatnonzero(np.isfinite(lam.real) & np.isfinite(lam.imag))
        if finite.size == 0:
            raise PiArgumentError("Ritz extraction returned no finite eigenvalues; enlarge krylovdim or change the "
                                  "initial vector")
        order = finite[np.argsort(np.abs(lam[finite] - requested), kind="stable")]
        sel = order[:min(nev, order.size)]
        vals = lam[sel]
        X = space.combine(V, k, Y[:, sel])
        LX = space.combine(LV, k, Y[:, sel])
        residuals = np.empty(sel.size)
        for j in range(sel.size):
            nx = space.norm(X[j])
            X[j] = X[j] / nx
            LX[j] = LX[j] / nx
            residuals[j] = space.norm(LX[j] - complex(vals[j]) * X[j])
        del LX
        tolerance = atol + rtol * scale
        converged = residuals <= tolerance
        extraction = "rayleigh_ritz" if exhausted else "harmonic"
        history.append(dict(cycle=cycle, subspace_dimension=k, locked=int(converged.sum()),
                            maximum_residual=float(residuals.max()), residual_scale=scale,
                            ritz_extraction=extraction, search_space_exhausted=exhausted))
        best = dict(values=vals, residuals=residuals, converged=converged, restarts=cycle, iterations=applications,
                    krylov_dimension=m, retained_dimension=keep, final_retained_dimension=nkeep,
                    initial_retained_dimension=initial_retained, locked=int(converged.sum()), dimension=n,
                    target=requested, harmonic_shift=sigma, algorithm="harmonic", ritz_extraction=extraction,
                    search_space_exhausted=exhausted, residual_scale=scale, residual_tolerance=tolerance,
                    restart_history=list(history), workspace_reused=False, operator_applications=applications)
        if vals.size >= nev and converged.all():
            break
        if exhausted:
            if require_convergence:
                raise PiArgumentError("Rayleigh--Ritz extraction in the complete search space did not converge; "
                                      f"maximum requested Ritz residual={residuals.max()}")
            break
        if cycle == maxrestarts:
            if require_convergence:
                raise PiArgumentError(f"thick-restarted harmonic Arnoldi did not converge in {maxrestarts} restarts; "
                                      f"maximum requested Ritz residual={residuals.max()}")
            break
        retain = [int(idx) for j, idx in enumerate(sel) if converged[j]]
        for idx in order:
            if int(idx) in retain:
                continue
            retain.append(int(idx))
            if len(retain) >= min(keep, order.size):
                break
        R = space.combine(V, k, Y[:, retain])
        nkeep = _orthonormalize_rows(space, R, len(retain))
        if nkeep == 0:
            raise PiArgumentError("harmonic restart lost the retained invariant subspace")
        V[:nkeep] = R[:nkeep]
        del R
    if vectors:
        best["vectors"] = space.download(X)
    return best


def _check_harmonic_arguments(n, nev, krylovdim, thickdim, maxrestarts, target, initial_vector, initial_subspace,
                              projector):
    """Argument checks of harmonic_arnoldi_spectrum (krylov.jl:1378-1412, 53-58); returns
    the resolved krylovdim, thickdim, initial vector and initial subspace."""
    if projector is not None:
        raise PiArgumentError("the CUDA path does not implement symmetry projectors; pass projector=None")
    for name, value in (("nev", nev), ("maxrestarts", maxrestarts)):
        if isinstance(value, bool) or not isinstance(value, (int, np.integer)):
            raise PiArgumentError(f"{name} must be an integer")
    if not (0 < nev <= n):
        raise PiArgumentError("nev must lie between 1 and the operator dimension")
    if maxrestarts < 0:
        raise PiArgumentError("maxrestarts must be nonnegative")
    krylovdim = max(30, 3 * nev + 6) if krylovdim is None else int(krylovdim)
    thickdim = max(nev + 2, 2 * nev) if thickdim is None else int(thickdim)
    if min(n, max(krylovdim, nev + 2)) > _COMBINE_VECTORS:
        raise PiArgumentError(f"the CUDA harmonic Arnoldi process supports krylov dimensions up to {_COMBINE_VECTORS}")
    try:
        t = complex(target)
    except TypeError:
        raise PiArgumentError("Krylov target must be a finite number") from None
    if not (np.isfinite(t.real) and np.isfinite(t.imag)):
        raise PiArgumentError("Krylov target must be a finite number")
    if initial_vector is not None and initial_subspace is not None:
        raise PiArgumentError("initial_vector and initial_subspace are mutually exclusive")
    if initial_vector is not None:
        initial_vector = np.asarray(initial_vector, dtype=np.complex128)
        if initial_vector.shape != (n,):
            raise PiDimensionMismatch("initial_vector has wrong length")
    if initial_subspace is not None:
        initial_subspace = np.asarray(initial_subspace, dtype=np.complex128)
        if initial_subspace.ndim != 2:
            raise PiArgumentError("initial_subspace must be a matrix or nothing")
        if initial_subspace.shape[0] != n:
            raise PiDimensionMismatch("initial_subspace has the wrong row dimension")
        if initial_subspace.shape[1] == 0:
            raise PiArgumentError("initial_subspace cannot have zero columns")
    return krylovdim, thickdim, t, initial_vector, initial_subspace


def harmonic_arnoldi_spectrum(L, nev=6, krylovdim=None, thickdim=None, maxrestarts=20, target=0, initial_vector=None,
                              initial_subspace=None, projector=None, atol=1e-10, rtol=1e-8, vectors=False, rng=None,
                              require_convergence=True):
    """harmonic_arnoldi_spectrum(L; nev=6, krylovdim=max(30, 3nev+6), thickdim=max(nev+2, 2nev),
    maxrestarts=20, target=0, initial_vector, initial_subspace, projector, atol, rtol, vectors,
    rng, require_convergence) (krylov.jl:1378-1551): eigenvalues nearest `target` by
    thick-restarted harmonic Arnoldi.

    Every L x is a device apply of the compiled plan and every projection a device multi-dot;
    the basis, its images and the Ritz vectors stay on the GPU.  The small harmonic pencil
    (Z^H Z, Z^H V) with Z = L V - sigma V, its eigenproblem, the ordering by distance to the
    target and the restart selection run on the host, as the reference hands them to LAPACK.
    Symmetry projectors are not provided (projector must be None).  Returns a dict with the
    reference's result fields; `vectors` adds the (dim, nev) Ritz vectors.

    The projections use pi_mdot_f64_noalloc, whose partial sums live in one array of the
    library per device, so the solves of one process run one at a time (a module lock); a
    caller of that function outside this module must not overlap a solve."""
    compiled = _as_compiled(L)
    n = len(compiled.basis)
    krylovdim, thickdim, t, v0, s0 = _check_harmonic_arguments(n, nev, krylovdim, thickdim, maxrestarts, target,
                                                               initial_vector, initial_subspace, projector)
    rng = rng if rng is not None else np.random.default_rng()
    m = min(n, max(krylovdim, nev + 2))
    with _NOALLOC_LOCK:
        space = _DeviceKrylovSpace(compiled, m)
        return _harmonic_arnoldi(space, n, int(nev), krylovdim, thickdim, int(maxrestarts), t, v0, s0, float(atol),
                                 float(rtol), bool(vectors), rng, bool(require_convergence))


def _ritz_order(values, which):
    """_ritz_order (krylov.jl:893-898): stable order by largest real part, largest modulus or
    smallest modulus."""
    key = {"LR": -values.real, "LM": -np.abs(values), "SM": np.abs(values)}[which]
    return np.argsort(key, kind="stable")


def _arnoldi_expand(space, V, H, first, last):
    """_arnoldi_expand! (krylov.jl:1000-1015) over the vector operations of `space`, 0-based
    columns first..last-1 of the (m+1)-vector block V and the host Hessenberg matrix H: two
    Gram-Schmidt passes per step (classical, as in _orthogonalize), breakdown at
    |h| <= eps * max(|L v_j|, tiny).  Returns the number of basis vectors with images."""
    eps = np.finfo(float).eps
    k = first
    w = space.copy(V[0])
    for j in range(first, last):
        space.apply(w, V[j])
        image_norm = space.norm(w)
        H[:j + 1, j] = 0
        for _ in range(2):
            h = space.dots(V, j + 1, w)
            H[:j + 1, j] += h
            space.subtract(w, V, j + 1, h)
        H[j + 1, j] = space.norm(w)
        k = j + 1
        if abs(H[j + 1, j]) <= eps * max(image_norm, np.finfo(float).tiny):
            break
        V[j + 1] = w / float(H[j + 1, j].real)
    return k


def _iram(space, n, nev, krylovdim, retained_dimension, maxrestarts, which, target, initial_vector, atol, rtol,
          vectors, rng, require_convergence):
    """Implicitly restarted Arnoldi (krylov.jl:1035-1110) over the vector operations of
    `space`: m-step Arnoldi, then per restart exact shifts at the unwanted Ritz values by
    implicit QR steps on the host Hessenberg matrix, the basis rotated and truncated to the
    retained vectors on the device (one combination), and re-expansion."""
    eps = np.finfo(float).eps
    tiny = np.finfo(float).tiny
    m = min(n, max(krylovdim, nev + 1))
    keep = min(m - 1, max(retained_dimension, nev))
    V = space.block(m + 1)
    H = np.zeros((m + 1, m), dtype=np.complex128)
    if initial_vector is None:
        initial_vector = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
    q = space.upload(initial_vector)
    nq = space.norm(q)
    if not nq > 0:
        raise PiArgumentError("initial_vector must be nonzero")
    V[0] = q / nq
    k = _arnoldi_expand(space, V, H, 0, m)
    applications = k
    history = []
    best = None
    order = sel = Y_all = None
    for cycle in range(maxrestarts + 1):
        vals_all, Y_all = np.linalg.eig(H[:k, :k])
        order = np.argsort(np.abs(vals_all - target), kind="stable") if target is not None else \
            _ritz_order(vals_all, which)
        sel = order[:min(nev, k)]
        vals = vals_all[sel]
        residuals = np.abs(H[k, k - 1] * Y_all[-1, sel])
        scale = max(max(np.linalg.norm(H[:k + 1, j]) for j in range(k)), tiny)
        tolerance = atol + rtol * scale
        converged = residuals <= tolerance
        history.append(dict(cycle=cycle, subspace_dimension=k, converged=int(converged.sum()),
                            maximum_residual=float(residuals.max()), residual_scale=scale))
        best = dict(values=vals, residuals=residuals, converged=converged, iterations=applications, restarts=cycle,
                    krylov_dimension=m, retained_dimension=keep, dimension=n, which=which, target=target,
                    algorithm="implicit_qr_arnoldi", residual_scale=scale, residual_tolerance=tolerance,
                    restart_history=list(history), workspace_reused=False, operator_applications=applications)
        if vals.size >= nev and converged.all():
            break
        failure = (f"implicitly restarted Arnoldi did not converge in {maxrestarts} restarts; maximum requested "
                   f"Ritz residual={residuals.max()}")
        if cycle == maxrestarts or k <= keep:
            if require_convergence:
                raise PiArgumentError(failure)
            break
        # Exact unwanted Ritz shifts: by the implicit-Q theorem the first `keep` rotated
        # vectors keep an Arnoldi factorisation.
        Hs = H[:k, :k].copy()
        Qt = np.eye(k, dtype=np.complex128)
        for shift in vals_all[order[keep:]]:
            Q, _ = np.linalg.qr(Hs - shift * np.eye(k))
            Hs = Q.conj().T @ Hs @ Q
            Qt = Qt @ Q
        Vp = space.combine(V, k, Qt[:, :keep + 1])
        # The new residual joins the retained Hessenberg coupling and the old residual.
        q = Vp[keep] * complex(Hs[keep, keep - 1])
        if H[k, k - 1] != 0:
            q = q + complex(H[k, k - 1] * Qt[k - 1, keep - 1]) * V[k]
        beta = _orthogonalize(space, q, Vp, keep)
        if not beta > np.sqrt(eps) * max(scale, tiny):
            if require_convergence:
                raise PiArgumentError(failure)
            break
        V[:keep] = Vp[:keep]
        V[keep] = q / beta
        del Vp
        H[:] = 0
        H[:keep, :keep] = Hs[:keep, :keep]
        H[keep, keep - 1] = beta
        k = _arnoldi_expand(space, V, H, keep, m)
        applications += k - keep
    if vectors:
        best["vectors"] = space.download(space.combine(V, k, Y_all[:, sel]))
    return best


def implicitly_restarted_arnoldi_spectrum(L, nev=6, krylovdim=None, retained_dimension=None, maxrestarts=20,
                                          which="LR", target=None, initial_vector=None, atol=1e-10, rtol=1e-8,
                                          vectors=False, rng=None, require_convergence=True):
    """implicitly_restarted_arnoldi_spectrum(L; nev=6, krylovdim=max(30, 3nev+6),
    retained_dimension=max(nev, min(2nev, krylovdim-1)), maxrestarts=20, which=:LR,
    target=nothing, initial_vector, atol, rtol, vectors, rng, require_convergence)
    (krylov.jl:1035-1110): eigenpairs at the spectral edge (:LR, :LM, :SM) or nearest
    `target`, by Arnoldi with exact-shift implicit QR restarts.

    The basis stays on the GPU (applies through pi_apply_f64, projections through
    pi_mdot_f64_noalloc, the restart rotation and Ritz vectors through pi_combine_f64); the
    Hessenberg matrix, its eigenproblem and the QR shift steps run on the host.  One solve
    at a time per process, as for harmonic_arnoldi_spectrum."""
    compiled = _as_compiled(L)
    n = len(compiled.basis)
    for name, value in (("nev", nev), ("maxrestarts", maxrestarts)):
        if isinstance(value, bool) or not isinstance(value, (int, np.integer)):
            raise PiArgumentError(f"{name} must be an integer")
    if not (0 < nev <= n):
        raise PiArgumentError("nev must lie between 1 and the operator dimension")
    if which not in ("LR", "LM", "SM"):
        raise PiArgumentError("which must be :LR, :LM, or :SM")
    if maxrestarts < 0:
        raise PiArgumentError("maxrestarts must be nonnegative")
    if target is not None:
        t = complex(target)
        if not (np.isfinite(t.real) and np.isfinite(t.imag)):
            raise PiArgumentError("Krylov target must be a finite number")
        target = t
    krylovdim = max(30, 3 * nev + 6) if krylovdim is None else int(krylovdim)
    retained_dimension = (max(nev, min(2 * nev, krylovdim - 1)) if retained_dimension is None
                          else int(retained_dimension))
    m = min(n, max(krylovdim, nev + 1))
    if m + 1 > _COMBINE_VECTORS:
        raise PiArgumentError(f"the CUDA implicitly restarted Arnoldi process supports krylov dimensions up to "
                              f"{_COMBINE_VECTORS - 1}")
    if initial_vector is not None:
        initial_vector = np.asarray(initial_vector, dtype=np.complex128)
        if initial_vector.shape != (n,):
            raise PiDimensionMismatch("initial_vector has wrong length")
    rng = rng if rng is not None else np.random.default_rng()
    with _NOALLOC_LOCK:
        space = _DeviceKrylovSpace(compiled, m + 1)
        return _iram(space, n, int(nev), krylovdim, retained_dimension, int(maxrestarts), which, target,
                     initial_vector, float(atol), float(rtol), bool(vectors), rng, bool(require_convergence))


@dataclass
class SpectrumResult:
    """Typed high-level spectral result (highlevel.jl:215-219)."""
    values: np.ndarray
    vectors: object
    info: dict


_SPECTRUM_TARGETS = ("largest_real", "near_zero", "largest_magnitude")


def liouvillian_spectrum(x, target="largest_real", nev=6, algorithm="auto", vectors=False, return_info=False,
                         **kwargs):
    """liouvillian_spectrum(x; target=:largest_real, nev=6, algorithm=:auto, vectors=false,
    return_info=false, kwargs...) (highlevel.jl:735-835).

    Automatic selection runs harmonic Arnoldi for target=:near_zero and Arnoldi otherwise
    (the reference's dense branch for dim <= 256 materialises the matrix; the CUDA path has
    none).  An explicit Arnoldi or implicitly restarted Arnoldi (:iram) request orders by
    largest real part, largest modulus or, for :near_zero, smallest modulus;
    HarmonicArnoldiAlgorithm fixes nev, krylovdim, thickdim and maxrestarts.  Remaining keywords (krylovdim, atol, rtol, initial_vector, rng,
    require_convergence, and for harmonic Arnoldi thickdim, maxrestarts, initial_subspace)
    go to the solver.  Returns the values, a dict of values and vectors, or with
    return_info=True a SpectrumResult whose info holds the solver's fields."""
    if target not in _SPECTRUM_TARGETS:
        raise PiArgumentError("target must be :largest_real, :near_zero, or :largest_magnitude")
    explicit = isinstance(algorithm, HarmonicArnoldiAlgorithm)
    if not explicit and algorithm not in ("auto", "krylov", "arnoldi", "harmonic", "iram", "implicit_qr"):
        raise PiArgumentError(f"unsupported spectrum algorithm {algorithm!r}; the CUDA path runs Arnoldi and "
                              "harmonic Arnoldi")
    if isinstance(nev, bool):
        raise PiArgumentError("nev must be an integer, not a Bool")
    if nev <= 0:
        raise PiArgumentError("nev must be positive")
    compiled = _as_compiled(x)
    n = len(compiled.basis)
    if explicit:
        if algorithm.nev > n:
            raise PiArgumentError("HarmonicArnoldiAlgorithm.nev exceeds the source dimension")
        requested = algorithm.nev
    else:
        requested = min(n, int(nev))
    opts = dict(nev=requested, krylovdim=max(20, 2 * requested + 4))
    if explicit or algorithm == "harmonic" or (algorithm == "auto" and target == "near_zero"):
        method = "harmonic"
        if explicit:
            opts.update(krylovdim=algorithm.krylovdim, thickdim=algorithm.thickdim, maxrestarts=algorithm.maxrestarts)
        opts.setdefault("rng", np.random.default_rng(0))
        opts.update(kwargs)
        res = harmonic_arnoldi_spectrum(compiled, vectors=vectors, **opts)
    else:
        method = "iram" if algorithm in ("iram", "implicit_qr") else "arnoldi"
        which = {"largest_real": "LR", "largest_magnitude": "LM", "near_zero": "SM"}[target]
        opts.setdefault("rng", np.random.default_rng(0))
        opts.update(kwargs)
        solve = implicitly_restarted_arnoldi_spectrum if method == "iram" else krylov_liouvillian_spectrum
        res = solve(compiled, which=which, vectors=vectors, **opts)
    take = min(requested, len(res["values"]))
    values = res["values"][:take]
    if not vectors and not return_info:
        return values
    vecs = res["vectors"][:, :take] if vectors else None
    info = {k: v for k, v in res.items() if k not in ("values", "vectors")}
    info.update(requested_algorithm=algorithm, selected_algorithm=method)
    if return_info:
        return SpectrumResult(values, vecs, info)
    return dict(values=values, vectors=vecs)


def _liouvillian_gap_info(values, atol, rtol, check_stability):
    """_liouvillian_gap_info (spectra.jl:289-308): the gap -max Re(lambda) over the values
    outside the stationary cluster |lambda| <= atol + rtol * max(max |lambda|, 1)."""
    values = np.asarray(values, dtype=np.complex128)
    scale = max(float(np.abs(values).max(initial=0.0)), 1.0)
    tol = atol + rtol * scale
    stationary = np.abs(values) <= tol
    nullity = int(stationary.sum())
    if nullity == 0:
        raise PiArgumentError(f"no stationary eigenvalue was found within tolerance {tol}")
    abscissa = float(values.real.max())
    stable = abscissa <= tol
    if check_stability and not stable:
        raise PiArgumentError(f"Liouvillian is unstable: spectral abscissa is {abscissa}")
    candidates = values[~stationary]
    if candidates.size == 0:
        gap, mode, frequency = float("inf"), None, float("nan")
    else:
        mode = complex(candidates[int(np.argmax(candidates.real))])
        gap = -mode.real
        if abs(gap) <= tol:
            gap = 0.0
        frequency = mode.imag
    return dict(gap=gap, decay_eigenvalue=mode, oscillation_frequency=frequency, stationary_multiplicity=nullity,
                unique_stationary_mode=nullity == 1, stable=stable, spectral_abscissa=abscissa, tolerance=tol,
                dimension=values.size)


_GAP_METHODS = {"krylov": "arnoldi", "ordinary_arnoldi": "arnoldi", "arnoldi": "arnoldi", "iram": "iram",
                "implicit_qr": "iram"}


def pi_liouvillian_gap(x, atol=1e-12, rtol=1e-10, check_stability=True, return_info=False, symmetry=None,
                       method="krylov", nev=6, krylovdim=None, require_convergence=True, initial_vector=None,
                       rng=None, retained_dimension=None, maxrestarts=20):
    """pi_liouvillian_gap(x; method=:krylov, nev, krylovdim=max(20, 2nev+4), atol, rtol,
    check_stability, return_info, initial_vector, rng) (spectra.jl:262-470, the Arnoldi
    branch :441-466): the asymptotic decay gap -max Re(lambda) outside the stationary
    cluster, from the nev largest-real Ritz values of the device Arnoldi process, or with
    method=:iram of implicitly restarted Arnoldi (retained_dimension, maxrestarts).  The
    count of stationary modes is certified when fewer than nev of the returned values are
    stationary.

    The CUDA path provides these two methods: the reference's default method=:dense
    materialises the matrix, and harmonic selection cannot certify a global gap without a
    symmetry projector (spectra.jl:414-422), which the CUDA path does not provide."""
    if not isinstance(method, str):
        raise PiArgumentError("method must be a Symbol")
    if method == "harmonic":
        raise PiArgumentError("method=:harmonic selects modes nearest zero in modulus and cannot certify the global "
                              "largest-real Liouvillian gap; use method=:krylov")
    if method not in _GAP_METHODS:
        raise PiArgumentError(f"the CUDA path computes Liouvillian gaps with method=:krylov or :iram, not :{method}")
    if symmetry is not None:
        raise PiArgumentError("use method=:harmonic for matrix-free symmetry projection")
    if isinstance(nev, bool) or not isinstance(nev, (int, np.integer)):
        raise PiArgumentError("nev must be an integer")
    krylovdim = max(20, 2 * nev + 4) if krylovdim is None else krylovdim
    if _GAP_METHODS[method] == "iram":
        retained = max(nev, min(2 * nev, krylovdim - 1)) if retained_dimension is None else retained_dimension
        arn = implicitly_restarted_arnoldi_spectrum(x, nev=nev, krylovdim=krylovdim, retained_dimension=retained,
                                                    maxrestarts=maxrestarts, which="LR",
                                                    initial_vector=initial_vector, atol=atol, rtol=rtol, rng=rng,
                                                    require_convergence=require_convergence)
    else:
        arn = krylov_liouvillian_spectrum(x, nev=nev, krylovdim=krylovdim, which="LR", initial_vector=initial_vector,
                                          atol=atol, rtol=rtol, rng=rng, require_convergence=require_convergence)
    info = _liouvillian_gap_info(arn["values"], atol, rtol, check_stability)
    # A partial spectrum certifies the returned slow mode, but not that every stationary
    # mode was counted when all nev returned values are stationary.
    complete = info["stationary_multiplicity"] < nev
    info.update(dimension=arn["dimension"], symmetry_used=False, symmetry_name=None, symmetry_sectors=None,
                symmetry_residual=None, method=_GAP_METHODS[method], ritz_residuals=arn["residuals"],
                stationary_multiplicity_certified=complete, krylov_dimension=arn["krylov_dimension"],
                scope="global", selection="largest_real", gap_certified=complete, stability_certified=complete)
    return info if return_info else info["gap"]


def apply_element_major_(y, compiled: CompiledPIModel, x, coords="population"):
    """Batched FP32 apply on an element-major batch: y[e, c] = (L x[:, c])[e].

    x, y: complex64 CUDA tensors of shape (dim, ncols) with unit column stride and an even
    row stride (ncols even) -- the batch kept side by side per PI coordinate.  Needs a plan
    with compiled.info["batched_kernel"] == 2 (real one-body qubit operators)."""
    torch = _torch()
    lib = _lib.load()
    n = len(compiled.basis)
    if x.shape != y.shape or x.dim() != 2 or x.shape[0] != n or not x.is_cuda or not y.is_cuda:
        raise PiDimensionMismatch("element-major batches have shape (dim, ncols) on the GPU")
    if x.dtype != torch.complex64 or y.dtype != torch.complex64:
        raise PiArgumentError("element-major apply needs complex64 tensors")
    if x.stride(1) != 1 or y.stride(1) != 1 or x.stride(0) != y.stride(0):
        raise PiArgumentError("element-major batches need unit column stride and equal row strides")
    cc = _lib.PI_COORDS_POPULATION if coords == "population" else _lib.PI_COORDS_REFERENCE
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.pi_apply_f32_em(compiled.handle, _ptr(y), _ptr(x), x.shape[1], x.stride(0), cc, stream),
               "apply! (element-major batch)")
    return y


EM_KERNELS = {0: "tma", 1: "plain"}


def element_major_tuning(compiled: CompiledPIModel, ncols, coords="population"):
    """The element-major kernel in use for a batch width and coordinate system, as chosen by
    the autotuner on the first apply_element_major_ call (or pinned with
    select_element_major_kernel): {"kernel": "tma" | "plain", "rows": tile rows, "ms": timed
    duration of one apply (0 when pinned)}."""
    lib = _lib.load()
    cc = _lib.PI_COORDS_POPULATION if coords == "population" else _lib.PI_COORDS_REFERENCE
    kind, rows, ms = C.c_int(), C.c_int(), C.c_double()
    _lib.check(lib.pi_apply_f32_em_tuning(compiled.handle, int(ncols), cc, C.byref(kind), C.byref(rows),
                                          C.byref(ms)), "element-major tuning")
    return {"kernel": EM_KERNELS[kind.value], "rows": rows.value, "ms": ms.value}


def select_element_major_kernel(compiled: CompiledPIModel, ncols, kernel="tma", rows=32, coords="population"):
    """Pins the element-major kernel for a batch width and coordinate system instead of
    autotuning it: kernel "tma" (tile rows 16, 32 or, without pumping terms, 64) or "plain"."""
    kinds = {v: k for k, v in EM_KERNELS.items()}
    if kernel not in kinds:
        raise PiArgumentError(f"element-major kernel must be one of {sorted(kinds)}, got {kernel!r}")
    if coords not in ("population", "reference"):
        raise PiArgumentError(f"coords must be 'population' or 'reference', got {coords!r}")
    lib = _lib.load()
    cc = _lib.PI_COORDS_POPULATION if coords == "population" else _lib.PI_COORDS_REFERENCE
    _lib.check(lib.pi_apply_f32_em_select(compiled.handle, int(ncols), cc, kinds[kernel], int(rows)),
               "element-major kernel choice")


def mul(compiled: CompiledPIModel, x):
    """L * x for a host vector (allocating wrapper of apply!)."""
    y = np.empty_like(np.asarray(x, dtype=np.complex128))
    return apply_(y, compiled, np.asarray(x, dtype=np.complex128))


# ---------------------------------------------------------------------------------------
# Algorithms (highlevel.jl:32-125)
# ---------------------------------------------------------------------------------------

@dataclass(frozen=True)
class GMRESAlgorithm:
    """Restarted matrix-free GMRES (highlevel.jl:32-41); precision 'fp64' (the reference's
    method) or 'mixed' (FP32 inner applies with FP64 refinement)."""
    krylovdim: int = 30
    maxiter: int = 500
    preconditioner: object = None
    precision: str = "fp64"
    drive_preconditioner: object = None

    def __post_init__(self):
        if isinstance(self.krylovdim, bool) or self.krylovdim < 1:
            raise PiArgumentError("krylovdim must be at least 1")
        if isinstance(self.maxiter, bool) or self.maxiter < 1:
            raise PiArgumentError("maxiter must be at least 1")
        if self.preconditioner is not None and not isinstance(self.preconditioner, LevelPreconditioner):
            raise PiArgumentError("the CUDA backend takes a LevelPreconditioner (level_preconditioner(compiled)) "
                                  "or a DrivePreconditioner (drive_preconditioner(compiled)) as the GMRES "
                                  "preconditioner")
        if self.drive_preconditioner is not None:
            if not isinstance(self.drive_preconditioner, DrivePreconditioner):
                raise PiArgumentError("drive_preconditioner must be a DrivePreconditioner")
            if self.preconditioner is None or isinstance(self.preconditioner, DrivePreconditioner):
                raise PiArgumentError("drive_preconditioner goes beside a level preconditioner "
                                      "(preconditioner=level_preconditioner(compiled))")
        if self.precision not in ("fp64", "mixed"):
            raise PiArgumentError("precision must be 'fp64' or 'mixed'")


@dataclass(frozen=True)
class HarmonicArnoldiAlgorithm:
    """Thick-restarted harmonic Arnoldi parameters for modes near zero (highlevel.jl:126-150):
    krylovdim defaults to max(30, 3nev+6) and thickdim to max(nev+2, 2nev)."""
    nev: int = 6
    krylovdim: int = None
    thickdim: int = None
    maxrestarts: int = 20

    def __post_init__(self):
        for name, minimum in (("nev", 1), ("krylovdim", 1), ("thickdim", 1), ("maxrestarts", 0)):
            value = getattr(self, name)
            if value is None and name in ("krylovdim", "thickdim"):
                continue
            if isinstance(value, bool):
                raise PiArgumentError(f"{name} must be an integer, not a Bool")
            if not isinstance(value, (int, np.integer)):
                raise PiArgumentError(f"{name} must be an integer or nothing")
            if value < minimum:
                raise PiArgumentError(f"{name} must be at least {minimum}")
        if self.krylovdim is None:
            object.__setattr__(self, "krylovdim", max(30, 3 * self.nev + 6))
        if self.thickdim is None:
            object.__setattr__(self, "thickdim", max(self.nev + 2, 2 * self.nev))


@dataclass(frozen=True)
class ExpvAlgorithm:
    """Adaptive restarted-Arnoldi exponential action (highlevel.jl:81-125)."""
    krylovdim: int = 30
    atol: float = 1e-10
    rtol: float = 1e-8
    initial_step: float | None = None
    minimum_step: float | None = None
    maximum_step: float | None = None
    max_steps: int = 10_000
    safety: float = 0.9
    precision: str = "fp64"

    def __post_init__(self):
        if not (np.isfinite(self.atol) and np.isfinite(self.rtol) and self.atol >= 0 and self.rtol >= 0):
            raise PiArgumentError("atol and rtol must be finite nonnegative real numbers")
        if not (0 < self.safety < 1):
            raise PiArgumentError("safety must lie strictly between zero and one")
        for name, allow_zero in (("initial_step", False), ("minimum_step", True), ("maximum_step", False)):
            v = getattr(self, name)
            if v is not None and (not np.isfinite(v) or (v < 0 if allow_zero else v <= 0)):
                raise PiArgumentError(f"{name} must be nothing or a finite {'nonnegative' if allow_zero else 'positive'} real number")
        if self.minimum_step is not None and self.maximum_step is not None and self.minimum_step > self.maximum_step:
            raise PiArgumentError("minimum_step must not exceed maximum_step")
        if self.minimum_step is not None and self.initial_step is not None and self.initial_step < self.minimum_step:
            raise PiArgumentError("initial_step must not be smaller than minimum_step")
        if self.precision not in ("fp64", "mixed"):
            raise PiArgumentError("precision must be 'fp64' or 'mixed'")

    def opts(self):
        o = _lib.pi_expv_opts_t()
        _lib.load().pi_expv_default_opts(C.byref(o))
        o.krylovdim = self.krylovdim
        o.atol = self.atol
        o.rtol = self.rtol
        o.initial_step = self.initial_step or 0.0
        o.minimum_step = self.minimum_step or 0.0
        o.maximum_step = self.maximum_step or 0.0
        o.max_steps = self.max_steps
        o.safety = self.safety
        o.precision = _lib.PI_FP32 if self.precision == "mixed" else _lib.PI_FP64
        return o


@dataclass
class SteadyStateResult:
    """SteadyStateResult: state plus solver information (krylov.jl:876-889)."""
    state: PIState
    info: dict
    algorithm: GMRESAlgorithm


@dataclass
class DynamicsResult:
    t: list
    states: list
    algorithm: str = "expv"

    def __len__(self):
        return len(self.t)

    def __getitem__(self, i):
        return self.states[i]


@dataclass
class DynamicsStreamResult:
    t: list
    states: list | None
    values: dict = field(default_factory=dict)
    algorithm: str = "expv"


def _as_compiled(x) -> CompiledPIModel:
    if isinstance(x, CompiledPIModel):
        return x
    if isinstance(x, PIModel):
        return compile(x, backend="cuda")
    raise PiArgumentError("expected a PIModel or a CompiledPIModel")


_COORDS = {"reference": _lib.PI_COORDS_REFERENCE, "population": _lib.PI_COORDS_POPULATION}


class LevelPreconditioner:
    """Left preconditioner of the trace-fixed steady-state GMRES (pi_precond_create), the CUDA
    path's counterpart of schur_sector_preconditioner (krylov.jl:594-700).

    It inverts exactly, by level sweeps on the GPU, M = L0/s + v t', where L0 keeps every term
    of L that preserves the charge m - m' (the Jz-covariant dissipators and the diagonal of
    the Hamiltonian) and leaves out the drive (Jx, Jy), which changes it.  `coords` fixes the
    coordinates of the solves it serves: "population" (z = sqrt(f) x, whose norms weigh
    populations; FP32 sweeps) or "reference" (FP64 sweeps).  The operator scale s is
    estimated from three random probes in those coordinates unless given, and the solve uses
    it, as the reference's prepared preconditioner does."""

    def __init__(self, compiled, coords="population", regularization=0.0, operator_scale=None):
        if coords not in _COORDS:
            raise PiArgumentError("coords must be 'reference' or 'population'")
        self.compiled = _as_compiled(compiled)
        self.coords = coords
        handle = C.c_void_p()
        _lib.check(_lib.load().pi_precond_create(self.compiled.handle, _COORDS[coords], float(regularization),
                                                 float(operator_scale) if operator_scale else 0.0,
                                                 C.byref(handle)), "level_preconditioner")
        self._handle = handle
        info = _lib.pi_precond_info_t()
        _lib.check(_lib.load().pi_precond_info(handle, C.byref(info)), "pi_precond_info")
        self.info = {f: getattr(info, f) for f, _ in info._fields_}

    @property
    def handle(self):
        if self._handle is None:
            raise _lib.PiError("the preconditioner has been closed")
        return self._handle

    @property
    def operator_scale(self):
        return self.info["operator_scale"]

    def apply(self, z, r):
        """z = M^-1 r for complex128 CUDA tensors in the preconditioner's coordinates
        (the ldiv! of krylov.jl:202-209), on torch's current stream."""
        torch = _torch()
        n = len(self.compiled.basis)
        if r.shape != (n,) or z.shape != (n,) or r.dtype != torch.complex128 or z.dtype != torch.complex128:
            raise PiDimensionMismatch("preconditioner vector has wrong length or type")
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.check(_lib.load().pi_precond_apply(self.handle, _ptr(z), _ptr(r), stream), "ldiv!")
        return z

    def close(self):
        if getattr(self, "_handle", None) is not None:
            _lib.load().pi_precond_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def level_preconditioner(compiled, coords="population", regularization=0.0, operator_scale=None):
    """Builds a LevelPreconditioner for a compiled model (see its docstring)."""
    return LevelPreconditioner(compiled, coords=coords, regularization=regularization, operator_scale=operator_scale)


class DrivePreconditioner(LevelPreconditioner):
    """The drive part of the trace-fixed steady-state operator (pi_precond_create_drive): per
    Schur sector the commutator with the sector's Hamiltonian block H_s and the loss each of its
    eigenmodes sees, solved exactly in the orthogonal eigenbasis of H_s, plus the trace border by
    Sherman-Morrison, in the precision of the vectors it maps.  It carries the drive (Jx, Jy), which the level sweep
    leaves out, and leaves out the loss variation along a sector and the gains, which the level
    sweep carries.  As the GMRES preconditioner it is applied twice per step; beside a level
    preconditioner (GMRESAlgorithm(preconditioner=level, drive_preconditioner=drive)) the solve
    moves from the level sweep to it, and then to both in turn, when a restart cycle makes
    little progress.  No counterpart in the reference, whose Schur-sector preconditioner
    LU-factors every sector block densely (krylov.jl:594-700)."""

    def __init__(self, compiled, coords="population", operator_scale=None):
        if coords not in _COORDS:
            raise PiArgumentError("coords must be 'reference' or 'population'")
        self.compiled = _as_compiled(compiled)
        self.coords = coords
        handle = C.c_void_p()
        _lib.check(_lib.load().pi_precond_create_drive(self.compiled.handle, _COORDS[coords],
                                                       float(operator_scale) if operator_scale else 0.0,
                                                       C.byref(handle)), "drive_preconditioner")
        self._handle = handle
        info = _lib.pi_precond_info_t()
        _lib.check(_lib.load().pi_precond_info(handle, C.byref(info)), "pi_precond_info")
        self.info = {f: getattr(info, f) for f, _ in info._fields_}


def drive_preconditioner(compiled, coords="population", operator_scale=None):
    """Builds a DrivePreconditioner for a compiled model (see its docstring); pass the level
    preconditioner's operator_scale to use both in one solve."""
    return DrivePreconditioner(compiled, coords=coords, operator_scale=operator_scale)


def drive_preconditioner_tables(model):
    """Host-only export of the drive preconditioner's eigen tables (pi_precond_drive_export)
    for a PIModel: per sector the eigenvector matrix U (n x n, column i for h[i]), the
    eigenvalues h of the sector Hamiltonian block, c = -2 x the sector's mean loss and q, the
    loss each eigenmode sees (floored at -c / 4)."""
    lib = _lib.load()
    kinds, ops, rates, hbar, ks = _term_arrays(model)
    counts = np.zeros(3, dtype=np.int64)
    args = (model.basis.N, model.basis.d, len(ks), _lib.iptr(ks), len(model.terms), _lib.iptr(kinds),
            _lib.dptr(ops), _lib.dptr(rates), _lib.dptr(hbar), _lib.llptr(counts))
    _lib.check(lib.pi_precond_drive_export(*args, None, None, None, None), "pi_precond_drive_export")
    S, nu, nh = (int(v) for v in counts)
    U, h, c, q = np.zeros(nu), np.zeros(nh), np.zeros(S), np.zeros(nh)
    _lib.check(lib.pi_precond_drive_export(*args, _lib.dptr(U), _lib.dptr(h), _lib.dptr(c), _lib.dptr(q)),
               "pi_precond_drive_export")
    out, uo, ho = [], 0, 0
    for n in model.basis.dims:
        out.append(dict(U=U[uo:uo + n * n].reshape((n, n), order="F"), h=h[ho:ho + n], q=q[ho:ho + n]))
        uo += n * n
        ho += n
    for d, cs in zip(out, c):
        d["c"] = float(cs)
    return out


def level_preconditioner_tables(model, coords="population", regularization=0.0, operator_scale=1.0):
    """Host-only export of the preconditioner tables (pi_precond_export) for a PIModel: a
    dict of numpy arrays; no device needed."""
    lib = _lib.load()
    kinds, ops, rates, hbar, ks = _term_arrays(model)
    counts = np.zeros(4, dtype=np.int64)
    args = (model.basis.N, model.basis.d, len(ks), _lib.iptr(ks), len(model.terms), _lib.iptr(kinds),
            _lib.dptr(ops), _lib.dptr(rates), _lib.dptr(hbar), _COORDS[coords], float(regularization),
            float(operator_scale), _lib.llptr(counts))
    _lib.check(lib.pi_precond_export(*args, None), "pi_precond_export")
    nc, nl, ne, n0 = (int(v) for v in counts)
    out = dict(chain_lev=np.zeros(nc + 1, np.int32), lev_ent=np.zeros(nl + 1, np.int32), elem=np.zeros(ne, np.int32),
               W=np.zeros(ne, np.complex128), A=np.zeros(ne, np.complex128), C=np.zeros(ne, np.complex128),
               gsrc=np.zeros(ne, np.int32), G=np.zeros(3 * ne, np.complex128), t0=np.zeros(n0), v0=np.zeros(n0),
               w0=np.zeros(n0, np.complex128))
    t = _lib.pi_precond_tables_t()
    for name in ("chain_lev", "lev_ent", "elem", "gsrc"):
        setattr(t, name, out[name].ctypes.data_as(C.POINTER(C.c_int)))
    for name in ("W", "A", "C", "G", "t0", "v0", "w0"):
        setattr(t, name, out[name].ctypes.data_as(C.POINTER(C.c_double)))
    _lib.check(lib.pi_precond_export(*args, C.byref(t)), "pi_precond_export")
    meta = list(t.meta)
    out.update(chain0=meta[0], chain0_ent=meta[1], mode=meta[2], free_ent=meta[3], direction=meta[4],
               max_level=meta[5], sm_coef=complex(t.sm_coef[0], t.sm_coef[1]), operator_scale=float(operator_scale))
    return out


def stationary_state(x, algorithm=None, return_info=False, atol=1e-10, rtol=1e-8, operator_scale=None,
                     initial_state=None, max_refinements=200, coords="reference"):
    """stationary_state(x; algorithm=GMRESAlgorithm(...)) (highlevel.jl:321-371) on the GPU.

    coords="population" runs the solve on z = sqrt(f) x, where the residual and trace tests
    weigh populations (in reference coordinates the entries of high-multiplicity sectors
    vanish from every norm at large N); the state is returned in reference coordinates
    either way.  A LevelPreconditioner in the algorithm fixes the coordinates to its own."""
    torch = _torch()
    algorithm = algorithm or GMRESAlgorithm()
    if isinstance(algorithm, str):
        if algorithm not in ("gmres", "auto"):
            raise PiArgumentError("the CUDA backend solves stationary states with GMRES")
        algorithm = GMRESAlgorithm()
    compiled = _as_compiled(x)
    n = len(compiled.basis)
    P = algorithm.preconditioner
    if P is not None:
        coords = P.coords
        if P.compiled is not compiled:
            raise PiArgumentError("the preconditioner was built for another compiled model")
    if coords not in _COORDS:
        raise PiArgumentError("coords must be 'reference' or 'population'")
    o = _lib.pi_gmres_opts_t()
    lib = _lib.load()
    lib.pi_gmres_default_opts(C.byref(o))
    o.krylovdim = algorithm.krylovdim
    o.maxiter = algorithm.maxiter
    o.atol, o.rtol = atol, rtol
    o.operator_scale = float(operator_scale) if operator_scale else 0.0
    o.precision = _lib.PI_FP32 if algorithm.precision == "mixed" else _lib.PI_FP64
    o.max_refinements = max_refinements
    o.coords = _COORDS[coords]
    o.preconditioner = P.handle if P is not None else None
    Pd = algorithm.drive_preconditioner
    if Pd is not None:
        if Pd.compiled is not compiled or Pd.coords != coords:
            raise PiArgumentError("the drive preconditioner was built for another compiled model or coordinates")
        o.drive_preconditioner = Pd.handle
    xd = torch.zeros(n, dtype=torch.complex128, device="cuda")
    if initial_state is not None:
        init = initial_state.data if isinstance(initial_state, PIState) else np.asarray(initial_state)
        if init.shape != (n,):
            raise PiDimensionMismatch("initial_state has wrong length")
        xd.copy_(torch.from_numpy(np.ascontiguousarray(init, dtype=np.complex128)))
        o.use_initial = 1
    torch.cuda.synchronize()
    info = _lib.pi_gmres_info_t()
    _lib.check(lib.pi_steady_state(compiled.handle, _ptr(xd), C.byref(o), C.byref(info)),
               "stationary_state")
    rho = PIState(compiled.basis, xd.cpu().numpy())
    if not return_info:
        return rho
    d = {f: getattr(info, f) for f, _ in info._fields_}
    d.update(method="krylov", krylov_dimension=algorithm.krylovdim, precision=algorithm.precision,
             state=rho.data, coords=coords, preconditioned=P is not None,
             preconditioner=type(P).__name__ if P is not None else None,
             drive_preconditioner=Pd is not None)
    return SteadyStateResult(rho, d, algorithm)


def steady_state(x, method="krylov", **kwargs):
    """Low-level steady_state(compiled; method=:krylov) (liouvillian.jl:4752-4761)."""
    if method not in ("krylov", "gmres"):
        raise PiArgumentError("the CUDA backend supports method=:krylov")
    alg = GMRESAlgorithm(krylovdim=kwargs.pop("krylovdim", 30), maxiter=kwargs.pop("maxiter", 500),
                         precision=kwargs.pop("precision", "fp64"))
    return stationary_state(x, algorithm=alg, **kwargs).data


def krylov_expv(compiled, b, t, algorithm: ExpvAlgorithm | None = None, return_info=False):
    """krylov_expv(A, b, t; ...) (krylov_extensions.jl:1578-1585) on the GPU."""
    torch = _torch()
    algorithm = algorithm or ExpvAlgorithm()
    compiled = _as_compiled(compiled)
    lib = _lib.load()
    data = b.data if isinstance(b, PIState) else np.asarray(b)
    xd = torch.from_numpy(np.ascontiguousarray(data, dtype=np.complex128)).cuda()
    torch.cuda.synchronize()
    info = _lib.pi_expv_info_t()
    o = algorithm.opts()
    _lib.check(lib.pi_expv(compiled.handle, _ptr(xd), float(t), C.byref(o), C.byref(info)), "krylov_expv")
    out = xd.cpu().numpy()
    if return_info:
        return out, {f: getattr(info, f) for f, _ in info._fields_}
    return out


def saved_times(tspan, saveat):
    """Saved-time grid (highlevel.jl:434-465)."""
    t0, t1 = float(tspan[0]), float(tspan[1])
    if t1 < t0:
        raise PiArgumentError("tspan must be ordered")
    if saveat is None:
        return [t0, t1]
    if np.isscalar(saveat):
        step = float(saveat)
        if not (np.isfinite(step) and step > 0):
            raise PiArgumentError("saveat must be finite and positive")
        count = int(np.floor((t1 - t0) / step * (1 + 1e-15))) + 1
        ts = [t0 + i * step for i in range(count) if t0 + i * step <= t1]
        if not ts or ts[-1] < t1:
            ts.append(t1)
        return ts
    ts = [float(v) for v in saveat]
    if not ts:
        raise PiArgumentError("saveat cannot be empty")
    if ts[0] != t0 or ts[-1] != t1:
        raise PiArgumentError("explicit saveat times must include both endpoints of tspan")
    if any(b < a for a, b in zip(ts, ts[1:])):
        raise PiArgumentError("saveat times must be nondecreasing")
    return ts


def _observable_data(basis, obs):
    if isinstance(obs, (PIOperator, PIState)):
        return obs.data
    a = np.asarray(obs, dtype=np.complex128)
    if a.shape == (basis.d, basis.d):
        return collective_operator(basis, a).data  # a local matrix denotes its collective sum
    if a.shape == (len(basis),):
        return a
    raise PiDimensionMismatch("observable must be a PIOperator, a local d x d matrix or a PI vector")


_DYNAMICS_ALGORITHM_NAMES = ("auto", "rk4", "expv", "krylov_expv", "adaptive_or_rk4", "dynamics")


def _dynamics_algorithm(algorithm):
    """(name, ExpvAlgorithm or None) for a dynamics algorithm: symbols canonicalised as in
    solver_algorithms.jl:38-44 and highlevel.jl:285-298; :auto selects RK4 for a matrix-free
    source (highlevel.jl:1482-1523)."""
    if isinstance(algorithm, ExpvAlgorithm):
        return "expv", algorithm
    if isinstance(algorithm, str):
        name = {"adaptive_or_rk4": "rk4", "dynamics": "rk4", "krylov_expv": "expv"}.get(algorithm, algorithm)
        if name not in ("auto", "rk4", "expv"):
            raise PiArgumentError(f"unsupported dynamics algorithm {algorithm}; choose one of "
                                  f"{_DYNAMICS_ALGORITHM_NAMES}")
        if name == "auto":
            name = "rk4"
        return name, (ExpvAlgorithm() if name == "expv" else None)
    raise PiArgumentError("unsupported dynamics algorithm; use a dynamics algorithm name or ExpvAlgorithm()")


def _rk4_opts(steps, precision):
    if int(steps) <= 0:
        raise PiArgumentError("steps must be positive")
    if precision not in ("fp64", "mixed"):
        raise PiArgumentError("precision must be 'fp64' or 'mixed'")
    return _lib.pi_rk4_opts_t(int(steps), _lib.PI_FP32 if precision == "mixed" else _lib.PI_FP64)


def evolve_(dest, x, src, tspan, steps=256, precision="fp64"):
    """evolve!(dest, L, src, tspan; steps=256) (evolution.jl:75-118): fixed-step RK4 of
    h = (t1 - t0) / steps on the GPU.

    dest, src: complex128 CUDA tensors of length dim (device-resident; dest may be src but
    must not partially overlap it) or PIStates (host data, copied in and out).
    precision="mixed" applies the operator in FP32 population coordinates with an FP64 state
    and stage sum.  Returns dest.
    """
    torch = _torch()
    compiled = _as_compiled(x)
    n = len(compiled.basis)
    t0, t1 = float(tspan[0]), float(tspan[1])
    o = _rk4_opts(steps, precision)
    info = _lib.pi_rk4_info_t()
    lib = _lib.load()
    if isinstance(dest, PIState) or isinstance(src, PIState):
        if not (isinstance(dest, PIState) and isinstance(src, PIState)):
            raise PiArgumentError("dest and src must both be PIStates or both device tensors")
        if dest.basis.N != compiled.basis.N or src.basis.N != compiled.basis.N:
            raise PiArgumentError("source and destination use incompatible PI bases")
        xd = torch.from_numpy(np.ascontiguousarray(src.data, dtype=np.complex128)).cuda()
        torch.cuda.synchronize()
        _lib.check(lib.pi_evolve(compiled.handle, _ptr(xd), _ptr(xd), t0, t1, C.byref(o), C.byref(info)), "evolve!")
        dest.data[...] = xd.cpu().numpy()
        return dest
    if dest.shape != (n,) or src.shape != (n,) or not dest.is_cuda or not src.is_cuda:
        raise PiDimensionMismatch("source and destination dimensions differ from the Liouvillian's")
    if dest.dtype != torch.complex128 or src.dtype != torch.complex128:
        raise PiArgumentError("evolve! needs complex128 device vectors")
    if not (dest.is_contiguous() and src.is_contiguous()):
        raise PiArgumentError("device vectors must be contiguous")
    torch.cuda.synchronize()
    _lib.check(lib.pi_evolve(compiled.handle, _ptr(dest), _ptr(src), t0, t1, C.byref(o), C.byref(info)), "evolve!")
    return dest


def time_evolve(x, rho: PIState, tspan, steps=256, precision="fp64"):
    """time_evolve(L, rho, tspan; steps) (evolution.jl:131-134): a new PIState, rho unchanged."""
    out = PIState(rho.basis, np.array(rho.data, dtype=np.complex128))
    return evolve_(out, x, PIState(rho.basis, rho.data), tspan, steps=steps, precision=precision)


def solve_dynamics(x, rho0: PIState, tspan, algorithm="auto", saveat=None, observables=None,
                   save_states=True, parameters=None, steps_per_interval=64, precision="fp64"):
    """solve_dynamics(x, rho0, tspan; algorithm=:auto, saveat, steps_per_interval=64,
    observables, save_states) (highlevel.jl:559-733).

    algorithm :auto / :rk4 (the reference's default: fixed-step RK4 with steps_per_interval
    steps per saved interval) or :expv / ExpvAlgorithm(...) (adaptive Krylov exponential).
    precision="mixed" selects FP32 applies with an FP64 state for RK4 (ExpvAlgorithm carries
    its own precision).
    """
    torch = _torch()
    if int(steps_per_interval) <= 0:
        raise PiArgumentError("steps_per_interval must be positive")
    name, algorithm = _dynamics_algorithm(algorithm)
    if parameters is not None:
        raise PiArgumentError("the CUDA plan is one autonomous generator: parameters must be nothing")
    compiled = _as_compiled(x)
    if rho0.basis.N != compiled.basis.N or rho0.basis.sectors != compiled.basis.sectors:
        raise PiArgumentError("Liouvillian source and initial state use incompatible PI bases")
    if observables is None and not save_states:
        raise PiArgumentError("save_states=false requires at least one observable")
    ts = saved_times(tspan, saveat)
    lib = _lib.load()
    xd = torch.from_numpy(np.ascontiguousarray(rho0.data)).cuda()
    names = []
    obs_dev = None
    if observables:
        items = observables.items() if isinstance(observables, dict) else (
            [("observable", observables)] if not isinstance(observables, (list, tuple)) else observables)
        datas = []
        for k, v in items:
            names.append(k)
            datas.append(_observable_data(compiled.basis, v))
        obs_dev = torch.from_numpy(np.ascontiguousarray(np.stack(datas))).cuda()
    nobs = len(names)
    if name == "rk4":
        o = _rk4_opts(steps_per_interval, precision)
        info = _lib.pi_rk4_info_t()
    else:
        o = algorithm.opts()
        info = _lib.pi_expv_info_t()
    torch.cuda.synchronize()
    if not save_states:
        times = np.array(ts, dtype=np.float64)
        vals = np.zeros((len(ts), max(nobs, 1), 2), dtype=np.float64)
        fn = lib.pi_solve_dynamics_rk4 if name == "rk4" else lib.pi_solve_dynamics
        _lib.check(fn(compiled.handle, _ptr(xd), len(ts), _lib.dptr(times), nobs,
                      _ptr(obs_dev) if obs_dev is not None else None, _lib.dptr(vals), C.byref(o), C.byref(info)),
                   "solve_dynamics")
        values = {k: vals[:, i, 0] + 1j * vals[:, i, 1] for i, k in enumerate(names)}
        return DynamicsStreamResult(ts, None, values, algorithm=name)
    states = [rho0.copy()]
    series = {k: [] for k in names}

    def record(state_dev):
        # dot(op.data, rho.data) on the device (highlevel.jl:672-677)
        out = np.zeros(2, dtype=np.float64)
        for i, k in enumerate(names):
            _lib.check(lib.pi_dot_f64(compiled.handle, _ptr(obs_dev[i]), _ptr(state_dev), _lib.dptr(out)),
                       "observable")
            series[k].append(complex(out[0], out[1]))

    record(xd)
    for i in range(1, len(ts)):
        dt = ts[i] - ts[i - 1]
        if dt != 0:
            torch.cuda.synchronize()
            if name == "rk4":
                _lib.check(lib.pi_evolve(compiled.handle, _ptr(xd), _ptr(xd), ts[i - 1], ts[i], C.byref(o),
                                         C.byref(info)), "solve_dynamics")
            else:
                _lib.check(lib.pi_expv(compiled.handle, _ptr(xd), dt, C.byref(o), C.byref(info)), "solve_dynamics")
        states.append(PIState(compiled.basis, xd.cpu().numpy()))
        record(xd)
    if nobs:
        return DynamicsStreamResult(ts, states, {k: np.array(v) for k, v in series.items()}, algorithm=name)
    return DynamicsResult(ts, states, algorithm=name)


# ---------------------------------------------------------------------------------------
# Batched solves: many plans advance together in one engine (pi_*_batch).  The reference
# runs such workloads as a loop over parameter points (scans.jl:1457 parameter_scan); each
# batched result equals the single-instance result to solver tolerance.
# ---------------------------------------------------------------------------------------

def _device_states(compiled_list, states):
    torch = _torch()
    out = []
    for c, s in zip(compiled_list, states):
        data = s.data if isinstance(s, PIState) else np.asarray(s)
        if data.shape != (len(c.basis),):
            raise PiDimensionMismatch("batch state has the wrong length for its model")
        out.append(torch.from_numpy(np.ascontiguousarray(data, dtype=np.complex128)).cuda())
    return out


def _ptr_array(ptrs):
    arr = (C.c_void_p * len(ptrs))()
    for i, p in enumerate(ptrs):
        arr[i] = p
    return arr


def krylov_expv_batch(models, states, t, algorithm: ExpvAlgorithm | None = None, return_info=False):
    """exp(t_i L_i) b_i for every instance in one batched engine run."""
    torch = _torch()
    algorithm = algorithm or ExpvAlgorithm()
    compiled = [_as_compiled(m) for m in models]
    if len(states) != len(compiled):
        raise PiDimensionMismatch("one state per model is required")
    ts = np.broadcast_to(np.asarray(t, dtype=np.float64), (len(compiled),)).copy()
    xs = _device_states(compiled, states)
    torch.cuda.synchronize()
    infos = (_lib.pi_expv_info_t * len(compiled))()
    o = algorithm.opts()
    lib = _lib.load()
    _lib.check(lib.pi_expv_batch(len(compiled), _ptr_array([c.handle for c in compiled]),
                                 _ptr_array([_ptr(x) for x in xs]), _lib.dptr(ts), C.byref(o), infos),
               "krylov_expv_batch")
    out = [x.cpu().numpy() for x in xs]
    if return_info:
        return out, [{f: getattr(i, f) for f, _ in i._fields_} for i in infos]
    return out


def solve_dynamics_batch(models, rho0s, tspans, algorithm: ExpvAlgorithm | None = None, saveat=None,
                         observables=None, return_info=False):
    """solve_dynamics(...; save_states=false) for many models in one batched engine run.

    tspans and saveat may be one value for all instances or one per instance (a list of n
    tspans; a list of n saveat grids, each None or a sequence).  observables is one dict
    name -> operator for all instances, or a list of n such dicts (e.g. prebuilt PI
    vectors per instance).  Returns one
    DynamicsStreamResult per instance (values per observable name) plus the final states.
    """
    torch = _torch()
    algorithm = algorithm or ExpvAlgorithm()
    compiled = [_as_compiled(m) for m in models]
    n = len(compiled)
    if len(rho0s) != n:
        raise PiDimensionMismatch("one initial state per model is required")
    if isinstance(tspans, tuple) and len(tspans) == 2 and np.isscalar(tspans[0]):
        tspans = [tspans] * n
    per_instance = isinstance(saveat, list) and len(saveat) == n and all(
        v is None or not np.isscalar(v) for v in saveat)
    saves = saveat if per_instance else [saveat] * n
    grids = [np.array(saved_times(ts, sv), dtype=np.float64) for ts, sv in zip(tspans, saves)]
    xs = _device_states(compiled, rho0s)
    names, obs_dev = [], []
    if observables:
        per_instance = isinstance(observables, (list, tuple)) and len(observables) == n and all(
            isinstance(o, dict) for o in observables)
        first = observables[0] if per_instance else observables
        names = list(first.keys()) if isinstance(first, dict) else [k for k, _ in first]
        for i, c in enumerate(compiled):
            src = observables[i] if per_instance else dict(first) if not isinstance(first, dict) else first
            datas = [_observable_data(c.basis, src[k]) for k in names]
            obs_dev.append(torch.from_numpy(np.ascontiguousarray(np.stack(datas))).cuda())
    nobs = len(names)
    vals = [np.zeros((len(g), max(nobs, 1), 2), dtype=np.float64) for g in grids]
    jobs = (_lib.pi_dynamics_job_t * n)()
    for i in range(n):
        jobs[i].plan = compiled[i].handle
        jobs[i].state_dev = _ptr(xs[i])
        jobs[i].nt = len(grids[i])
        jobs[i].times = _lib.dptr(grids[i])
        jobs[i].nobs = nobs
        jobs[i].obs_dev = _ptr(obs_dev[i]) if nobs else None
        jobs[i].values_host = _lib.dptr(vals[i])
    infos = (_lib.pi_expv_info_t * n)()
    o = algorithm.opts()
    torch.cuda.synchronize()
    _lib.check(_lib.load().pi_dynamics_batch(n, jobs, C.byref(o), infos), "solve_dynamics_batch")
    results = []
    for i in range(n):
        values = {k: vals[i][:, j, 0] + 1j * vals[i][:, j, 1] for j, k in enumerate(names)}
        results.append(DynamicsStreamResult(list(grids[i]), None, values))
    finals = [x.cpu().numpy() for x in xs]
    if return_info:
        return results, finals, [{f: getattr(i, f) for f, _ in i._fields_} for i in infos]
    return results, finals


def stationary_state_batch(models, algorithm: GMRESAlgorithm | None = None, atol=1e-10, rtol=1e-8,
                           operator_scale=None, max_refinements=200, return_info=False,
                           raise_on_failure=True):
    """stationary_state for many models in one batched engine run.

    With raise_on_failure=False a non-converged instance does not raise: its info carries
    converged=False (a scan keeps the points that did converge)."""
    torch = _torch()
    algorithm = algorithm or GMRESAlgorithm()
    if algorithm.preconditioner is not None:
        raise PiArgumentError("batched steady states run unpreconditioned; solve preconditioned steady states "
                              "with stationary_state")
    compiled = [_as_compiled(m) for m in models]
    n = len(compiled)
    o = _lib.pi_gmres_opts_t()
    lib = _lib.load()
    lib.pi_gmres_default_opts(C.byref(o))
    o.krylovdim = algorithm.krylovdim
    o.maxiter = algorithm.maxiter
    o.atol, o.rtol = atol, rtol
    o.operator_scale = float(operator_scale) if operator_scale else 0.0
    o.precision = _lib.PI_FP32 if algorithm.precision == "mixed" else _lib.PI_FP64
    o.max_refinements = max_refinements
    xs = [torch.zeros(len(c.basis), dtype=torch.complex128, device="cuda") for c in compiled]
    torch.cuda.synchronize()
    infos = (_lib.pi_gmres_info_t * n)()
    rc = lib.pi_steady_state_batch(n, _ptr_array([c.handle for c in compiled]),
                                   _ptr_array([_ptr(x) for x in xs]), C.byref(o), infos)
    if raise_on_failure or rc != _lib.PI_ERR_NOT_CONVERGED:
        _lib.check(rc, "stationary_state_batch")
    states = [PIState(c.basis, x.cpu().numpy()) for c, x in zip(compiled, xs)]
    if return_info:
        return states, [{f: getattr(i, f) for f, _ in i._fields_} for i in infos]
    return states


def set_engine_schedule(schedule="auto"):
    """Step-apply schedule of the batched FP32 engine (scans, batched solves, FP32 servers):
    "auto" (timed per job-set shape, the default), "per_tile" (one block per (instance,
    sector-tile) item) or an int k >= 1 (a persistent launch of k blocks per SM).  Results
    are bitwise the same for every schedule.  Process-wide."""
    if schedule == "auto":
        code = _lib.PI_SCHEDULE_AUTO
    elif schedule == "per_tile":
        code = _lib.PI_SCHEDULE_PER_TILE
    elif isinstance(schedule, int) and not isinstance(schedule, bool) and schedule >= 1:
        code = schedule
    else:
        raise _lib.PiArgumentError(f"engine schedule must be 'auto', 'per_tile' or a positive int, got {schedule!r}")
    _lib.check(_lib.load().pi_engine_set_apply_schedule(code), "set_engine_schedule")


def engine_schedule_info():
    """The batched engine's last step-apply schedule choice: the schedule ("per_tile" or
    blocks per SM), the work-list size it was made for, the resident-block limit, and the
    median time of every candidate when the choice was timed."""
    info = _lib.pi_schedule_info_t()
    _lib.check(_lib.load().pi_engine_schedule_info(C.byref(info)), "engine_schedule_info")

    def name(k):
        return "per_tile" if k == _lib.PI_SCHEDULE_PER_TILE else int(k)

    return {"choices": info.choices, "tunings": info.tunings, "schedule": name(info.schedule),
            "items": info.items, "resident_max": info.resident_max,
            "candidates_us": {str(name(info.cand[i])): info.cand_us[i] for i in range(info.ncand)}}
