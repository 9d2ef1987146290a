"""Compiled model families and parameter scans on the batched engine.

Mirrors the reference's compiled_families.jl (compile_family :154-174, specialize :260-309)
and scans.jl (ParameterScanPlan :42-213, ParameterScanPoint :256-275, ParameterScanResult
:285-292, parameter_scan :1457-1467) for the steady-state and spectral tasks.  Term indices
are 0-based (Python), where the reference's are 1-based.

Execution modes:
  - "serial" (the reference's default): points one after another through the single-instance
    solver, each warm-started from the previous success when continuation=True
    (scans.jl:935-972);
  - "threads" / "batched": every selected point's plan is built in host threads and all
    points are solved together in ONE batched engine run (pi_steady_state_batch), the GPU
    form of the reference's threaded execution, which likewise requires continuation=False.
A point's result does not depend on the other points of the batch.
"""
from __future__ import annotations

import inspect
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field, replace
from numbers import Integral, Real

import numpy as np

from ._lib import PiArgumentError, PiDimensionMismatch, PiError, PiNotConverged
from .core import PIModel, Term

_SCAN_TASKS = ("steady_state", "spectrum")
_SCAN_EXECUTIONS = ("serial", "threads", "batched")
_SCAN_FAILURE_POLICIES = ("stop", "record", "throw")


# ---------------------------------------------------------------------------------------
# Families (compiled_families.jl)
# ---------------------------------------------------------------------------------------

@dataclass
class CompiledPIModelFamily:
    """A fixed-operator prototype whose selected term rates vary (compiled_families.jl:12-18)."""
    model: PIModel
    rate_indices: tuple
    default_rates: tuple

    def __len__(self):
        return len(self.model.basis)


def _family_rate_indices(model: PIModel, rate_indices):
    """compiled_families.jl:53-64 (0-based here)."""
    nterms = len(model.terms)
    indices = list(range(nterms)) if rate_indices is None else list(rate_indices)
    if not indices:
        raise PiArgumentError("rate_indices cannot be empty")
    if not all(isinstance(i, Integral) and not isinstance(i, bool) for i in indices):
        raise PiArgumentError("rate_indices must contain integers")
    if not all(0 <= i < nterms for i in indices):
        raise IndexError(f"rate_indices {indices} out of range for {nterms} terms")
    if len(set(indices)) != len(indices):
        raise PiArgumentError("rate_indices must be unique")
    return tuple(sorted(int(i) for i in indices))


def compile_family(model: PIModel, rate_indices=None) -> CompiledPIModelFamily:
    """compile_family(model; rate_indices) (compiled_families.jl:154-174)."""
    if not isinstance(model, PIModel):
        raise PiArgumentError("compile_family requires a PIModel prototype")
    indices = _family_rate_indices(model, rate_indices)
    defaults = tuple(model.terms[i].rate for i in indices)
    if not all(isinstance(r, Real) and np.isfinite(r) for r in defaults):
        raise PiArgumentError("every selected family rate must be real and finite in the prototype")
    return CompiledPIModelFamily(model, indices, tuple(float(r) for r in defaults))


def _family_rates(family: CompiledPIModelFamily, rates):
    """compiled_families.jl:176-193."""
    count = len(family.rate_indices)
    if isinstance(rates, Real) and not isinstance(rates, bool):
        if count != 1:
            raise PiArgumentError("a scalar rate is valid only for a family with one selected term")
        values = (rates,)
    else:
        values = tuple(rates)
    if len(values) != count:
        raise PiDimensionMismatch(f"expected {count} family rates, got {len(values)}")
    for position, value in enumerate(values):
        if not isinstance(value, Real) or isinstance(value, bool):
            raise PiArgumentError(f"family rate {position} must be a real number")
        if not np.isfinite(value):
            raise PiArgumentError(f"family rate {position} must be finite")
    return tuple(float(v) for v in values)


def _family_model(family: CompiledPIModelFamily, rates) -> PIModel:
    """_family_replace_rates (compiled_families.jl:78-85)."""
    terms = list(family.model.terms)
    for position, index in enumerate(family.rate_indices):
        terms[index] = replace(terms[index], rate=rates[position])
    return PIModel(family.model.basis, terms)


def specialize(family: CompiledPIModelFamily, rates=None, backend: str = "cuda"):
    """specialize(family, rates) (compiled_families.jl:260-309): a CompiledPIModel of the
    prototype with the selected rates bound.  The plan is lowered again for the new rates
    (host lowering is tens of milliseconds at N ~ 100)."""
    from .backend import compile as _compile
    if backend not in ("cuda", "auto", "matrixfree"):
        raise PiArgumentError("backend must be :cuda, :auto or :matrixfree")
    bound = _family_rates(family, family.default_rates if rates is None else rates)
    compiled = _compile(_family_model(family, bound), backend="cuda")
    compiled.family = family
    compiled.rates = bound
    return compiled


# ---------------------------------------------------------------------------------------
# Parameter scans (scans.jl)
# ---------------------------------------------------------------------------------------

def _accepts(fn, nargs):
    """Whether fn can be called with nargs positional arguments (the reference's
    `applicable` test for builders, remakers and rate builders)."""
    try:
        inspect.signature(fn).bind(*([None] * nargs))
        return True
    except TypeError:
        return False
    except ValueError:  # no signature available (builtins): assume the one-argument form
        return nargs == 1


@dataclass
class _FamilyRequest:
    family: CompiledPIModelFamily
    rates: object


class ParameterScanPlan:
    """ParameterScanPlan(parameters, model_builder; task, algorithm, ...) (scans.jl:85-156),
    ParameterScanPlan(parameters, prototype, remaker) (:158-180) and
    ParameterScanPlan(parameters, family; rate_builder) (:189-213)."""

    def __init__(self, parameters, builder, remaker=None, *, task="steady_state", algorithm=None,
                 solver_options=None, continuation=True, save_outputs=True, save_vectors=False,
                 save_restart=True, spectrum_target="largest_real", nev=6, diagnostic=None, seed=0,
                 rate_builder=None, atol=1e-10, rtol=1e-8):
        from .backend import GMRESAlgorithm, HarmonicArnoldiAlgorithm
        if task not in _SCAN_TASKS:
            raise PiArgumentError("task must be :steady_state or :spectrum")
        if spectrum_target not in ("largest_real", "near_zero", "largest_magnitude"):
            raise PiArgumentError("spectrum_target must be :largest_real, :near_zero, or :largest_magnitude")
        if not isinstance(nev, Integral) or isinstance(nev, bool) or nev <= 0:
            raise PiArgumentError("nev must be positive")
        values = list(parameters)
        if not values:
            raise PiArgumentError("parameters cannot be empty")
        if isinstance(builder, CompiledPIModelFamily):
            family = builder
            if rate_builder is not None and not (_accepts(rate_builder, 2) or _accepts(rate_builder, 1)):
                raise PiArgumentError("rate_builder must accept (parameter) or (parameter, index)")

            def make(parameter, index):
                if rate_builder is None:
                    rates = parameter
                elif _accepts(rate_builder, 2):
                    rates = rate_builder(parameter, index)
                else:
                    rates = rate_builder(parameter)
                return _FamilyRequest(family, rates)
        elif remaker is not None:
            prototype = builder
            if not (_accepts(remaker, 3) or _accepts(remaker, 2)):
                raise PiArgumentError("remaker must accept (prototype, parameter) or (prototype, parameter, index)")

            def make(parameter, index):
                if _accepts(remaker, 3):
                    return remaker(prototype, parameter, index)
                return remaker(prototype, parameter)
        else:
            if not callable(builder) or not (_accepts(builder, 1) or _accepts(builder, 2)):
                raise PiArgumentError("model_builder must accept (parameter) or (parameter, index)")

            def make(parameter, index):
                if _accepts(builder, 2):
                    return builder(parameter, index)
                return builder(parameter)
        self.model_builder = make
        soptions = dict(solver_options or {})
        if task == "steady_state":
            algorithm = algorithm or GMRESAlgorithm()
            if isinstance(algorithm, str):
                if algorithm not in ("auto", "krylov", "gmres"):
                    raise PiArgumentError(f"unsupported steady-state scan algorithm {algorithm}")
                algorithm = GMRESAlgorithm()
            if not isinstance(algorithm, GMRESAlgorithm):
                raise PiArgumentError("steady-state scans on the CUDA path use GMRESAlgorithm")
            managed = ("return_info", "initial_state", "workspace", "memory_budget", "krylovdim")
        else:
            # _spectrum_algorithm (highlevel.jl:735-746): automatic selection takes harmonic
            # Arnoldi for modes near zero and Arnoldi otherwise (the CUDA path has no dense
            # spectrum); an explicit Arnoldi request for modes near zero orders by smallest
            # modulus.
            algorithm = algorithm or "auto"
            if not isinstance(algorithm, HarmonicArnoldiAlgorithm):
                if algorithm not in ("auto", "krylov", "arnoldi", "harmonic", "iram", "implicit_qr"):
                    raise PiArgumentError(f"unsupported spectral scan algorithm {algorithm}; the CUDA path runs "
                                          "Arnoldi, implicitly restarted Arnoldi and harmonic Arnoldi")
                if algorithm == "harmonic" or (algorithm == "auto" and spectrum_target == "near_zero"):
                    algorithm = HarmonicArnoldiAlgorithm(nev=int(nev), krylovdim=soptions.pop("krylovdim", None),
                                                         thickdim=soptions.pop("thickdim", None),
                                                         maxrestarts=soptions.pop("maxrestarts", 20))
                else:
                    algorithm = "iram" if algorithm in ("iram", "implicit_qr") else "arnoldi"
            managed = ("return_info", "initial_vector", "workspace", "rng", "vectors", "nev", "subspace_dim",
                       "target", "memory_budget")
        forbidden = [k for k in managed if k in soptions]
        if forbidden:
            raise PiArgumentError(f"solver_options contains internally managed keyword(s): {', '.join(forbidden)}")
        if not isinstance(seed, Integral) or seed < 0 or seed >= 2 ** 64:
            raise PiArgumentError("seed must be a nonnegative integer that fits in UInt64")
        self.parameters = values
        self.task = task
        self.algorithm = algorithm
        self.solver_options = soptions
        self.continuation = bool(continuation)
        self.save_outputs = bool(save_outputs)
        self.save_vectors = bool(save_vectors)
        self.save_restart = bool(save_restart)
        self.diagnostic = diagnostic
        self.spectrum_target = spectrum_target
        self.nev = int(nev)
        self.seed = int(seed)
        self.atol = float(soptions.pop("atol", atol))
        self.rtol = float(soptions.pop("rtol", rtol))

    def __len__(self):
        return len(self.parameters)


@dataclass
class ParameterScanPoint:
    """One scan record (scans.jl:256-275); status "success" or "failed"."""
    index: int
    parameter: object
    status: str
    output: object
    residual: object
    trace_error: object
    converged: bool
    iterations: object
    compile_seconds: float
    solve_seconds: float
    elapsed_seconds: float
    warm_started: bool
    workspace_reused: bool
    diagnostics: object
    error_type: str | None
    message: str | None


@dataclass
class ParameterScanResult:
    """Scan output (scans.jl:285-292): parameters, point records, restart prefix and seed."""
    task: str
    parameters: list
    points: list
    restart_index: int
    restart_seed: object
    metadata: dict = field(default_factory=dict)

    def __len__(self):
        return len(self.points)

    def __getitem__(self, i):
        return self.points[i]

    def __iter__(self):
        return iter(self.points)


def _scan_indices(plan, indices):
    """scans.jl:1106-1114 (0-based)."""
    if indices is None:
        return list(range(len(plan.parameters)))
    selected = [int(i) for i in indices]
    if not all(0 <= i < len(plan.parameters) for i in selected):
        raise IndexError(f"scan indices {selected} out of range")
    if any(b <= a for a, b in zip(selected, selected[1:])):
        raise PiArgumentError("scan indices must be strictly increasing and unique")
    return selected


def _scan_max_points(indices, max_points):
    """scans.jl:1116-1121."""
    if max_points is None:
        return indices
    if not isinstance(max_points, Integral) or isinstance(max_points, bool) or max_points < 0:
        raise PiArgumentError("max_points must be a nonnegative integer or nothing")
    return indices[:int(max_points)]


def _scan_callback(callback, point):
    """scans.jl:1123-1131: the callback returns None or "stop"."""
    if callback is None:
        return False
    value = callback(point)
    if value is None:
        return False
    if value == "stop":
        return True
    raise PiArgumentError("callback must return nothing or :stop")


def _compile_point(plan, parameter, index):
    from .backend import CompiledPIModel, compile as _compile
    made = plan.model_builder(parameter, index)
    if isinstance(made, _FamilyRequest):
        return specialize(made.family, made.rates)
    if isinstance(made, CompiledPIModel):
        return made
    if isinstance(made, PIModel):
        return _compile(made, backend="cuda")
    raise PiArgumentError("model_builder must return a PIModel or a CompiledPIModel")


def _failed(index, parameter, err, elapsed):
    return ParameterScanPoint(index, parameter, "failed", None, None, None, False, None, 0.0, 0.0, elapsed,
                              False, False, None, type(err).__name__, str(err))


def _success(plan, index, parameter, compiled, state, info, compile_s, solve_s, elapsed, warm):
    user = plan.diagnostic(state, parameter, index) if plan.diagnostic is not None else None
    diagnostics = dict(solver=info, user=user, backend="cuda", dimension=len(compiled.basis))
    return ParameterScanPoint(index, parameter, "success", state if plan.save_outputs else None,
                              info.get("residual"), info.get("trace_error"), bool(info.get("converged")),
                              info.get("iterations"), compile_s, solve_s, elapsed, warm, False, diagnostics,
                              None, None)


def _handle_failure(on_error, err):
    if on_error == "throw":
        raise err


def _point_rng(seed, index):
    """Per-point generator from the plan seed and the point index (scans.jl:1055-1060), so a
    point's starting vector does not depend on the execution order."""
    mixed = (seed ^ ((index * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF)) & 0xFFFFFFFFFFFFFFFF
    return np.random.default_rng(mixed)


def _spectrum_points(plan, selected, callback, on_error, kw):
    """Spectral task (scans.jl:974-1053): one device Arnoldi, implicitly restarted Arnoldi or
    harmonic Arnoldi process per point.  With continuation=True, harmonic Arnoldi starts
    from the previous point's Ritz vectors as an initial subspace; the Arnoldi methods start
    from their combination v_1 + sum_c v_c / c, normalised (scans.jl:1020-1041)."""
    from .backend import (HarmonicArnoldiAlgorithm, harmonic_arnoldi_spectrum, implicitly_restarted_arnoldi_spectrum,
                          krylov_liouvillian_spectrum)
    harmonic = isinstance(plan.algorithm, HarmonicArnoldiAlgorithm)
    ordinary = implicitly_restarted_arnoldi_spectrum if plan.algorithm == "iram" else krylov_liouvillian_spectrum
    which = {"largest_real": "LR", "largest_magnitude": "LM", "near_zero": "SM"}[plan.spectrum_target]
    points, seed, stopped = [], None, False
    for index in selected:
        parameter = plan.parameters[index]
        t0 = time.perf_counter()
        try:
            compiled = _compile_point(plan, parameter, index)
            n = len(compiled.basis)
            t1 = time.perf_counter()
            warm = plan.continuation and seed is not None and seed.shape[0] == n
            want_vectors = plan.save_vectors or plan.continuation
            if harmonic:
                a = plan.algorithm
                opts = dict(nev=a.nev, krylovdim=a.krylovdim, thickdim=a.thickdim, maxrestarts=a.maxrestarts)
                opts.update(kw)
                res = harmonic_arnoldi_spectrum(compiled, initial_subspace=seed if warm else None,
                                                vectors=want_vectors, rng=_point_rng(plan.seed, index), **opts)
            else:
                res = ordinary(compiled, nev=plan.nev, which=which, initial_vector=seed if warm else None,
                               vectors=want_vectors, rng=_point_rng(plan.seed, index), **kw)
            t2 = time.perf_counter()
            vecs = res.pop("vectors", None)
            if plan.continuation and vecs is not None and vecs.shape[1] > 0:
                seed = vecs.copy() if harmonic else _arnoldi_continuation(vecs)
            output = dict(values=res["values"], vectors=vecs if plan.save_vectors else None, info=res)
            user = plan.diagnostic(output, parameter, index) if plan.diagnostic is not None else None
            point = ParameterScanPoint(index, parameter, "success", output if plan.save_outputs else None,
                                       float(res["residuals"].max()), None, bool(res["converged"].all()),
                                       res["iterations"], t1 - t0, t2 - t1, t2 - t0, warm, False,
                                       dict(solver=res, user=user, backend="cuda", dimension=n,
                                            method="harmonic" if harmonic else plan.algorithm), None, None)
        except (PiError, ValueError) as err:
            _handle_failure(on_error, err)
            point = _failed(index, parameter, err, time.perf_counter() - t0)
        points.append(point)
        if _scan_callback(callback, point) or (point.status == "failed" and on_error == "stop"):
            stopped = True
            break
    return points, seed, stopped


def _arnoldi_continuation(vecs):
    """The Arnoldi continuation vector (scans.jl:1026-1041): an exactly converged single
    eigenvector would make the next factorisation break down after one step, so the seed is
    v_1 + sum_{c >= 2} v_c / c over the selected modes, normalised (v_1 when that vanishes)."""
    vector = vecs[:, 0].copy()
    for column in range(1, vecs.shape[1]):
        vector += vecs[:, column] / (column + 1)
    norm = np.linalg.norm(vector)
    return vecs[:, 0].copy() if norm == 0 else vector / norm


def parameter_scan(plan: ParameterScanPlan, callback=None, indices=None, execution="serial", on_error="stop",
                   max_points=None):
    """parameter_scan(plan; callback, indices, execution, on_error, max_points)
    (scans.jl:1457-1467).  Steady-state points run batched for execution "threads" /
    "batched"; spectral points run one device Arnoldi process each in every mode."""
    from .backend import stationary_state, stationary_state_batch
    if execution not in _SCAN_EXECUTIONS:
        raise PiArgumentError("execution must be :serial, :threads or :batched")
    if on_error not in _SCAN_FAILURE_POLICIES:
        raise PiArgumentError("on_error must be :stop, :record, or :throw")
    if execution != "serial" and plan.continuation:
        raise PiArgumentError("threaded execution requires continuation=false")
    selected = _scan_max_points(_scan_indices(plan, indices), max_points)
    started = time.perf_counter()
    points = []
    seed_state = None
    stopped = False
    kw = dict(atol=plan.atol, rtol=plan.rtol, **plan.solver_options)
    if plan.task == "spectrum":
        points, seed_state, stopped = _spectrum_points(plan, selected, callback, on_error, kw)
    elif execution == "serial":
        for index in selected:
            parameter = plan.parameters[index]
            t0 = time.perf_counter()
            try:
                compiled = _compile_point(plan, parameter, index)
                t1 = time.perf_counter()
                warm = (plan.continuation and seed_state is not None
                        and len(seed_state.data) == len(compiled.basis))
                res = stationary_state(compiled, algorithm=plan.algorithm, return_info=True,
                                       initial_state=seed_state.data if warm else None, **kw)
                t2 = time.perf_counter()
                info = dict(res.info)
                info.pop("state", None)
                point = _success(plan, index, parameter, compiled, res.state, info, t1 - t0, t2 - t1,
                                 t2 - t0, warm)
                if plan.continuation:
                    seed_state = res.state
            except (PiError, ValueError) as err:
                _handle_failure(on_error, err)
                point = _failed(index, parameter, err, time.perf_counter() - t0)
            points.append(point)
            if _scan_callback(callback, point) or (point.status == "failed" and on_error == "stop"):
                stopped = True
                break
    else:
        compiled, failures, compile_s = {}, {}, {}

        def build(index):
            t0 = time.perf_counter()
            try:
                return index, _compile_point(plan, plan.parameters[index], index), None, time.perf_counter() - t0
            except (PiError, ValueError) as err:
                return index, None, err, time.perf_counter() - t0
        with ThreadPoolExecutor(max_workers=16) as ex:
            for index, c, err, dt in ex.map(build, selected):
                compile_s[index] = dt
                if err is None:
                    compiled[index] = c
                else:
                    _handle_failure(on_error, err)
                    failures[index] = err
        ok = [i for i in selected if i in compiled]
        t1 = time.perf_counter()
        states, infos = (stationary_state_batch([compiled[i] for i in ok], algorithm=plan.algorithm,
                                                return_info=True, raise_on_failure=False, **kw)
                         if ok else ([], []))
        solve_s = time.perf_counter() - t1
        solved = dict(zip(ok, zip(states, infos)))
        for index in selected:
            parameter = plan.parameters[index]
            if index in failures:
                point = _failed(index, parameter, failures[index], compile_s[index])
            else:
                state, info = solved[index]
                if not info["converged"]:
                    err = PiNotConverged(f"steady state did not converge: residual {info['residual']:.3e} "
                                         f"after {info['iterations']} iterations")
                    _handle_failure(on_error, err)
                    point = _failed(index, parameter, err, compile_s[index] + solve_s)
                else:
                    point = _success(plan, index, parameter, compiled[index], state, dict(info),
                                     compile_s[index], solve_s, compile_s[index] + solve_s, False)
            points.append(point)
            if _scan_callback(callback, point) or (point.status == "failed" and on_error == "stop"):
                stopped = True
                break
    prefix = 0
    by_index = {p.index: p for p in points}
    while prefix < len(selected) and selected[prefix] in by_index and by_index[selected[prefix]].status == "success":
        prefix += 1
    restart_seed = seed_state if (plan.continuation and plan.save_restart) else None
    metadata = dict(continuation=plan.continuation, save_outputs=plan.save_outputs,
                    save_vectors=plan.save_vectors, save_restart=plan.save_restart, execution=execution,
                    requested_indices=selected, stopped=stopped, elapsed_seconds=time.perf_counter() - started,
                    atol=plan.atol, rtol=plan.rtol)
    return ParameterScanResult(plan.task, plan.parameters, points, prefix, restart_seed, metadata)
