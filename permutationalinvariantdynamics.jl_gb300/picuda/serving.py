"""Continuous-batching solve server over libpicuda's multi-instance engine (pi_server_*).

A Server accepts time-evolution requests (the work of one solve_dynamics(...; saveat=dt)
call, highlevel.jl:559-733) and steady-state requests (one stationary_state call,
krylov.jl:797-891) from Python, keeps their device buffers alive while the library's worker
thread serves them, and hands back results with submit/admit/finish timestamps.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .backend import CompiledPIModel, _as_compiled, _observable_data, _torch, saved_times
from .core import PIState


@dataclass
class Completion:
    tag: int
    kind: str
    status: int
    message: str
    submit_time: float
    start_time: float
    finish_time: float
    iterations: int
    operator_applications: int
    residual: float
    trace_error: float
    state: np.ndarray | None = None
    times: list | None = None
    values: dict = field(default_factory=dict)

    @property
    def latency(self) -> float:
        return self.finish_time - self.submit_time

    @property
    def ok(self) -> bool:
        return self.status == _lib.PI_OK


class Server:
    """Serving engine: precision 'fp64' or 'mixed', memory_budget in bytes of HBM.
    steady_solvers = k > 0 solves steady-state requests on k host threads beside the batched
    engine, each preconditioned (level sweep and drive part, adaptive); 0 keeps them in the
    engine, unpreconditioned."""

    def __init__(self, krylovdim=30, precision="fp64", memory_budget=160e9, max_active=0,
                 use_graphs=True, device=0, steady_solvers=0):
        if isinstance(steady_solvers, bool) or int(steady_solvers) < 0:
            raise _lib.PiArgumentError("steady_solvers must be a nonnegative integer")
        if precision not in ("fp64", "mixed"):
            raise _lib.PiArgumentError("precision must be 'fp64' or 'mixed'")
        self._torch = _torch()
        self._lib = _lib.load()
        o = _lib.pi_server_opts_t()
        self._lib.pi_server_default_opts(C.byref(o))
        o.krylovdim = krylovdim
        o.precision = _lib.PI_FP32 if precision == "mixed" else _lib.PI_FP64
        o.memory_budget = float(memory_budget)
        o.max_active = int(max_active)
        o.use_graphs = 1 if use_graphs else 0
        o.steady_solvers = int(steady_solvers)
        h = C.c_void_p()
        _lib.check(self._lib.pi_server_create(C.byref(o), device, C.byref(h)), "pi_server_create")
        self._h = h
        self._live = {}
        self._next = 1
        self.precision = precision

    def _tag(self, tag):
        if tag is None:
            tag = self._next
            self._next += 1
        if tag in self._live:
            raise _lib.PiArgumentError(f"request tag {tag} is already in flight")
        return int(tag)

    def submit_dynamics(self, model, rho0, t_final, dt, observables=None, atol=None, rtol=None, tag=None):
        """Evolves rho0 to t_final with saved times 0:dt:t_final; returns the request tag."""
        torch = self._torch
        c: CompiledPIModel = _as_compiled(model)
        data = rho0.data if isinstance(rho0, PIState) else np.asarray(rho0)
        x = torch.from_numpy(np.ascontiguousarray(data, dtype=np.complex128)).cuda()
        names, obs, vals = [], None, None
        times = saved_times((0.0, float(t_final)), float(dt))
        if observables:
            names = list(observables)
            obs = torch.from_numpy(np.ascontiguousarray(
                np.stack([_observable_data(c.basis, observables[k]) for k in names]))).cuda()
            vals = np.zeros((len(times), len(names), 2), dtype=np.float64)
        torch.cuda.synchronize()
        tag = self._tag(tag)
        r = _lib.pi_request_t()
        r.kind = _lib.PI_REQUEST_DYNAMICS
        r.plan = c.handle
        r.state_dev = x.data_ptr()
        r.t_final = float(t_final)
        r.dt = float(dt)
        r.atol = atol or 0.0
        r.rtol = rtol or 0.0
        r.nobs = len(names)
        r.obs_dev = obs.data_ptr() if obs is not None else None
        r.values_host = _lib.dptr(vals) if vals is not None else None
        r.tag = tag
        _lib.check(self._lib.pi_server_submit(self._h, C.byref(r)), "pi_server_submit")
        self._live[tag] = dict(kind="dynamics", compiled=c, x=x, obs=obs, vals=vals, names=names, times=times)
        return tag

    def submit_steady(self, model, atol=None, rtol=None, maxiter=None, tag=None):
        """Solves for the trace-one stationary state; returns the request tag."""
        torch = self._torch
        c: CompiledPIModel = _as_compiled(model)
        x = torch.zeros(len(c.basis), dtype=torch.complex128, device="cuda")
        torch.cuda.synchronize()
        tag = self._tag(tag)
        r = _lib.pi_request_t()
        r.kind = _lib.PI_REQUEST_STEADY
        r.plan = c.handle
        r.state_dev = x.data_ptr()
        r.atol = atol or 0.0
        r.rtol = rtol or 0.0
        r.maxiter = maxiter or 0
        r.tag = tag
        _lib.check(self._lib.pi_server_submit(self._h, C.byref(r)), "pi_server_submit")
        self._live[tag] = dict(kind="steady", compiled=c, x=x)
        return tag

    def poll(self, max_items=256, timeout_ms=0, fetch_state=True):
        """Completed requests (waits up to timeout_ms; < 0 waits for at least one)."""
        buf = (_lib.pi_completion_t * max_items)()
        n = C.c_int(0)
        _lib.check(self._lib.pi_server_poll(self._h, buf, max_items, C.byref(n), int(timeout_ms)),
                   "pi_server_poll")
        out = []
        for i in range(n.value):
            c = buf[i]
            live = self._live.pop(int(c.tag))
            comp = Completion(int(c.tag), live["kind"], c.status, c.message.decode(errors="replace"),
                              c.submit_time, c.start_time, c.finish_time, c.iterations,
                              c.operator_applications, c.residual, c.trace_error)
            if fetch_state:
                comp.state = live["x"].cpu().numpy()
            if live["kind"] == "dynamics":
                comp.times = live["times"]
                if live["vals"] is not None:
                    v = live["vals"]
                    comp.values = {k: v[:, j, 0] + 1j * v[:, j, 1] for j, k in enumerate(live["names"])}
            out.append(comp)
        return out

    def drain(self, fetch_state=True):
        """Waits until every submitted request has completed; returns their completions."""
        out = []
        while self._live:
            out.extend(self.poll(timeout_ms=-1, fetch_state=fetch_state))
        return out

    def stats(self) -> dict:
        s = _lib.pi_server_stats_t()
        _lib.check(self._lib.pi_server_stats(self._h, C.byref(s)), "pi_server_stats")
        return {f: getattr(s, f) for f, _ in s._fields_}

    def close(self):
        if self._h:
            self._lib.pi_server_destroy(self._h)
            self._h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
