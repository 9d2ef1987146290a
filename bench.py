"""Benchmark of the Schur-block Liouvillian hot path on GB300.

Workload (one step): the fused L x of the N=120 qubit-ensemble model (H = 0.3 Jz + 1.2 Jx,
local decay 0.2, local dephasing 0.1, collective decay 0.05/N; PI dimension 302,621) applied
to a batch of 128 resident state vectors (inputs larger than L2, no flush needed).  The
headline is the plain complex FP64 apply on that batch in the reference's matrix layout
(128 columns of the PI dimension, the layout of apply!(Y, compiled, X) on Julia matrices):
value = algorithmic bytes (read x once, write y once) / device time; e2e is the same apply
through the host-buffer C-ABI call pi_apply_host_f64 with the copies inside the timed
region.  The FP32 apply of the mixed-precision path (element-major batch, population
coordinates) is reported with its own roofline under "fp32"; steady-state, expv, RK4, scan
and serving rates and the CPU baseline (C restatement of the reference's threaded apply)
are reported beside them.  --impl reference times that CPU restatement on the same FP64
workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "permutationalinvariantdynamics.jl_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "L·x HBM GB/s; solves/s + p50/p99 latency at 1e-8 residual, mixed vs FP64"
N_QUBITS = 120
BATCH = 128


def model_c2(picuda, N=N_QUBITS):
    s = picuda.spin_matrices(2)
    return picuda.qubit_ensemble_model(N, hamiltonian=0.3 * s["jz"] + 1.2 * s["jx"], emission=0.2,
                                       dephasing=0.1, collective_emission=0.05 / N)


def to_oracle(model):
    """The same model for the CPU oracle (checker / CPU baseline only)."""
    from oracle import pi_oracle as O
    names = {0: "H", 1: "LJ", 2: "CJ"}
    b = O.PIBasis(model.basis.N, 2, sectors=model.basis.sectors)
    return O.PIModel(b, [O.Term(names[t.kind], t.operator, t.rate, t.hbar) for t in model.terms])


def solve_rates(picuda, torch):
    """Solves/s of the reference's Krylov methods, plain FP64 vs mixed precision.

    steady state: driven qubits N=16 (H = Jx, local decay 0.5; dim 969), GMRES(50) to
    atol 1e-10 / rtol 1e-8 -- a size of this family that the reference's unpreconditioned
    restarted GMRES brings to tolerance with margin (N=20 sits on the edge of its final
    trace test);
    dynamics: the N=120 ensemble, expv m=30 over 20 saved intervals of dt = 0.05 from the
    all-excited state with observables Jz and J+J- streamed at every saved time (the large
    time-evolution configuration runs 200 such intervals); observables built once.  The same
    dynamics with the reference's default algorithm, fixed-step RK4 with 64 steps per saved
    interval, FP64 and mixed (FP32 applies, double-float state)."""
    out = {}
    sm = picuda.spin_matrices(2)
    ss_model = picuda.Models.driven_qubits(16, drive=1.0, emission=0.5, pumping=0.0)
    cm = picuda.compile(ss_model)
    for prec in ("fp64", "mixed"):
        alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=5000, precision=prec)
        r = picuda.stationary_state(cm, algorithm=alg, return_info=True)  # warm
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            r = picuda.stationary_state(cm, algorithm=alg, return_info=True, operator_scale=r.info["operator_scale"])
            times.append(time.perf_counter() - t0)
        out[f"steady_{prec}"] = {"solves_per_s": 1.0 / statistics.median(times),
                                 "p50_ms": statistics.median(times) * 1e3, "p99_ms": max(times) * 1e3,
                                 "iterations": r.info["iterations"],
                                 "normalized_residual": r.info["normalized_residual"],
                                 "trace_error": r.info["trace_error"]}
    ref = None
    # the FP64 oracle's expv observables of the same 20 intervals (tests/golden, made by the
    # oracle on the CPU): every dynamics result states its error against them
    golden = ROOT / "tests" / "golden" / "ensemble_c2_N120_expv.npz"
    oracle_obs = np.load(golden) if golden.exists() else None

    def vs_oracle(vals):
        if oracle_obs is None:
            return None
        return float(max(np.abs(v - oracle_obs[k]).max() / np.abs(oracle_obs[k]).max()
                         for k, v in zip(("Jz", "JpJm"), vals)))

    c2 = picuda.compile(model_c2(picuda))
    rho0 = picuda.computational_product_state(c2.basis, 2)
    obs = {"Jz": picuda.collective_operator(c2.basis, sm["jz"]),
           "JpJm": picuda.collective_operator(c2.basis, sm["jp"] @ sm["jm"])}
    nint = 20
    for prec in ("fp64", "mixed"):
        alg = picuda.ExpvAlgorithm(krylovdim=30, precision=prec)
        picuda.solve_dynamics(c2, rho0, (0.0, 0.05), algorithm=alg, observables=obs, save_states=False)  # warm
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            res = picuda.solve_dynamics(c2, rho0, (0.0, 0.05 * nint), saveat=0.05, algorithm=alg, observables=obs,
                                        save_states=False)
            times.append(time.perf_counter() - t0)
        vals = np.array([res.values[k] for k in obs])
        if prec == "fp64":
            ref = vals
        per = statistics.median(times) / nint
        out[f"expv_{prec}"] = {"intervals_per_s": 1.0 / per, "ms_per_interval": per * 1e3,
                               "p50_ms_per_call": statistics.median(times) * 1e3, "p99_ms_per_call": max(times) * 1e3,
                               "intervals_per_call": nint,
                               "max_obs_rel_err_vs_fp64": float(np.max(np.abs(vals - ref) / np.abs(ref).max())),
                               "max_obs_rel_err_vs_oracle": vs_oracle(vals)}
    # The reference's default dynamics algorithm: fixed-step RK4, 64 steps per saved interval.
    ref_expv = ref
    for prec in ("fp64", "mixed"):
        kw = dict(observables=obs, save_states=False, steps_per_interval=64, precision=prec)
        picuda.solve_dynamics(c2, rho0, (0.0, 0.05), **kw)  # warm
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            res = picuda.solve_dynamics(c2, rho0, (0.0, 0.05 * nint), saveat=0.05, **kw)
            times.append(time.perf_counter() - t0)
        vals = np.array([res.values[k] for k in obs])
        if prec == "fp64":
            ref = vals
        per = statistics.median(times) / nint
        out[f"rk4_{prec}"] = {"intervals_per_s": 1.0 / per, "ms_per_interval": per * 1e3,
                              "us_per_stage": per / 256 * 1e6,
                              "p50_ms_per_call": statistics.median(times) * 1e3, "p99_ms_per_call": max(times) * 1e3,
                              "intervals_per_call": nint, "steps_per_interval": 64,
                              "max_obs_rel_err_vs_fp64": float(np.max(np.abs(vals - ref) / np.abs(ref).max())),
                              "max_obs_rel_dev_vs_expv_fp64": float(np.max(np.abs(vals - ref_expv)
                                                                           / np.abs(ref_expv).max())),
                              "max_obs_rel_err_vs_oracle": vs_oracle(vals)}
    return out


def scan_model(picuda, N, omega, gdown, gphi):
    """Parameter-scan family: H = Omega Jx, local decay gdown, local dephasing gphi,
    collective decay 1/N on J-."""
    s = picuda.spin_matrices(2)
    return picuda.qubit_ensemble_model(N, hamiltonian=omega * s["jx"], emission=gdown, dephasing=gphi,
                                       collective_emission=1.0 / N)


def scan_draws(count, seed=0, nmin=20, nmax=160):
    """Seeded scan points: N ~ U{nmin..nmax}, Omega ~ U[0.2, 2], gdown ~ U[0.05, 0.5],
    gphi ~ U[0, 0.2]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        N = int(rng.integers(nmin, nmax + 1))
        out.append((N, float(rng.uniform(0.2, 2.0)), float(rng.uniform(0.05, 0.5)), float(rng.uniform(0.0, 0.2))))
    return out


def compile_all(picuda, models, threads=16):
    """Plans built in parallel host threads (the C call releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(picuda.compile, models))


def scan_rates(picuda, torch, count=256, intervals=2, seed=0, precisions=("fp64", "mixed")):
    """Batched parameter scan: `count` instances (N ~ U{20..160}, uneven PI dimensions) each
    advance `intervals` saved intervals of dt = 0.05 from the all-excited state (expv m = 30,
    tol 1e-10/1e-8) in one batched engine run, observables Jz and J+J- at every saved time.
    Timed end to end: initial states uploaded from host, final states and observables read
    back.  Reported per precision, with the mixed run's deviation from the FP64 run."""
    sm = picuda.spin_matrices(2)
    draws = scan_draws(count, seed)
    models = [scan_model(picuda, *d) for d in draws]
    t0 = time.perf_counter()
    comp = compile_all(picuda, models)
    compile_s = time.perf_counter() - t0
    rho0 = [picuda.computational_product_state(m.basis, 2) for m in models]
    obs_ops = {"Jz": sm["jz"], "JpJm": sm["jp"] @ sm["jm"]}
    # per-instance PI vectors of the observables, built before the clock starts
    obs = [{k: picuda.collective_operator(m.basis, v) for k, v in obs_ops.items()} for m in models]
    dims = [len(m.basis) for m in models]
    out = {"instances": count, "intervals": intervals, "dt": 0.05, "sum_dim": int(sum(dims)),
           "min_dim": int(min(dims)), "max_dim": int(max(dims)), "plan_build_s": compile_s}
    vals = {}
    for prec in precisions:
        alg = picuda.ExpvAlgorithm(krylovdim=30, precision=prec)
        # untimed first call: memory-pool growth, graph instantiation
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        picuda.solve_dynamics_batch(comp, rho0, (0.0, 0.05), algorithm=alg, saveat=0.05)
        torch.cuda.synchronize()
        first_s = time.perf_counter() - t0
        tuning = picuda.engine_schedule_info() if prec == "mixed" else None
        t0 = time.perf_counter()
        res, fin, infos = picuda.solve_dynamics_batch(comp, rho0, (0.0, 0.05 * intervals), algorithm=alg, saveat=0.05,
                                                      observables=obs, return_info=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        vals[prec] = res
        out[prec] = {"seconds": dt, "instance_intervals_per_s": count * intervals / dt,
                     "first_call_1_interval_s": first_s,
                     "converged": int(sum(1 for i in infos if i["converged"])),
                     "accepted_steps": int(sum(i["accepted_steps"] for i in infos)),
                     "operator_applications": int(sum(i["operator_applications"] for i in infos))}
        out[prec]["applies_per_s"] = out[prec]["operator_applications"] / dt
        if prec == "mixed":  # the FP32 engine's step-apply schedule: timed in the untimed call
            out[prec]["apply_schedule_tuning"] = tuning
            out[prec]["apply_schedule"] = picuda.engine_schedule_info()["schedule"]
    if len(vals) < 2:
        return out
    dev = 0.0
    for a, b in zip(vals["mixed"], vals["fp64"]):
        for k in obs_ops:
            ref = np.abs(b.values[k]).max()
            dev = max(dev, float(np.abs(a.values[k] - b.values[k]).max() / max(ref, 1e-300)))
    out["mixed_max_observable_rel_dev_vs_fp64"] = dev
    out["speedup_mixed_vs_fp64"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    return out


def request_stream(count, seed=0, nmin=10, nmax=300, steady_fraction=0.3):
    """Served request mix: N = floor(exp(U[ln nmin, ln nmax])); 70% time evolution with
    t_final ~ U[1, 10], dt = 0.05; 30% steady state; parameters drawn as in the scan."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        N = int(np.floor(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        p = (N, float(rng.uniform(0.2, 2.0)), float(rng.uniform(0.05, 0.5)), float(rng.uniform(0.0, 0.2)))
        kind = "steady" if rng.uniform() < steady_fraction else "dynamics"
        reqs.append({"params": p, "kind": kind, "t_final": float(rng.uniform(1.0, 10.0)), "dt": 0.05})
    return reqs


def serve_rates(picuda, torch, count=24, rate=50.0, seed=0, budget=160e9, precisions=("fp64", "mixed"),
                steady_solvers=4):
    """Continuous-batching server on a Poisson request stream at `rate` req/s (the lowest
    rate of the served configuration; the stream saturates the GPU): p50/p99 latency
    (finish - submit) and completed solves/s, FP64 vs mixed, same requests and arrival
    times.  Plans are built before the clock starts.  steady_solvers > 0 solves the steady
    requests preconditioned on that many solver threads beside the batched engine (level
    sweep and drive part, adaptive); 0 runs them unpreconditioned in the engine."""
    reqs = request_stream(count, seed)
    sm = picuda.spin_matrices(2)
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=count))
    models = [scan_model(picuda, *r["params"]) for r in reqs]
    comp = compile_all(picuda, models)
    rho0 = [picuda.computational_product_state(m.basis, 2) for m in models]
    out = {"requests": count, "rate_per_s": rate, "memory_budget_bytes": budget,
           "dynamics": sum(1 for r in reqs if r["kind"] == "dynamics"),
           "steady": sum(1 for r in reqs if r["kind"] == "steady"),
           "max_dim": int(max(len(m.basis) for m in models)), "steady_solvers": steady_solvers}
    states, finals = {}, {}
    for prec in precisions:
        with picuda.Server(precision=prec, memory_budget=budget, steady_solvers=steady_solvers) as srv:
            t0 = time.perf_counter()
            done = []
            for i, r in enumerate(reqs):
                while time.perf_counter() - t0 < arrivals[i]:
                    done.extend(srv.poll(timeout_ms=1))
                if r["kind"] == "dynamics":
                    srv.submit_dynamics(comp[i], rho0[i], r["t_final"], r["dt"], tag=i + 1,
                                        observables={"tr": np.eye(2) / models[i].basis.N, "Jz": sm["jz"]})
                else:
                    srv.submit_steady(comp[i], tag=i + 1)
            done.extend(srv.drain())
            wall = time.perf_counter() - t0
            st = srv.stats()
        lat = np.array([c.latency for c in done])
        ok = [c for c in done if c.ok]
        span = max(c.finish_time for c in done) - min(c.submit_time for c in done)
        res = {"wall_s": wall, "completed": len(done), "ok": len(ok), "solves_per_s": len(ok) / span,
               "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
               "ticks": st["ticks"], "cycles": st["cycles"]}
        for kind in ("dynamics", "steady"):
            kl = np.array([c.latency for c in done if c.kind == kind])
            if len(kl):
                res[f"{kind}_p50_ms"] = float(np.percentile(kl, 50) * 1e3)
                res[f"{kind}_p99_ms"] = float(np.percentile(kl, 99) * 1e3)
        res["failed"] = [f"{c.tag}:{c.message[:80]}" for c in done if not c.ok][:5]
        res["ok_by_kind"] = {k: sum(1 for c in ok if c.kind == k) for k in ("dynamics", "steady")}
        res["failed_by_kind"] = {k: sum(1 for c in done if not c.ok and c.kind == k) for k in ("dynamics", "steady")}
        dyn = [c for c in done if c.ok and c.kind == "dynamics"]
        res["max_final_trace_error_dynamics"] = max((abs(c.values["tr"][-1] - 1) for c in dyn), default=None)
        out[prec] = res
        states[prec] = {c.tag: c.state for c in done if c.ok}
        finals[prec] = {c.tag: (c.values["tr"][-1], c.values["Jz"][-1]) for c in dyn}
    if len(precisions) < 2:
        return out
    # observable deviation on requests whose FP64 trace stayed within 1e-6 (the reference's
    # reference-coordinate error control loses trace at large N; see the FP64 trace errors)
    jdev, kept = 0.0, 0
    for tag, (tr64, jz64) in finals["fp64"].items():
        if tag in finals["mixed"] and abs(tr64 - 1) < 1e-6:
            kept += 1
            jdev = max(jdev, abs(finals["mixed"][tag][1] - jz64) / reqs[tag - 1]["params"][0])
    out["mixed_max_Jz_per_N_dev_vs_fp64"] = jdev
    out["requests_compared"] = kept
    for kind in ("steady",):
        # compared in population coordinates z = sqrt(f) x, the coordinates of the solves'
        # residual tests: at large N the reference coordinates of the high-multiplicity
        # sectors vanish and the max-norm would weigh only negligible populations
        dev, worst = 0.0, None
        for tag, ref in states["fp64"].items():
            got = states["mixed"].get(tag)
            if got is None or reqs[tag - 1]["kind"] != kind:
                continue
            sq = np.concatenate([np.full(n * n, f) for n, f in zip(comp[tag - 1].basis.dims,
                                                                     comp[tag - 1].sector_scales())])
            d = float(np.abs(sq * (got - ref)).max() / max(np.abs(sq * ref).max(), 1e-300))
            if d >= dev:
                dev, worst = d, tag
        out[f"mixed_max_state_rel_dev_vs_fp64_{kind}"] = dev
        if worst is not None:
            out[f"worst_{kind}_request"] = {"N": reqs[worst - 1]["params"][0], "params": reqs[worst - 1]["params"],
                                            "t_final": reqs[worst - 1]["t_final"]}
    out["solves_per_s_ratio_mixed_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    return out


def serve_sweep(picuda, torch, rates, count, fp64_rates=1, steady_solvers=4):
    """The served configuration's rate sweep: `count` requests per rate, mixed precision at
    every rate, plain FP64 at the first `fp64_rates` rates (the FP64 server needs minutes per
    rate at this size)."""
    out = {"requests_per_rate": count, "rates": list(rates), "per_rate": {}, "steady_solvers": steady_solvers}
    for i, rate in enumerate(rates):
        precs = ("fp64", "mixed") if i < fp64_rates else ("mixed",)
        out["per_rate"][str(rate)] = serve_rates(picuda, torch, count, rate, precisions=precs,
                                                 steady_solvers=steady_solvers)
    return out


def steady_family(picuda, family, count, seed):
    """Steady-state request sets.  'driven': driven qubits (H = Omega Jx, local decay gamma),
    N ~ U{8..20}, Omega ~ U[0.5, 1.5], gamma ~ U[0.3, 0.7] -- a family the reference's
    unpreconditioned restarted GMRES brings to tolerance (GMRES(50), maxiter 5000).
    'served': the served configuration's steady requests (N log-uniform in 10..300,
    parameters as in the scan; GMRES(30), maxiter 500)."""
    rng = np.random.default_rng(seed)
    if family == "driven":
        models = []
        for _ in range(count):
            N = int(rng.integers(8, 21))
            models.append(picuda.Models.driven_qubits(N, drive=float(rng.uniform(0.5, 1.5)),
                                                      emission=float(rng.uniform(0.3, 0.7)), pumping=0.0))
        return models, 50, 5000
    reqs = request_stream(count, seed, steady_fraction=1.0)
    return [scan_model(picuda, *r["params"]) for r in reqs], 30, 500


def steady_rates(picuda, torch, count=16, seed=7, family="driven"):
    """Steady-state solves/s at the reference's tolerance (atol 1e-10, rtol 1e-8 on the
    trace-bordered system): the plain FP64 GPU path (one pi_steady_state call per request,
    in turn) against the served engine in FP64 and in mixed precision (all requests
    submitted at once).  Solves/s counts converged solves only."""
    models, m, maxiter = steady_family(picuda, family, count, seed)
    comp = compile_all(picuda, models)
    out = {"family": family, "requests": count, "krylovdim": m, "maxiter": maxiter,
           "max_dim": int(max(len(x.basis) for x in models)), "n_values": [x.basis.N for x in models]}
    t0 = time.perf_counter()
    plain, its = {}, []
    for i, c in enumerate(comp):
        try:
            r = picuda.stationary_state(c, algorithm=picuda.GMRESAlgorithm(krylovdim=m, maxiter=maxiter),
                                        return_info=True)
            plain[i] = r.state.data
            its.append(r.info["iterations"])
        except picuda.PiNotConverged:
            plain[i] = None
            its.append(-1)
    dt = time.perf_counter() - t0
    okc = sum(1 for v in its if v >= 0)
    out["plain_fp64"] = {"seconds": dt, "converged": okc, "solves_per_s": okc / dt, "iterations": its,
                         "converged_without_iterations": sum(1 for v in its if v == 0)}
    for prec in ("fp64", "mixed"):
        with picuda.Server(krylovdim=m, precision=prec) as srv:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for i, c in enumerate(comp):
                srv.submit_steady(c, maxiter=maxiter, tag=i + 1)
            done = srv.drain()
            dt = time.perf_counter() - t0
        ok = [c for c in done if c.ok]
        lat = np.array([c.latency for c in done])
        dev = 0.0
        for c in ok:
            ref = plain.get(c.tag - 1)
            if ref is not None:
                dev = max(dev, float(np.abs(c.state - ref).max() / max(np.abs(ref).max(), 1e-300)))
        out[f"served_{prec}"] = {"seconds": dt, "converged": len(ok), "solves_per_s": len(ok) / dt,
                                 "p50_ms": float(np.percentile(lat, 50) * 1e3),
                                 "p99_ms": float(np.percentile(lat, 99) * 1e3),
                                 "max_normalized_residual": max((c.residual for c in ok), default=None),
                                 "max_state_rel_dev_vs_plain_fp64": dev}
    out["ratio_served_mixed_vs_plain_fp64"] = (out["served_mixed"]["solves_per_s"] /
                                               max(out["plain_fp64"]["solves_per_s"], 1e-300))
    return out


def drive_steady(picuda, torch, N=100, omega=1.5, gdown=0.1, gphi=0.05, repeats=3):
    """A strongly driven steady state (H = Omega Jx, local decay, local dephasing, collective
    decay 1/N; Omega well above the dissipation), where the reference's unpreconditioned
    GMRES and the level sweep stall: GMRES(30) in population coordinates with the level
    sweep and the drive part (adaptive ladder), FP64 against mixed precision, atol 1e-10,
    rtol 1e-8.  Preconditioners are built before the clock (their setup time is reported);
    each solve is timed alone."""
    m = scan_model(picuda, N, omega, gdown, gphi)
    c = picuda.compile(m)
    t0 = time.perf_counter()
    lev = picuda.level_preconditioner(c, coords="population")
    t1 = time.perf_counter()
    drv = picuda.drive_preconditioner(c, coords="population", operator_scale=lev.operator_scale)
    t2 = time.perf_counter()
    out = {"N": N, "dim": len(m.basis), "omega": omega, "gamma_down": gdown, "gamma_phi": gphi,
           "krylovdim": 50, "level_setup_s": t1 - t0, "drive_setup_s": t2 - t1,
           "drive_device_bytes": drv.info["device_bytes"]}
    states = {}
    for prec in ("fp64", "mixed"):
        alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=3000, precision=prec, preconditioner=lev,
                                    drive_preconditioner=drv)
        times, info = [], None
        for _ in range(repeats):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            try:
                res = picuda.stationary_state(c, algorithm=alg, return_info=True)
            except picuda.PiNotConverged as e:
                torch.cuda.synchronize()
                out[prec] = {"converged": False, "seconds": time.perf_counter() - t0, "message": str(e)[-120:]}
                break
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            info = res.info
        if info is None:
            continue
        states[prec] = res.state.data
        out[prec] = {"seconds_median": float(np.median(times)), "converged": bool(info["converged"]),
                     "iterations": info["iterations"], "restarts": info["restarts"],
                     "stage": info["preconditioner_stage"], "normalized_residual": info["normalized_residual"],
                     "trace_error": info["trace_error"], "operator_applications": info["operator_applications"]}
    if len(states) == 2:
        sq = np.concatenate([np.full(n * n, f) for n, f in zip(c.basis.dims, c.sector_scales())])
        out["mixed_state_rel_dev_vs_fp64_population"] = float(
            np.abs(sq * (states["mixed"] - states["fp64"])).max() / np.abs(sq * states["fp64"]).max())
        out["speedup_mixed_vs_fp64"] = out["fp64"]["seconds_median"] / out["mixed"]["seconds_median"]
    return out


def btc_model(picuda, N, omega_over_kappa):
    """Boundary-time-crystal-like steady-state configuration: H = Omega Jx with
    Omega = omega_over_kappa * kappa, collective decay kappa = 1/N on J-, local dephasing 0.01,
    all Schur sectors."""
    s = picuda.spin_matrices(2)
    kappa = 1.0 / N
    return picuda.qubit_ensemble_model(N, hamiltonian=omega_over_kappa * kappa * s["jx"], collective_emission=kappa,
                                       dephasing=0.01)


def steady_c3_rates(picuda, torch, N=200, omegas=(0.5, 1.0, 2.0), repeats=5, tol=5e-11, plain=True, concurrent=True,
                    served_per_omega=3):
    """Steady states of the N=200 boundary-time-crystal-like model (dim 1,373,701) for
    Omega in {0.5, 1, 2} kappa: restarted GMRES(50) left-preconditioned by the level sweep,
    in population coordinates, to a normalized residual and trace error of 1e-10
    (atol = rtol = 5e-11), plain FP64 against mixed precision (FP32 applies, Krylov basis and
    sweeps; FP64 residual refinement).  Plans and preconditioners are built before the clock;
    each solve is timed alone (host call to host return).  The reference's unpreconditioned
    GMRES(50) is run once per Omega in population coordinates with maxiter 500 to record
    whether it gets there."""
    out = {"N": N, "krylovdim": 50, "omegas_over_kappa": list(omegas), "repeats": repeats,
           "tolerance": {"atol": tol, "rtol": tol}, "coords": "population"}
    per = {}
    lat = {"fp64": [], "mixed": []}
    for w in omegas:
        c = picuda.compile(btc_model(picuda, N, w))
        t0 = time.perf_counter()
        P = picuda.level_preconditioner(c, coords="population")
        setup = time.perf_counter() - t0
        res = {}
        states = {}
        for prec in ("fp64", "mixed"):
            alg = picuda.GMRESAlgorithm(krylovdim=50, maxiter=2000, preconditioner=P, precision=prec)
            picuda.stationary_state(c, algorithm=alg, atol=tol, rtol=tol)  # warm
            times = []
            for _ in range(repeats):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r = picuda.stationary_state(c, algorithm=alg, return_info=True, atol=tol, rtol=tol)
                times.append(time.perf_counter() - t0)
            lat[prec].extend(times)
            states[prec] = r.state.data
            res[prec] = {"ms_p50": statistics.median(times) * 1e3, "ms_max": max(times) * 1e3,
                         "iterations": r.info["iterations"], "restarts": r.info["restarts"],
                         "refinements": r.info["refinements"],
                         "normalized_residual": r.info["normalized_residual"],
                         "trace_error": r.info["trace_error"], "converged": bool(r.info["converged"])}
        sq = c.sector_scales()
        scale = np.concatenate([np.full(n * n, sq[i]) for i, n in enumerate(c.basis.dims)])
        z64, z32 = states["fp64"] * scale, states["mixed"] * scale
        res["mixed_state_rel_dev_vs_fp64"] = float(np.abs(z32 - z64).max() / np.abs(z64).max())
        res["preconditioner_setup_s"] = setup
        res["preconditioner_bytes"] = P.info["device_bytes"]
        try:
            if plain:
                ref = picuda.stationary_state(c, algorithm=picuda.GMRESAlgorithm(krylovdim=50, maxiter=500),
                                              return_info=True, atol=tol, rtol=tol, coords="population")
                res["unpreconditioned_fp64"] = {"converged": True, "iterations": ref.info["iterations"]}
        except picuda.PiNotConverged as err:
            res["unpreconditioned_fp64"] = {"converged": False, "maxiter": 500, "message": str(err)[-120:]}
        per[str(w)] = res
        P.close()
    out["per_omega"] = per
    for prec in ("fp64", "mixed"):
        a = np.array(lat[prec])
        out[prec] = {"solves_per_s": len(a) / a.sum(), "p50_ms": float(np.percentile(a, 50) * 1e3),
                     "p99_ms": float(np.percentile(a, 99) * 1e3), "solves": int(len(a))}
    out["solves_per_s_ratio_mixed_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    if concurrent:
        out["served"] = steady_c3_served(picuda, torch, N, omegas, repeats, tol, per_omega=served_per_omega)
        out["served_mixed_vs_plain_fp64"] = out["served"]["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    return out


def steady_c3_served(picuda, torch, N, omegas, repeats, tol, per_omega=2):
    """The same solves in served form: per_omega host threads per Omega, each with its own
    compiled model, preconditioner and CUDA stream, keep solving, so independent requests
    overlap on the GPU.  Throughput = solves / wall time; latency = each solve's own duration."""
    from concurrent.futures import ThreadPoolExecutor
    comps = [picuda.compile(btc_model(picuda, N, w)) for w in omegas for _ in range(per_omega)]
    precs = [picuda.level_preconditioner(c, coords="population") for c in comps]
    nw = len(comps)
    out = {"workers": nw, "solves_per_worker": repeats}
    for prec in ("fp64", "mixed"):
        algs = [picuda.GMRESAlgorithm(krylovdim=50, maxiter=2000, preconditioner=P, precision=prec) for P in precs]
        for c, a in zip(comps, algs):
            picuda.stationary_state(c, algorithm=a, atol=tol, rtol=tol)  # warm

        def worker(i):
            torch.cuda.set_device(torch.cuda.current_device())
            lat = []
            for _ in range(repeats):
                t0 = time.perf_counter()
                r = picuda.stationary_state(comps[i], algorithm=algs[i], return_info=True, atol=tol, rtol=tol)
                lat.append(time.perf_counter() - t0)
                if not r.info["converged"]:
                    raise RuntimeError("served C3 solve did not converge")
            return lat

        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=nw) as ex:
            lats = [x for part in ex.map(worker, range(nw)) for x in part]
        wall = time.perf_counter() - t0
        a = np.array(lats)
        out[prec] = {"solves_per_s": len(a) / wall, "wall_s": wall, "p50_ms": float(np.percentile(a, 50) * 1e3),
                     "p99_ms": float(np.percentile(a, 99) * 1e3), "solves": int(len(a))}
    for P in precs:
        P.close()
    return out


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name):
    """DRAM bytes per launch recorded from an ncu capture summary in profiles/ (or None)."""
    p = ROOT / "profiles" / "traffic.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith(name + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [v.strip() for v in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    """One process per GPU (torchrun): NCCL on GPUs, gloo where CUDA is absent (the CPU tests
    of the replica path)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value, world):
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(bytes_per_rank, ms_per_step, world):
    """Whole-job throughput of independent replicas (weak scaling): every rank processes
    bytes_per_rank per step, and the job takes the slowest rank's time (max over ranks)."""
    ms = max_over_ranks(ms_per_step, world)
    return world * bytes_per_rank / (ms * 1e-3) / 1e9, ms


def stencil_flops(picuda, model):
    """Algorithmic real flops of one FP64 apply (fma counted as 2) from the stencil tables."""
    table, _ = picuda.stencil_tables(model)
    dims = model.basis.dims
    cost = {(0, 0): 10, (0, 1): 10, (0, 2): 10, (1, 0): 4, (1, 1): 4, (1, 2): 8,
            (2, 0): 4, (2, 1): 4, (2, 2): 8, (3, 0): 5, (3, 1): 14, (3, 2): 14}
    total = 0
    for row in table.tolist():
        s, src, kind, cls, dr, dc = row[:6]
        n, m = dims[s], dims[src]
        rows = max(0, min(n, m - dr) - max(0, -dr))
        cols = max(0, min(n, m - dc) - max(0, -dc))
        total += cost[(kind, cls)] * rows * cols
    return total


def cpu_baseline_apply(model_oracle_plan, n, budget_s=10.0, max_vectors=2000):
    """Times the oracle's C threaded apply (FP64, all host cores) on a bounded sample."""
    from oracle import cpu_baseline
    ta = cpu_baseline.ThreadedApply(model_oracle_plan)
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(1)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex128)
    y = np.empty_like(x)
    ta(x, y, threads)  # warm
    count = 0
    t0 = time.perf_counter()
    while count < max_vectors:
        ta(x, y, threads)
        count += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    gbs = 2 * 16 * n * count / dt / 1e9
    return gbs, threads, count, dt


WORKLOAD = ("fused L x, N=120 qubit ensemble (dim 302,621), batch of 128 state vectors as 128 columns "
            "(the layout of apply!(Y, compiled, X)), complex FP64")


def config_of(n):
    """The workload's config, identical on both arms."""
    return {"workload": WORKLOAD, "batch": BATCH, "pi_dim": n,
            "model": "H=0.3Jz+1.2Jx, local decay 0.2, local dephasing 0.1, collective decay 0.05/N",
            "l2": "inputs larger than L2 (620 MB read per step), no flush needed"}


def run_reference(args, world, rank):
    """--impl reference: the reference's CPU matrix-free apply (restated in C, threaded over
    all host cores) on the headline workload: every step applies L to the same 128 FP64
    columns."""
    if rank != 0:
        return 0
    import picuda
    from oracle import pi_oracle as O
    model = model_c2(picuda)
    plan = O.Plan(to_oracle(model))
    from oracle import cpu_baseline
    ta = cpu_baseline.ThreadedApply(plan)
    n = len(plan)
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(1)
    X = (rng.standard_normal((BATCH, n)) + 1j * rng.standard_normal((BATCH, n))).astype(np.complex128)
    Y = np.empty_like(X)

    def step():
        for c in range(BATCH):
            ta(X[c], Y[c], threads)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    bytes_step = 2 * 16 * n * BATCH
    value = bytes_step * args.steps / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": config_of(n),
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{BATCH} FP64 applies per step x {args.steps} steps, N=120 (C restatement of "
                                   "the reference's output-sector-owned threaded apply, all host threads)"},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def fp64_gemm_tflops(torch, size=4096, reps=5):
    """FP64 throughput of a cuBLAS DGEMM (torch.matmul) on this GPU, measured in this run: the
    denominator of the FP64-pipe fraction of the plain apply."""
    a = torch.randn((size, size), dtype=torch.float64, device="cuda")
    b = torch.randn((size, size), dtype=torch.float64, device="cuda")
    c = a @ b
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(reps):
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2.0 * size ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b, c
    return best


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only-apply", action="store_true",
                    help="time only the device applies (used for ncu captures)")
    ap.add_argument("--layout", default="element-major", choices=["columns", "element-major"],
                    help="batch layout of the headline apply: (batch, dim) columns or (dim, batch)")
    ap.add_argument("--only-solves", action="store_true",
                    help="run only the solve-rate section (used for ncu launch lists)")
    ap.add_argument("--only-scan", action="store_true", help="run only the batched-scan section")
    ap.add_argument("--only-serve", action="store_true", help="run only the serving section")
    ap.add_argument("--scan-instances", type=int, default=256)
    ap.add_argument("--scan-intervals", type=int, default=2)
    ap.add_argument("--scan-precision", default="both", choices=["both", "fp64", "mixed"])
    ap.add_argument("--engine-schedule", default="auto",
                    help="FP32 engine step-apply schedule: auto, per_tile or blocks per SM (an int)")
    ap.add_argument("--serve-requests", type=int, default=24)
    ap.add_argument("--serve-steady-solvers", type=int, default=4,
                    help="preconditioned steady-state solver threads of the served sections (0: in the engine)")
    ap.add_argument("--serve-fp64-rates", type=int, default=1,
                    help="rates of the sweep that also run the plain FP64 server")
    ap.add_argument("--serve-sweep", default=None,
                    help="comma-separated request rates: run only the served rate sweep (e.g. 50,200,1000,2000)")
    ap.add_argument("--only-steady", action="store_true", help="run only the steady-state rate section")
    ap.add_argument("--only-steady-c3", action="store_true",
                    help="run only the N=200 preconditioned steady-state section")
    ap.add_argument("--c3-repeats", type=int, default=5)
    ap.add_argument("--c3-served-per-omega", type=int, default=3,
                    help="concurrent solvers per Omega in the served form of the N=200 section")
    ap.add_argument("--c3-omegas", default="0.5,1,2", help="Omega/kappa values of the N=200 steady-state section")
    ap.add_argument("--c3-no-plain", action="store_true",
                    help="skip the unpreconditioned reference-method attempt (profiling runs)")
    ap.add_argument("--steady-requests", type=int, default=16)
    ap.add_argument("--only-drive-steady", type=int, default=None, metavar="N",
                    help="one strongly driven steady state of N qubits with the drive preconditioner")
    ap.add_argument("--only-rk4", default=None, choices=["fp64", "mixed"],
                    help="one short RK4 solve of the large time-evolution model (a profiling target)")
    ap.add_argument("--only-expv", default=None, choices=["fp64", "mixed"],
                    help="one short expv solve of the large time-evolution model (a profiling target)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch

    import __graft_entry__
    __graft_entry__.build()
    import picuda
    torch.cuda.set_device(local)
    sched = args.engine_schedule
    picuda.set_engine_schedule(int(sched) if sched.lstrip("-").isdigit() else sched)
    if args.only_solves:
        print(json.dumps({"only_solves": True, "solves": solve_rates(picuda, torch)}))
        return 0
    if args.only_scan:
        precs = ("fp64", "mixed") if args.scan_precision == "both" else (args.scan_precision,)
        print(json.dumps({"only_scan": True, "scan": scan_rates(picuda, torch, args.scan_instances,
                                                                  args.scan_intervals, precisions=precs)}))
        return 0
    if args.only_drive_steady:
        print(json.dumps({"only_drive_steady": True,
                          "drive_steady": drive_steady(picuda, torch, N=args.only_drive_steady)}))
        return 0
    if args.only_steady:
        print(json.dumps({"only_steady": True, "steady": steady_rates(picuda, torch, args.steady_requests),
                          "steady_served_family": steady_rates(picuda, torch, args.steady_requests,
                                                               family="served")}))
        return 0
    if args.only_steady_c3:
        omegas = tuple(float(v) for v in args.c3_omegas.split(","))
        print(json.dumps({"only_steady_c3": True,
                          "steady_c3": steady_c3_rates(picuda, torch, omegas=omegas, repeats=args.c3_repeats,
                                                       plain=not args.c3_no_plain,
                                                       served_per_omega=args.c3_served_per_omega)}))
        return 0
    if args.serve_sweep:
        rates = [float(v) for v in args.serve_sweep.split(",")]
        print(json.dumps({"serve_sweep": serve_sweep(picuda, torch, rates, args.serve_requests,
                                                     fp64_rates=args.serve_fp64_rates,
                                                     steady_solvers=args.serve_steady_solvers)}))
        return 0
    if args.only_serve:
        print(json.dumps({"only_serve": True, "serve": serve_rates(picuda, torch, args.serve_requests,
                                                                   steady_solvers=args.serve_steady_solvers)}))
        return 0
    if args.only_expv:
        # two saved intervals of dt = 0.05 (expv m = 30), Jz and J+J- streamed
        sm = picuda.spin_matrices(2)
        c2 = picuda.compile(model_c2(picuda))
        rho0 = picuda.computational_product_state(c2.basis, 2)
        res = picuda.solve_dynamics(c2, rho0, (0.0, 0.1), saveat=0.05, save_states=False,
                                    algorithm=picuda.ExpvAlgorithm(krylovdim=30, precision=args.only_expv),
                                    observables={"Jz": sm["jz"], "JpJm": sm["jp"] @ sm["jm"]})
        print(json.dumps({"only_expv": args.only_expv, "Jz": [float(v.real) for v in res.values["Jz"]]}))
        return 0
    if args.only_rk4:
        # two saved intervals of 0.05 (64 RK4 steps each), Jz and J+J- streamed
        sm = picuda.spin_matrices(2)
        c2 = picuda.compile(model_c2(picuda))
        rho0 = picuda.computational_product_state(c2.basis, 2)
        res = picuda.solve_dynamics(c2, rho0, (0.0, 0.1), saveat=0.05, save_states=False, precision=args.only_rk4,
                                    observables={"Jz": sm["jz"], "JpJm": sm["jp"] @ sm["jm"]})
        print(json.dumps({"only_rk4": args.only_rk4, "Jz": [float(v.real) for v in res.values["Jz"]]}))
        return 0
    model = model_c2(picuda)
    compiled = picuda.compile(model)
    n = len(model.basis)
    g = torch.Generator(device="cuda").manual_seed(1234 + rank)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    peak, peak_kind = measured_peaks()

    # Headline: the plain FP64 apply of 128 columns (pi_apply_f64 on torch's current stream,
    # so the CUDA events on that stream bracket exactly the launches).
    X64 = torch.randn((BATCH, n), dtype=torch.complex128, device="cuda", generator=g)
    Y64 = torch.empty_like(X64)
    for _ in range(args.warmup):
        picuda.apply_(Y64, compiled, X64)
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            picuda.apply_(Y64, compiled, X64)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms64_rank = e0.elapsed_time(e1) / args.steps
    bytes64 = 2 * 16 * n * BATCH
    value, ms64 = replica_throughput(bytes64, ms64_rank, world)
    achieved64 = bytes64 / (ms64_rank * 1e-3) / 1e9
    flops64 = stencil_flops(picuda, model) * BATCH

    # FP32 apply of the mixed-precision path (population coordinates), element-major batch
    # by default; its own roofline.
    em = args.layout == "element-major"
    shape = (n, BATCH) if em else (BATCH, n)
    X32 = torch.randn(shape, dtype=torch.complex64, device="cuda", generator=g)
    Y32 = torch.empty_like(X32)

    def step32():
        if em:
            picuda.apply_element_major_(Y32, compiled, X32, coords="population")
        else:
            picuda.apply_(Y32, compiled, X32, precision="fp32", coords="population")

    for _ in range(max(args.warmup, 3)):
        step32()  # the first element-major call autotunes the kernel choice for this width
    torch.cuda.synchronize()
    em_choice = picuda.element_major_tuning(compiled, BATCH) if em else None
    barrier(world)
    k32 = max(args.steps, 20)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(k32):
        step32()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms32 = e0.elapsed_time(e1) / k32
    bytes32 = 2 * 8 * n * BATCH
    value32, ms32 = replica_throughput(bytes32, ms32, world)
    achieved32 = bytes32 / (ms32 * 1e-3) / 1e9

    if args.only_apply:
        if rank == 0:
            print(json.dumps({"only_apply": True, "ms_fp64": ms64, "gbs_fp64": achieved64, "ms_fp32": ms32,
                              "gbs_fp32": achieved32, "kernel": em_choice}))
        return 0

    dgemm = fp64_gemm_tflops(torch) if rank == 0 else None
    lib = picuda.load_library()
    import ctypes as C
    # End to end through the host-buffer C-ABI call, FP64: pinned host columns, H2D + apply +
    # D2H inside the timed region, every step.
    xh64 = X64.cpu().pin_memory()
    yh64 = torch.empty_like(xh64).pin_memory()
    del X64, Y64
    for _ in range(2):
        lib.pi_apply_host_f64(compiled.handle, C.c_void_p(yh64.data_ptr()), C.c_void_p(xh64.data_ptr()), BATCH)
    k_e2e = max(3, args.steps // 5)
    t0 = time.perf_counter()
    for _ in range(k_e2e):
        rc = lib.pi_apply_host_f64(compiled.handle, C.c_void_p(yh64.data_ptr()), C.c_void_p(xh64.data_ptr()),
                                   BATCH)
        if rc != 0:
            raise RuntimeError(picuda._lib.last_error())
    e2e_s = (time.perf_counter() - t0) / k_e2e
    e2e_s = max_over_ranks(e2e_s, world)
    e2e_value = world * bytes64 / e2e_s / 1e9
    del xh64, yh64
    # The same for the FP32 apply (pi_apply_host_f32, columns, population coordinates).
    xh = (X32.t().contiguous() if em else X32).cpu().pin_memory()
    yh = torch.empty_like(xh).pin_memory()
    for _ in range(2):
        lib.pi_apply_host_f32(compiled.handle, C.c_void_p(yh.data_ptr()), C.c_void_p(xh.data_ptr()), BATCH, 1)
    t0 = time.perf_counter()
    for _ in range(k_e2e):
        rc = lib.pi_apply_host_f32(compiled.handle, C.c_void_p(yh.data_ptr()), C.c_void_p(xh.data_ptr()), BATCH, 1)
        if rc != 0:
            raise RuntimeError(picuda._lib.last_error())
    e2e32_s = max_over_ranks((time.perf_counter() - t0) / k_e2e, world)
    del xh, yh, X32, Y32

    solves = solve_rates(picuda, torch) if rank == 0 else None
    scan = scan_rates(picuda, torch, args.scan_instances, args.scan_intervals) if rank == 0 else None
    serve = serve_rates(picuda, torch, args.serve_requests,
                        steady_solvers=args.serve_steady_solvers) if rank == 0 else None
    steady = steady_rates(picuda, torch, args.steady_requests) if rank == 0 else None
    steady_served = (steady_rates(picuda, torch, args.steady_requests, family="served")
                     if rank == 0 else None)
    steady_c3 = steady_c3_rates(picuda, torch, repeats=args.c3_repeats) if rank == 0 else None
    drive = drive_steady(picuda, torch, N=100, repeats=2) if rank == 0 else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import pi_oracle as O
        gbs, threads, count, dt = cpu_baseline_apply(O.Plan(to_oracle(model)), n)
        cpu = {"value": gbs, "unit": "GB/s", "cores": threads, "kind": "port",
               "sample": f"{count} FP64 applies of one N=120 state vector in {dt:.1f} s "
                         "(C restatement of the reference's sector-owned threaded apply)"}

    if rank == 0:
        cl = clocks.summary()
        line = {
            "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms64, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": config_of(n),
            "call": "pi_apply_f64 (k_apply_canon<double>: canonical-position register kernel)",
            "parallelism": "replicas" if world > 1 else "single GPU",
            "roofline": {"bound": "hbm", "achieved": achieved64, "peak": peak, "unit": "GB/s",
                         "frac": achieved64 / peak, "peak_kind": peak_kind,
                         "traffic": profile_traffic("apply_f64_batch128_N120"),
                         "algorithmic_bytes_per_launch": bytes64,
                         "fp64_pipe": {"achieved_tflops": flops64 / (ms64_rank * 1e-3) / 1e12,
                                       "peak_tflops": dgemm,
                                       "frac": (flops64 / (ms64_rank * 1e-3) / 1e12 / dgemm) if dgemm else None,
                                       "peak_kind": "cuBLAS DGEMM 4096^3 measured in this run",
                                       "algorithmic_flops_per_launch": flops64,
                                       "note": "the FP64 apply is bound by GB300's FP64 pipe, not by HBM"}},
            "e2e": {"value": e2e_value, "unit": "GB/s", "h2d_bytes_per_step": 16 * n * BATCH,
                    "d2h_bytes_per_step": 16 * n * BATCH, "ms_per_step": e2e_s * 1e3,
                    "call": "pi_apply_host_f64 (pinned host columns; copies and apply pipelined over three streams)"},
            "fp32": {"value": value32, "unit": "GB/s", "ms_per_step": ms32, "steps": k32,
                     "workload": "the same L x and batch in complex FP32, population coordinates (the operator of "
                                 "the mixed-precision solvers)",
                     "layout": ("element-major (dim, 128): pi_apply_f32_em" if em else "columns (128, dim): pi_apply_f32"),
                     "kernel": em_choice,
                     "roofline": {"bound": "hbm", "achieved": achieved32, "peak": peak, "unit": "GB/s",
                                  "frac": achieved32 / peak, "peak_kind": peak_kind,
                                  "traffic": profile_traffic("apply_em_f32_batch128_N120" if em else
                                                             "apply_f32_batch128_N120"),
                                  "algorithmic_bytes_per_launch": bytes32},
                     "e2e": {"value": world * bytes32 / e2e32_s / 1e9, "unit": "GB/s",
                             "h2d_bytes_per_step": 8 * n * BATCH, "d2h_bytes_per_step": 8 * n * BATCH,
                             "ms_per_step": e2e32_s * 1e3, "call": "pi_apply_host_f32 (pinned host buffers)"}},
            "solves": solves,
            "scan": scan,
            "serve": serve,
            "steady": steady,
            "steady_served_family": steady_served,
            "steady_c3": steady_c3,
            "drive_steady": drive,
            "cpu_baseline": cpu,
            "gpu_launches": args.steps,
            "clocks": cl,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
