"""Generates the golden fixtures in this directory from the CPU oracle.

The reference (Julia) cannot run in this environment, so fixtures come from the oracle
restatement, which tests/test_oracle_pins.py pins to the reference's own analytic and
structural known answers.  Inputs are seeded; rerun with
    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import pi_oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def driven_c1():
    """Driven qubits N=8: H = 1.0 Jx, local decay 0.5, no pumping (model_zoo.jl:214-242)."""
    return O.driven_qubits(8, drive=1.0, emission=0.5, pumping=0.0)


def ensemble_c2(N=120):
    """The large time-evolution configuration: H = 0.3 Jz + 1.2 Jx, local decay 0.2, local
    dephasing 0.1, collective decay 0.05/N on J-."""
    s = O.spin_matrices(2)
    return O.qubit_ensemble_model(N, hamiltonian=0.3 * s["jz"] + 1.2 * s["jx"], emission=0.2, dephasing=0.1,
                                  collective_emission=0.05 / N)


def c2_dynamics(nint=20):
    """Oracle FP64 expv dynamics of the N=120 configuration from the all-excited state: saved
    every dt = 0.05 for nint intervals (m = 30, atol 1e-10, rtol 1e-8), observables Jz and
    J+J- (the references for the mixed and FP64 GPU paths)."""
    plan = O.Plan(ensemble_c2(120))
    b = plan.basis
    s = O.spin_matrices(2)
    obs = {"Jz": O.collective_operator(b, s["jz"]), "JpJm": O.collective_operator(b, s["jp"] @ s["jm"])}
    rho0 = O.computational_product_state(b, 2)
    dyn = O.solve_dynamics_expv(plan, rho0, (0.0, 0.05 * nint), saveat=0.05, observables=obs, save_states=False)
    np.savez_compressed(OUT / "ensemble_c2_N120_expv.npz", t=np.array(dyn["t"]), Jz=dyn["values"]["Jz"],
                        JpJm=dyn["values"]["JpJm"])


def main():
    c2_dynamics()
    rng = np.random.default_rng(20261203)
    plan = O.Plan(driven_c1())
    b = plan.basis
    n = len(plan)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
    y = O.apply(plan, x)
    ss, info = O.krylov_steady_state(plan, operator_scale=2.0)
    rho0 = O.computational_product_state(b, 2)
    s = O.spin_matrices(2)
    obs = {"excited": O.collective_operator(b, s["jp"] @ s["jm"]), "Jz": O.collective_operator(b, s["jz"])}
    dyn = O.solve_dynamics_expv(plan, rho0, (0.0, 4.0), saveat=0.1, observables=obs, save_states=False)
    np.savez_compressed(
        OUT / "driven_qubits_N8.npz",
        x=x, Lx=y, steady=ss, steady_operator_scale=2.0, t=np.array(dyn["t"]),
        excited=dyn["values"]["excited"], Jz=dyn["values"]["Jz"],
        offsets=np.array(b.offsets), dims=np.array(b.dims),
        trace_idx=plan.trace_idx, trace_val=plan.trace_val.real)
    # Two-row hook dimensions f^(N-k, k) for the configured sizes (exact integers).
    with open(OUT / "multiplicities.txt", "w") as f:
        f.write("# N k f^(N-k,k)  (exact, from the hook-length formula)\n")
        for N in (8, 120, 200, 300):
            for k in range(N // 2 + 1):
                f.write(f"{N} {k} {O.symmetric_group_dimension((N - k, k))}\n")
    print("wrote fixtures to", OUT)


if __name__ == "__main__":
    main()
