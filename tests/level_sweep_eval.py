"""Numpy evaluation of the level-sweep preconditioner tables exported by libpicuda
(pi_precond_export) -- test helper only.  Runs the same sweep as the device kernel in FP64:
per charge chain, per level in sweep order, right-hand sides s (r - alpha v) minus the gains
from the previous level, then the forward and backward Thomas recurrences."""
import numpy as np

NO_GAIN = 1023


def sweep(T, r, s):
    r = np.asarray(r, dtype=np.complex128)
    z = np.zeros_like(r)
    chain_lev, lev_ent, elem = T["chain_lev"], T["lev_ent"], T["elem"]
    c0, c0e, mode = T["chain0"], T["chain0_ent"], T["mode"]
    for c in range(len(chain_lev) - 1):
        lev0, lev1 = chain_lev[c], chain_lev[c + 1]
        is0 = c == c0
        end0 = lev_ent[lev1]
        uprev = None
        rho_r = 0.0
        for lev in range(lev0, lev1):
            e0, e1 = lev_ent[lev], lev_ent[lev + 1]
            rhs = s * r[elem[e0:e1]]
            for i in range(e1 - e0):
                e = e0 + i
                for k in range(3):
                    pos = (int(T["gsrc"][e]) >> (10 * k)) & 1023
                    if pos != NO_GAIN:
                        rhs[i] -= T["G"][3 * e + k] * uprev[pos]
                if e == T["free_ent"]:
                    rho_r = rhs[i]
            y = T["W"][e0:e1] * rhs
            for i in range(1, e1 - e0):
                y[i] += T["A"][e0 + i] * y[i - 1]
            u = np.zeros_like(y)
            u[-1] = y[-1]
            for i in range(e1 - e0 - 2, -1, -1):
                u[i] = y[i] + T["C"][e0 + i] * u[i + 1]
            z[elem[e0:e1]] = u
            uprev = u
        if is0:
            idx = elem[c0e:end0]
            if mode == 0:
                # beta = rho_r / rho_v; y = y_r - beta y_v; z_f = (beta - t^H y) / t_f
                beta = rho_r / T["sm_coef"]
                z[idx] -= beta * T["w0"]
                f = T["free_ent"]
                z[elem[f]] = (beta - np.dot(T["t0"], z[idx])) / T["t0"][f - c0e]
            else:
                z[idx] -= T["w0"] * (np.dot(T["t0"], z[idx]) * T["sm_coef"])
    return z
