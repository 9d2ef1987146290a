"""The level-sweep preconditioner's host construction (pi_precond_export, no GPU).

The exported tables, swept in numpy exactly as the device kernel sweeps them, must invert
M = L0/s + v t^H, where L0 keeps the charge-preserving stencil terms of the library's own
lowering (dr == dc) and v, t are the trace border in the chosen coordinates; the element
maps must cover the basis once."""
import numpy as np
import pytest

import picuda
from tests import models as M
from tests.level_sweep_eval import sweep
from tests.stencil_eval import _shifted


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    picuda.load_library()


def dense_L0(model, coords):
    """L0 (charge-keeping terms only) as a dense matrix in the given coordinates."""
    table, coef = picuda.stencil_tables(model)
    b = model.basis
    n = len(b)
    L = np.zeros((n, n), dtype=np.complex128)
    for col in range(n):
        x = np.zeros(n, dtype=np.complex128)
        x[col] = 1.0
        blocks = [x[o:o + m * m].reshape((m, m), order="F") for o, m in zip(b.offsets, b.dims)]
        out = [np.zeros((m, m), dtype=np.complex128) for m in b.dims]
        for (s, src, kind, cls, dr, dc, ao, bo) in table:
            if dr != dc:
                continue
            m = b.dims[s]
            Z = _shifted(blocks[src], dr, dc, m)
            al = coef[ao:ao + m] if ao >= 0 else None
            be = coef[bo:bo + m] if bo >= 0 else None
            if kind == 0:
                out[s] += (al[:, None] + be[None, :]) * Z
            elif kind == 1:
                out[s] += al[:, None] * Z
            elif kind == 2:
                out[s] += be[None, :] * Z
            else:
                out[s] += (al[:, None] * be[None, :]) * Z
        L[:, col] = np.concatenate([o.reshape(-1, order="F") for o in out])
    return L


def border(model, coords):
    b = model.basis
    lib = picuda.load_library()
    n = len(b)
    t = np.zeros(n)
    fvals = []
    for s, (o, m) in enumerate(zip(b.offsets, b.dims)):
        f = np.zeros(1)
        sf = np.zeros(1)
        lib.pi_sector_multiplicity(b.N, b.sectors[s][1], picuda._lib.dptr(f), picuda._lib.dptr(sf))
        fvals.append((f[0], sf[0], o, m))
    norm2 = sum(m * f for f, _, _, m in fvals)
    v = np.zeros(n)
    S = np.ones(n)
    for f, sf, o, m in fvals:
        idx = o + np.arange(m) * (m + 1)
        t[idx] = 1.0 if coords == "population" else sf
        v[idx] = f / norm2 if coords == "population" else sf / norm2
        S[o:o + m * m] = sf
    return t, v, S


CASES = [
    ("btc_N6", lambda: M.btc_c3(6, 1.0)),
    ("btc_N9", lambda: M.btc_c3(9, 2.0)),
    ("btc_N12", lambda: M.btc_c3(12, 0.5)),
    ("ensemble_N8", lambda: M.ensemble_c2(8)),
    ("driven_N7", lambda: M.driven_c1(7)),
    ("scan_N10", lambda: M.scan_model(10, 1.3, 0.2, 0.1)),
    ("btc_restricted", lambda: picuda.qubit_ensemble_model(
        picuda.PIBasis(10, 2, sectors=[(10, 0), (9, 1), (7, 3)]),
        hamiltonian=0.02 * picuda.spin_matrices(2)["jx"], collective_emission=0.1, dephasing=0.01)),
]


@pytest.mark.parametrize("coords", ["population", "reference"])
@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_sweep_inverts_bordered_charge_keeping_part(name, make, coords):
    model = make()
    n = len(model.basis)
    s = 0.7
    T = picuda.level_preconditioner_tables(model, coords=coords, operator_scale=s)
    assert np.array_equal(np.sort(T["elem"]), np.arange(n)), "every PI coordinate appears once"
    L0 = dense_L0(model, coords)
    t, v, S = border(model, coords)
    if coords == "population":
        L0 = (S[:, None] * L0) / S[None, :]
    Mb = L0 / s + np.outer(v, t)
    rng = np.random.default_rng(3)
    for _ in range(2):
        r = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        z = sweep(T, r, s)
        ref = np.linalg.solve(Mb, r)
        assert np.abs(z - ref).max() <= 1e-9 * np.abs(ref).max(), (name, coords, np.abs(z - ref).max())
        assert np.abs(Mb @ z - r).max() <= 1e-9 * np.abs(r).max()


def test_decay_models_have_one_free_dark_entry():
    """The all-down population is L0's only null direction for decay-type models: the
    singular mode, whose free entry is the last of the d = 0 chain, at the last diagonal
    element of the symmetric sector (GT order puts M = -N/2 last)."""
    model = M.btc_c3(12, 1.0)
    T = picuda.level_preconditioner_tables(model, operator_scale=1.0)
    assert T["mode"] == 0 and T["direction"] == -1
    assert T["free_ent"] == T["lev_ent"][T["chain_lev"][T["chain0"] + 1]] - 1
    n0 = model.basis.dims[0]
    assert T["elem"][T["free_ent"]] == n0 * n0 - 1


def test_models_with_decay_and_pumping_are_rejected():
    with pytest.raises(picuda.PiArgumentError, match="raise, or all to lower"):
        picuda.level_preconditioner_tables(picuda.Models.local_pump_decay(6, down=1.0, up=0.3), operator_scale=1.0)


def test_pumping_only_sweeps_upward():
    spin = picuda.spin_matrices(2)
    model = picuda.qubit_ensemble_model(8, hamiltonian=0.3 * spin["jx"], pumping=0.4, dephasing=0.05)
    T = picuda.level_preconditioner_tables(model, operator_scale=1.0)
    assert T["direction"] == 1


def test_chain_and_level_counts_at_N200():
    model = M.btc_c3(200, 1.0)
    T = picuda.level_preconditioner_tables(model, operator_scale=1.0)
    assert len(T["chain_lev"]) - 1 == 2 * 201 - 1
    assert T["max_level"] == 101
    assert len(T["t0"]) == sum(model.basis.dims)
    assert T["mode"] == 0
