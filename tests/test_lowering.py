"""Host-side lowering in libpicuda (no GPU): exported symbols, stencil tables, basis maps,
collective blocks and error behaviour, all checked against the oracle."""
import math
import re
from pathlib import Path

import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from tests import models as M
from tests.stencil_eval import evaluate

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    picuda.load_library()


def test_library_exports_every_declared_symbol():
    header = (ROOT / "include" / "picuda.h").read_text()
    declared = sorted(set(re.findall(r"\b(?:int|void)\s+(pi_[a-z0-9_]+)\s*\(", header)))
    assert len(declared) >= 20
    lib = picuda.load_library()
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing
    from picuda import _lib
    assert set(declared) == set(_lib.PROTOTYPES), "ctypes prototypes must match the header"


CASES = [
    ("driven_c1_N8", lambda: M.driven_c1(8)),
    ("ensemble_c2_N9", lambda: M.ensemble_c2(9)),
    ("btc_c3_N10", lambda: M.btc_c3(10, 2.0)),
    ("general_N1", lambda: M.general(1, 1)),
    ("general_N2", lambda: M.general(2, 2)),
    ("general_N5", lambda: M.general(5, 3)),
    ("general_N6", lambda: M.general(6, 4)),
    ("general_N7_restricted", lambda: M.general(7, 5, sectors=[(7, 0), (5, 2)])),
    ("general_N8_gap", lambda: M.general(8, 6, sectors=[(8, 0), (6, 2), (4, 4)])),
    ("btc_symmetric_only", lambda: picuda.Models.boundary_time_crystal(9, omega=1.5, kappa=1.0)),
    ("pump_decay_N6", lambda: picuda.Models.local_pump_decay(6, down=1.0, up=0.3)),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_stencil_matches_oracle_apply(name, make):
    model = make()
    table, coef = picuda.stencil_tables(model)
    oplan = O.Plan(M.to_oracle(model))
    for seed in range(3):
        x = M.random_state_vector(len(model.basis), seed)
        y_ref = O.apply(oplan, x)
        y = evaluate(model.basis, table, coef, x)
        scale = np.abs(y_ref).max()
        assert np.abs(y - y_ref).max() <= 1e-13 * scale, name


def test_stencil_term_counts_c2_shape():
    """H tridiagonal, diagonal losses, one collective and two local channels: 14 terms in a
    generic interior sector (ADD + 2 LEFT + 2 RIGHT + 1 collective + 4 + 4 one-body)."""
    model = M.ensemble_c2(12)
    table, _ = picuda.stencil_tables(model)
    counts = np.bincount(table[:, 0])
    assert counts.max() == 14
    # hamiltonian-only off-diagonals are purely imaginary: class 1
    left = table[(table[:, 2] == 1)]
    assert set(left[:, 3]) == {1}


def test_basis_maps_bit_exact():
    for N in (1, 2, 7, 8, 120, 301):
        b = picuda.PIBasis(N, 2)
        ob = O.PIBasis(N, 2) if N <= 120 else None
        assert len(b) == math.comb(N + 3, 3)
        assert b.sectors == [(N - k, k) for k in range(N // 2 + 1)]
        if ob is not None:
            assert b.sectors == ob.sectors
            assert b.offsets == ob.offsets
            assert [[tuple(p) for p in pats] for pats in b.patterns] == ob.patterns


def test_multiplicities_and_trace_functional():
    for N in (4, 9, 60, 200, 300):
        b = picuda.PIBasis(N, 2)
        scales = b.multiplicity_scales()
        for s, p in enumerate(b.sectors):
            f = O.symmetric_group_dimension(p)
            assert scales[s] == math.sqrt(float(f))
    b = picuda.PIBasis(8, 2)
    idx, val = b.trace_functional()
    oidx, oval = O.trace_functional(O.PIBasis(8, 2))
    assert np.array_equal(idx, oidx) and np.array_equal(val, oval)


def test_collective_blocks_match_oracle():
    rng = np.random.default_rng(7)
    X = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    for N in (1, 4, 9):
        ob = O.PIBasis(N, 2)
        g = O.OneBodyGeometry(ob)
        op = picuda.collective_operator(picuda.PIBasis(N, 2), X)
        ref = O.collective_operator(ob, X, g)
        assert np.abs(op.data - ref).max() <= 1e-14 * np.abs(ref).max()


def test_unsupported_models_raise_argument_errors():
    with pytest.raises(picuda.PiArgumentError):
        picuda.PIBasis(4, 3)
    s = picuda.spin_matrices(2)
    with pytest.raises(picuda.PiArgumentError):
        picuda.CollectiveHamiltonian(s["jm"])  # non-Hermitian Hamiltonian
    with pytest.raises(picuda.PiArgumentError):
        picuda.LocalJump(np.eye(3))
    with pytest.raises(picuda.PiArgumentError):
        picuda.PIBasis(4, 2, sectors=[(3, 1), (3, 1)])
    with pytest.raises(picuda.PiArgumentError):
        picuda.PIBasis(4, 2, sectors=[(2, 1)])
    with pytest.raises(picuda.PiArgumentError):
        picuda.PIModel(picuda.PIBasis(3), [object()])
    # non-finite operators are rejected by the native lowering
    bad = picuda.PIModel(picuda.PIBasis(3), [picuda.LocalJump(np.array([[np.nan, 0], [0, 0]]))])
    with pytest.raises(picuda.PiArgumentError):
        picuda.stencil_tables(bad)


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_adjoint_stencil_is_the_conjugate_transpose(name, make):
    """The adjoint plan's stencil (pi_stencil_export_adjoint) applies the conjugate
    transpose of the oracle's PI-coordinate matrix (apply_adjoint!, liouvillian.jl:3275)."""
    model = make()
    table, coef = picuda.stencil_tables(model, adjoint=True)
    LH = O.adjoint_matrix(O.Plan(M.to_oracle(model)))
    for seed in range(2):
        x = M.random_state_vector(len(model.basis), seed)
        y_ref = LH @ x
        y = evaluate(model.basis, table, coef, x)
        assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max(), name


def test_element_major_entry_points_reject_null_arguments():
    """The element-major apply and its tuning entry points validate arguments on the host
    before any device work."""
    import ctypes as C

    from picuda import _lib
    lib = picuda.load_library()
    kind, rows, ms = C.c_int(), C.c_int(), C.c_double()
    assert lib.pi_apply_f32_em_tuning(None, 128, 1, C.byref(kind), C.byref(rows), C.byref(ms)) == \
        _lib.PI_ERR_INVALID_ARGUMENT
    assert lib.pi_apply_f32_em_select(None, 128, 1, 0, 32) == _lib.PI_ERR_INVALID_ARGUMENT
    assert lib.pi_apply_f32_em(None, None, None, 128, 128, 1, None) == _lib.PI_ERR_INVALID_ARGUMENT
    assert "null" in _lib.last_error()


def test_element_major_kernel_choice_validates_names():
    with pytest.raises(picuda.PiArgumentError):
        picuda.select_element_major_kernel(object(), 128, "fastest")
    with pytest.raises(picuda.PiArgumentError):
        picuda.select_element_major_kernel(object(), 128, "tma", 32, coords="spherical")
