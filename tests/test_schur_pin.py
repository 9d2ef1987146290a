"""The PI coordinates pinned to the full 2^N Lindbladian through the reference's dense Schur
oracle (test/test_dense_schur_reference.jl:5-23, restated in oracle/schur_reference.py).

The reference test's own assertions hold for the restated transform S: it is orthogonal,
and S rho S^T of iid states and collective observables is block diagonal with the PI blocks.
Then the library's lowered Liouvillian (its exported stencil tables, evaluated on unit
vectors) and its adjoint must equal Psi o L_full o Phi and its conjugate transpose for every
supported term kind, block by block, to 1e-12: this fixes sector order, GT order,
column-major blocks, the sqrt(f) scale and the CG signs independently of the oracle's own
lowering."""
import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from oracle import schur_reference as SR
from tests import models as M
from tests.stencil_eval import evaluate


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    picuda.load_library()


@pytest.mark.parametrize("N", [3, 4, 5, 6])
def test_schur_transform_matches_reference_assertions(N):
    S, labels = SR.dense_schur_reference(N, 2)
    assert S.shape == (2 ** N, 2 ** N)
    assert np.abs(S @ S.T - np.eye(2 ** N)).max() <= 2e-13
    b = O.PIBasis(N, 2)
    maps = SR.SchurMaps(b)
    psi = np.array([0.6, 0.8j])
    v = np.ones(1, dtype=np.complex128)
    for _ in range(N):
        v = np.kron(v, psi)
    rho = np.outer(v, v.conj())
    assert np.abs(maps.psi(rho) - O.iid_pure_state(b, psi)).max() <= 3e-13
    assert maps.offblock_norm(rho) <= 5e-13
    for X in (np.diag([0.0, 1.0]), np.array([[0.0, 0.2 + 0.1j], [0.2 - 0.1j, 0.0]])):
        full = SR.collective_sum(X, N, 2)
        assert np.abs(maps.psi(full) - O.collective_operator(b, X)).max() <= 3e-13 * N
        assert maps.offblock_norm(full) <= 5e-13 * N


def library_dense(model, adjoint=False):
    table, coef = picuda.stencil_tables(model, adjoint=adjoint)
    n = len(model.basis)
    L = np.zeros((n, n), dtype=np.complex128)
    e = np.zeros(n, dtype=np.complex128)
    for k in range(n):
        e[k] = 1.0
        L[:, k] = evaluate(model.basis, table, coef, e)
        e[k] = 0.0
    return L


CASES = [
    ("driven_N5", lambda: M.driven_c1(5)),
    ("ensemble_N6", lambda: M.ensemble_c2(6)),
    ("btc_N6", lambda: M.btc_c3(6, 1.0)),
    ("scan_N5", lambda: M.scan_model(5, 1.3, 0.2, 0.1)),
    ("pump_decay_N4", lambda: picuda.Models.local_pump_decay(4, down=1.0, up=0.3)),
    ("general_N4", lambda: M.general(4, 2)),
    ("general_N5", lambda: M.general(5, 3)),
    ("general_N6_restricted", lambda: M.general(6, 4, sectors=[(6, 0), (5, 1), (4, 2)])),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_library_liouvillian_equals_full_space_conjugation(name, make):
    model = make()
    omodel = M.to_oracle(model)
    maps = SR.SchurMaps(omodel.basis)
    ref = maps.liouvillian(omodel)
    scale = np.abs(ref).max()
    L = library_dense(model)
    b = model.basis
    for s, (o, n) in enumerate(zip(b.offsets, b.dims)):
        for t, (o2, n2) in enumerate(zip(b.offsets, b.dims)):
            blk = L[o:o + n * n, o2:o2 + n2 * n2]
            rblk = ref[o:o + n * n, o2:o2 + n2 * n2]
            assert np.abs(blk - rblk).max() <= 1e-12 * scale, (name, s, t)
    LH = library_dense(model, adjoint=True)
    assert np.abs(LH - ref.conj().T).max() <= 1e-12 * scale
