"""Adjoint apply (apply_adjoint!) and Arnoldi spectra (krylov_liouvillian_spectrum) on the
GPU against the oracle's conjugate transpose, dense spectrum and Arnoldi restatement."""
import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from tests import models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


CASES = [("driven8", lambda: M.driven_c1(8)), ("general6", lambda: M.general(6, seed=4)),
         ("restricted7", lambda: M.general(7, 5, sectors=[(7, 0), (5, 2)])),
         ("pump_decay6", lambda: picuda.Models.local_pump_decay(6, down=1.0, up=0.3))]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_adjoint_apply_matches_oracle(torch_cuda, name, make):
    torch = torch_cuda
    model = make()
    c = picuda.compile(model)
    LH = O.adjoint_matrix(O.Plan(M.to_oracle(model)))
    X = np.stack([M.random_state_vector(len(model.basis), s) for s in range(3)])
    xd = torch.from_numpy(X).cuda()
    yd = torch.empty_like(xd)
    picuda.apply_adjoint_(yd[0], c, xd[0])
    picuda.apply_adjoint_(yd, c, xd)  # three columns: the batched kernels on the adjoint plan
    torch.cuda.synchronize()
    Y = yd.cpu().numpy()
    for j in range(3):
        ref = LH @ X[j]
        assert np.abs(Y[j] - ref).max() <= 1e-12 * np.abs(ref).max(), (name, j)


def test_adjoint_duality_and_trace_at_scale(torch_cuda):
    """<y, L x> = <L^H y, x> and L^H t = 0 for the trace functional t
    (test_liouvillian_properties.jl:139-168) at N = 60."""
    torch = torch_cuda
    model = M.ensemble_c2(60)
    c = picuda.compile(model)
    n = len(model.basis)
    x = torch.from_numpy(M.random_state_vector(n, 1)).cuda()
    y = torch.from_numpy(M.random_state_vector(n, 2)).cuda()
    Lx, LHy = torch.empty_like(x), torch.empty_like(y)
    picuda.apply_(Lx, c, x)
    picuda.apply_adjoint_(LHy, c, y)
    lhs = complex(torch.vdot(y, Lx).item())
    rhs = complex(torch.vdot(LHy, x).item())
    assert abs(lhs - rhs) <= 1e-12 * float(torch.linalg.norm(Lx)) * float(torch.linalg.norm(y))
    idx, val = c.library_trace_functional()
    t = np.zeros(n, dtype=np.complex128)
    t[idx] = val
    td = torch.from_numpy(t).cuda()
    out = torch.empty_like(td)
    picuda.apply_adjoint_(out, c, td)
    # t holds sqrt(f) (up to ~1e8 at N = 60): measure against |t| times the operator's scale
    op_scale = float(LHy.abs().max()) / float(y.abs().max())
    assert float(out.abs().max()) <= 1e-12 * float(np.abs(t).max()) * op_scale


@pytest.mark.parametrize("N", [4, 6])
def test_spectrum_matches_dense_with_full_krylov_space(torch_cuda, N):
    """test/test_krylov.jl:131-136 on the GPU."""
    model = M.general(N, seed=2)
    plan = O.Plan(M.to_oracle(model))
    L = O.materialize(plan)
    n = L.shape[0]
    dense = np.linalg.eigvals(L)
    dense = dense[O.ritz_order(dense, "LR")]
    arn = picuda.krylov_liouvillian_spectrum(model, nev=4, krylovdim=n, vectors=True,
                                             rng=np.random.default_rng(7))
    canon = lambda v: v[np.lexsort((np.round(v.imag, 8), np.round(v.real, 8)))]
    assert np.allclose(canon(arn["values"]), canon(dense[:4]), atol=2e-10, rtol=0)
    assert arn["residuals"].max() < 2e-10 and arn["converged"].all()
    Vv = arn["vectors"]
    assert np.linalg.norm(L @ Vv - Vv * arn["values"][None, :]) < 2e-9


def test_spectrum_agrees_with_oracle_arnoldi_and_rejects_bad_input(torch_cuda):
    """Same initial vector, partial Krylov space: the converged leading Ritz values agree
    with the oracle's restatement; argument errors follow krylov.jl:920-933."""
    model = M.driven_c1(8)
    oplan = O.Plan(M.to_oracle(model))
    n = len(model.basis)
    v0 = M.random_state_vector(n, 11)
    kw = dict(nev=3, krylovdim=60, initial_vector=v0, require_convergence=False)
    ref = O.krylov_liouvillian_spectrum(lambda v: O.apply(oplan, v), n, **kw)
    got = picuda.krylov_liouvillian_spectrum(model, **kw)
    assert got["iterations"] == ref["iterations"] == 60
    for v, r in zip(got["values"], got["residuals"]):
        if r <= 1e-9:
            assert np.min(np.abs(ref["values"] - v)) <= 1e-8 * max(1.0, abs(v))
    with pytest.raises(picuda.PiArgumentError):
        picuda.krylov_liouvillian_spectrum(model, nev=0)
    with pytest.raises(picuda.PiArgumentError):
        picuda.krylov_liouvillian_spectrum(model, which="XX")
    with pytest.raises(picuda.PiArgumentError):
        picuda.krylov_liouvillian_spectrum(model, initial_vector=np.zeros(n))
