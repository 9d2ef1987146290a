"""The benchmarked kernels at the benchmarked shape against the oracle.

The bench's headline is the plain FP64 apply of the N=120 ensemble (H = 0.3 Jz + 1.2 Jx,
local decay 0.2, local dephasing 0.1, collective decay 0.05/N; dim 302,621) to 128 columns
(pi_apply_f64 -> the canonical-position register kernel); its `fp32` key is the element-major
FP32 apply of the same 128 vectors in population coordinates (the TMA-staged kernel with
64-row tiles, the autotuner's choice on that batch).  Each is checked column by column
against the oracle's apply on a sample of eight columns, in the coordinates it runs in."""
import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from tests import models as M

pytestmark = pytest.mark.gpu

TOL_F64 = 1e-12
TOL_F32 = 2e-6
COLS = [0, 17, 34, 51, 68, 85, 102, 127]


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def c2(torch_cuda):
    model = M.ensemble_c2(120)
    return model, picuda.compile(model), O.Plan(M.to_oracle(model))


def test_fp64_headline_shape_matches_oracle(torch_cuda, c2):
    torch = torch_cuda
    model, compiled, oplan = c2
    assert compiled.info["batched_kernel"] == 2  # canonical positions: k_apply_canon<double>
    n = len(model.basis)
    g = torch.Generator(device="cuda").manual_seed(1234)
    X = torch.randn((128, n), dtype=torch.complex128, device="cuda", generator=g)
    Y = torch.full_like(X, complex(np.nan, np.nan))
    picuda.apply_(Y, compiled, X)
    torch.cuda.synchronize()
    for c in COLS:
        x = X[c].cpu().numpy()
        ref = O.apply(oplan, x)
        got = Y[c].cpu().numpy()
        assert np.abs(got - ref).max() <= TOL_F64 * np.abs(ref).max(), c


def test_fp32_element_major_tma_shape_matches_oracle(torch_cuda, c2):
    torch = torch_cuda
    model, compiled, oplan = c2
    n = len(model.basis)
    b = model.basis
    sq = compiled.sector_scales()
    S = np.concatenate([np.full(m * m, sq[i]) for i, m in enumerate(b.dims)])  # z = S x
    g = torch.Generator(device="cuda").manual_seed(4321)
    Z = torch.randn((n, 128), dtype=torch.complex64, device="cuda", generator=g)
    picuda.select_element_major_kernel(compiled, 128, "tma", 64)
    Y = torch.full_like(Z, complex(np.nan, np.nan))
    picuda.apply_element_major_(Y, compiled, Z, coords="population")
    torch.cuda.synchronize()
    for c in COLS:
        z = Z[:, c].cpu().numpy().astype(np.complex128)
        ref = S * O.apply(oplan, z / S)  # the operator in population coordinates
        got = Y[:, c].cpu().numpy().astype(np.complex128)
        assert np.abs(got - ref).max() <= TOL_F32 * np.abs(ref).max(), c
