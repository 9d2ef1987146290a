"""GPU parity of the fused Schur-block apply (libpicuda, sm_103a) against the oracle."""
import numpy as np
import pytest

import picuda
from oracle import pi_oracle as O
from tests import models as M

pytestmark = pytest.mark.gpu

# Plain FP64 path: relative error bound against the oracle (max |dy| / max |y|).
TOL_F64 = 1e-12
# FP32 apply: FP32 rounding of ~15 accumulated terms.
TOL_F32 = 2e-6


@pytest.fixture(scope="module")
def torch_cuda(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _dev(torch, a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return t if dtype is None else t.to(dtype)


def _apply64(torch, compiled, x):
    xd = _dev(torch, x)
    yd = torch.empty_like(xd)
    picuda.apply_(yd, compiled, xd)
    torch.cuda.synchronize()
    return yd.cpu().numpy()


CASES = [
    ("driven_c1_N8", lambda: M.driven_c1(8)),
    ("general_N1", lambda: M.general(1, 1)),
    ("general_N6", lambda: M.general(6, 4)),
    ("general_N33", lambda: M.general(33, 8)),
    ("general_N8_restricted", lambda: M.general(8, 6, sectors=[(8, 0), (6, 2), (4, 4)])),
    ("ensemble_c2_N40", lambda: M.ensemble_c2(40)),
    ("btc_c3_N65", lambda: M.btc_c3(65, 0.5)),
    ("btc_symmetric_N50", lambda: picuda.Models.boundary_time_crystal(50)),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_apply_f64_matches_oracle(torch_cuda, name, make):
    model = make()
    compiled = picuda.compile(model)
    oplan = O.Plan(M.to_oracle(model))
    for seed in range(2):
        x = M.random_state_vector(len(model.basis), seed)
        y = _apply64(torch_cuda, compiled, x)
        ref = O.apply(oplan, x)
        assert np.abs(y - ref).max() <= TOL_F64 * np.abs(ref).max(), name


@pytest.mark.parametrize("N,make", [(120, M.ensemble_c2), (200, M.btc_c3)], ids=["c2_N120", "c3_N200"])
def test_apply_f64_batched_matches_oracle(torch_cuda, N, make):
    """Batched (fixed-structure) kernel on several right-hand sides vs the oracle."""
    torch = torch_cuda
    model = make(N)
    compiled = picuda.compile(model)
    oplan = O.Plan(M.to_oracle(model))
    n = len(model.basis)
    X = np.stack([M.random_state_vector(n, 20 + s) for s in range(3)])
    Xd = _dev(torch, X)
    Yd = torch.empty_like(Xd)
    picuda.apply_(Yd, compiled, Xd)
    torch.cuda.synchronize()
    Y = Yd.cpu().numpy()
    for c in range(3):
        ref = O.apply(oplan, X[c])
        assert np.abs(Y[c] - ref).max() <= TOL_F64 * np.abs(ref).max()
    X32 = _dev(torch, X, torch.complex64)
    Y32 = torch.empty_like(X32)
    picuda.apply_(Y32, compiled, X32, precision="fp32", coords="reference")
    torch.cuda.synchronize()
    for c in range(3):
        ref = O.apply(oplan, X[c])
        assert np.abs(Y32[c].cpu().numpy() - ref).max() <= TOL_F32 * np.abs(ref).max()


@pytest.mark.parametrize("N,make", [(120, M.ensemble_c2), (200, M.btc_c3)], ids=["c2_N120", "c3_N200"])
def test_apply_f64_full_size(torch_cuda, N, make):
    model = make(N)
    compiled = picuda.compile(model)
    oplan = O.Plan(M.to_oracle(model))
    x = M.random_state_vector(len(model.basis), 11)
    y = _apply64(torch_cuda, compiled, x)
    ref = O.apply(oplan, x)
    assert np.abs(y - ref).max() <= TOL_F64 * np.abs(ref).max()
    # trace preservation: t^H (L x) = 0 for every x (liouvillian property tests)
    idx, val = compiled.library_trace_functional()
    assert abs(np.sum(val * y[idx])) <= 1e-11 * np.sum(np.abs(val * y[idx]))


def test_apply_multi_rhs_and_determinism(torch_cuda):
    torch = torch_cuda
    model = M.ensemble_c2(30)
    compiled = picuda.compile(model)
    n = len(model.basis)
    X = np.stack([M.random_state_vector(n, s) for s in range(3)])
    Xd = _dev(torch, X)
    Yd = torch.empty_like(Xd)
    picuda.apply_(Yd, compiled, Xd)
    Y2 = torch.empty_like(Xd)
    picuda.apply_(Y2, compiled, Xd)
    torch.cuda.synchronize()
    assert torch.equal(Yd, Y2), "apply must be bitwise deterministic"
    # multi-column applies run the fixed-structure batched kernel, single columns the
    # general one: same operator to rounding
    for c in range(3):
        single = _apply64(torch, compiled, X[c])
        assert np.abs(Yd[c].cpu().numpy() - single).max() <= 1e-14 * np.abs(single).max()
    # host-buffer path (H2D + apply + D2H) gives the bits of the device path
    yh = np.empty_like(X[0])
    picuda.apply_(yh, compiled, X[0].copy())
    assert np.array_equal(yh, _apply64(torch, compiled, X[0]))


def test_apply_rejects_aliasing_and_bad_shapes(torch_cuda):
    torch = torch_cuda
    compiled = picuda.compile(M.driven_c1(4))
    n = len(compiled.basis)
    x = torch.zeros(n, dtype=torch.complex128, device="cuda")
    with pytest.raises(picuda.PiArgumentError):
        picuda.apply_(x, compiled, x)
    with pytest.raises(picuda.PiDimensionMismatch):
        picuda.apply_(torch.zeros(n + 1, dtype=torch.complex128, device="cuda"), compiled,
                      torch.zeros(n + 1, dtype=torch.complex128, device="cuda"))


@pytest.mark.parametrize("N,make", [(40, M.ensemble_c2), (120, M.ensemble_c2), (200, M.btc_c3)])
def test_apply_f32_both_coordinates(torch_cuda, N, make):
    torch = torch_cuda
    model = make(N)
    compiled = picuda.compile(model)
    oplan = O.Plan(M.to_oracle(model))
    n = len(model.basis)
    x = M.random_state_vector(n, 5)
    ref = O.apply(oplan, x)
    # reference coordinates
    xd = _dev(torch, x, torch.complex64)
    yd = torch.empty_like(xd)
    picuda.apply_(yd, compiled, xd, precision="fp32", coords="reference")
    torch.cuda.synchronize()
    y = yd.cpu().numpy().astype(np.complex128)
    assert np.abs(y - ref).max() <= TOL_F32 * np.abs(ref).max()
    # population coordinates z = sqrt(f) x: feed z, compare sqrt(f) * (L x)
    scales = compiled.sector_scales()
    w = np.concatenate([np.full(d * d, s) for d, s in zip(model.basis.dims, scales)])
    z = M.random_state_vector(n, 6)
    xz = z / w
    refz = w * O.apply(oplan, xz)
    zd = _dev(torch, z, torch.complex64)
    yz = torch.empty_like(zd)
    picuda.apply_(yz, compiled, zd, precision="fp32", coords="population")
    torch.cuda.synchronize()
    out = yz.cpu().numpy().astype(np.complex128)
    assert np.abs(out - refz).max() <= TOL_F32 * np.abs(refz).max()


def test_library_basis_maps_bit_exact(torch_cuda):
    for N in (8, 120):
        compiled = picuda.compile(M.ensemble_c2(N))
        ob = O.PIBasis(N, 2)
        ks, offs, dims = compiled.library_sectors()
        assert [(N - k, k) for k in ks] == ob.sectors
        assert list(offs) == ob.offsets[:-1]
        assert list(dims) == [len(p) for p in ob.patterns]
        for s in (0, len(ks) // 2, len(ks) - 1):
            assert [tuple(r) for r in compiled.library_patterns(s)] == ob.patterns[s]
        idx, val = compiled.library_trace_functional()
        oidx, oval = O.trace_functional(ob)
        assert np.array_equal(idx, oidx) and np.array_equal(val, oval.real)


@pytest.mark.parametrize("name,make,kernel", [
    ("c2_N40", lambda: M.ensemble_c2(40), 2),
    ("pump_decay_N12", lambda: picuda.Models.local_pump_decay(12, down=1.0, up=0.3), 2),
    ("driven_N9", lambda: M.driven_c1(9), 2),
    ("general_N7", lambda: M.general(7, 2), 0),
])
def test_batched_kernel_paths_match_oracle(torch_cuda, name, make, kernel):
    """The plan picks the canonical-position kernel for real-operator qubit models (with and
    without +1 diagonal shifts, i.e. pumping) and the general tile kernel otherwise; every
    path matches the oracle."""
    torch = torch_cuda
    model = make()
    compiled = picuda.compile(model)
    assert compiled.info["batched_kernel"] == kernel, name
    oplan = O.Plan(M.to_oracle(model))
    n = len(model.basis)
    X = np.stack([M.random_state_vector(n, 40 + s) for s in range(5)])
    Yd = torch.empty((5, n), dtype=torch.complex128, device="cuda")
    picuda.apply_(Yd, compiled, _dev(torch, X))
    Y32 = torch.empty((5, n), dtype=torch.complex64, device="cuda")
    picuda.apply_(Y32, compiled, _dev(torch, X, torch.complex64), precision="fp32", coords="reference")
    torch.cuda.synchronize()
    for c in range(5):
        ref = O.apply(oplan, X[c])
        assert np.abs(Yd[c].cpu().numpy() - ref).max() <= TOL_F64 * np.abs(ref).max(), name
        assert np.abs(Y32[c].cpu().numpy() - ref).max() <= TOL_F32 * np.abs(ref).max(), name


@pytest.mark.parametrize("name,make", [
    ("c2_N40", lambda: M.ensemble_c2(40)),
    ("c2_N121", lambda: M.ensemble_c2(121)),
    ("pump_decay_N12", lambda: picuda.Models.local_pump_decay(12, down=1.0, up=0.3)),
    ("scan_N33", lambda: M.scan_model(33, 1.3, 0.2, 0.05)),
])
@pytest.mark.parametrize("coords", ["reference", "population"])
def test_element_major_apply_matches_column_apply(torch_cuda, name, make, coords):
    """Element-major batch (dim, ncols) against the column-batch FP32 apply and the oracle."""
    torch = torch_cuda
    model = make()
    compiled = picuda.compile(model)
    n = len(model.basis)
    ncols = 6
    X = np.stack([M.random_state_vector(n, 60 + s) for s in range(ncols)])  # (ncols, n)
    Xc = _dev(torch, X, torch.complex64)
    Yc = torch.empty_like(Xc)
    picuda.apply_(Yc, compiled, Xc, precision="fp32", coords=coords)
    Xe = Xc.t().contiguous()  # (n, ncols)
    Ye = torch.empty_like(Xe)
    picuda.apply_element_major_(Ye, compiled, Xe, coords=coords)
    torch.cuda.synchronize()
    got = Ye.t().cpu().numpy()
    ref = Yc.cpu().numpy()
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 2e-6 * scale, name
    if coords == "reference":
        oplan = O.Plan(M.to_oracle(model))
        for c in range(ncols):
            r = O.apply(oplan, X[c])
            assert np.abs(got[c] - r).max() <= TOL_F32 * np.abs(r).max(), name


@pytest.mark.parametrize("name,make,ncols", [
    ("c2_N61_128", lambda: M.ensemble_c2(61), 128),            # two 64-column halves, <= 64 sectors
    ("pump_N130_130", lambda: picuda.Models.local_pump_decay(130, down=1.0, up=0.3), 130),  # 66 sectors
    ("c2_N130_66", lambda: M.ensemble_c2(130), 66),            # ragged second half
    ("c2_N331_2", lambda: M.ensemble_c2(331), 2),              # 166 sectors: plain-load kernel
])
def test_element_major_apply_wide_batches(torch_cuda, name, make, ncols):
    """Element-major batches wider than one 64-column block, plans whose sector count selects
    each tensor-map table size, and a plan beyond it, against the column-batch FP32 apply."""
    torch = torch_cuda
    model = make()
    compiled = picuda.compile(model)
    n = len(model.basis)
    g = torch.Generator(device="cuda").manual_seed(11)
    Xe = torch.randn((n, ncols), dtype=torch.complex64, device="cuda", generator=g)
    Ye = torch.full_like(Xe, float("nan"))
    picuda.apply_element_major_(Ye, compiled, Xe)
    ref = torch.empty((ncols, n), dtype=torch.complex64, device="cuda")
    picuda.apply_(ref, compiled, Xe.t().contiguous(), precision="fp32", coords="population")
    torch.cuda.synchronize()
    assert not torch.isnan(Ye).any().item(), name
    err = (Ye.t() - ref).abs().max().item()
    assert err <= 2e-6 * ref.abs().max().item(), (name, err)
    # a second batch at another address (new tensor maps) and the first one again (kept maps)
    X2 = torch.randn((n, ncols), dtype=torch.complex64, device="cuda", generator=g)
    Y2 = torch.empty_like(X2)
    picuda.apply_element_major_(Y2, compiled, X2)
    Y3 = torch.empty_like(Xe)
    picuda.apply_element_major_(Y3, compiled, Xe)
    ref2 = torch.empty_like(ref)
    picuda.apply_(ref2, compiled, X2.t().contiguous(), precision="fp32", coords="population")
    torch.cuda.synchronize()
    assert (Y2.t() - ref2).abs().max().item() <= 2e-6 * ref2.abs().max().item(), name
    assert torch.equal(Y3, Ye), name  # deterministic


@pytest.mark.parametrize("name,make,rows", [
    ("c2_N40", lambda: M.ensemble_c2(40), (16, 32, 64)),
    ("pump_decay_N30", lambda: picuda.Models.local_pump_decay(30, down=1.0, up=0.3), (16, 32)),
])
def test_element_major_autotuner(torch_cuda, name, make, rows):
    """The first element-major call times every candidate kernel and keeps the fastest; every
    candidate (TMA-staged tiles of each height, plain loads) gives the same y, bit for bit."""
    torch = torch_cuda
    compiled = picuda.compile(make())
    n = len(compiled.basis)
    ncols = 128
    with pytest.raises(picuda.PiArgumentError):
        picuda.element_major_tuning(compiled, ncols)  # nothing tuned yet
    g = torch.Generator(device="cuda").manual_seed(5)
    X = torch.randn((n, ncols), dtype=torch.complex64, device="cuda", generator=g)
    Y = torch.full_like(X, float("nan"))
    picuda.apply_element_major_(Y, compiled, X)  # tunes
    ref = torch.empty((ncols, n), dtype=torch.complex64, device="cuda")
    picuda.apply_(ref, compiled, X.t().contiguous(), precision="fp32", coords="population")
    torch.cuda.synchronize()
    assert (Y.t() - ref).abs().max().item() <= 2e-6 * ref.abs().max().item(), name
    choice = picuda.element_major_tuning(compiled, ncols)
    assert choice["kernel"] in ("tma", "plain") and choice["ms"] > 0, choice
    assert choice["kernel"] == "plain" or choice["rows"] in rows, choice
    for kernel, r in [("tma", r) for r in rows] + [("plain", 32)]:
        picuda.select_element_major_kernel(compiled, ncols, kernel, r)
        Yk = torch.full_like(X, float("nan"))
        picuda.apply_element_major_(Yk, compiled, X)
        torch.cuda.synchronize()
        assert torch.equal(Yk, Y), (name, kernel, r)
        assert picuda.element_major_tuning(compiled, ncols) == {"kernel": kernel, "rows": r, "ms": 0.0}
    with pytest.raises(picuda.PiArgumentError):
        picuda.select_element_major_kernel(compiled, ncols, "tma", 48)
    if 64 not in rows:
        with pytest.raises(picuda.PiArgumentError):
            picuda.select_element_major_kernel(compiled, ncols, "tma", 64)


@pytest.mark.parametrize("name,make,ncols", [
    ("c2_N1", lambda: M.ensemble_c2(1), 2),
    ("c2_N2", lambda: M.ensemble_c2(2), 4),
    ("pump_decay_N3", lambda: picuda.Models.local_pump_decay(3, down=1.0, up=0.3), 66),
    ("c2_N318", lambda: M.ensemble_c2(318), 2),  # 160 sectors: the largest TMA map table
])
def test_element_major_apply_edge_sizes(torch_cuda, name, make, ncols):
    """Plans whose sectors are all smaller than one tile and the largest plan the TMA-staged
    kernel takes: every candidate kernel against the column-batch apply."""
    torch = torch_cuda
    model = make()
    compiled = picuda.compile(model)
    n = len(model.basis)
    g = torch.Generator(device="cuda").manual_seed(3)
    X = torch.randn((n, ncols), dtype=torch.complex64, device="cuda", generator=g)
    Y = torch.full_like(X, float("nan"))
    picuda.apply_element_major_(Y, compiled, X)
    ref = torch.empty((ncols, n), dtype=torch.complex64, device="cuda")
    picuda.apply_(ref, compiled, X.t().contiguous(), precision="fp32", coords="population")
    torch.cuda.synchronize()
    assert not torch.isnan(Y).any().item(), name
    assert (Y.t() - ref).abs().max().item() <= 2e-6 * max(ref.abs().max().item(), 1e-30), name
    for kernel, r in [("tma", 16), ("tma", 32), ("plain", 32)]:
        picuda.select_element_major_kernel(compiled, ncols, kernel, r)
        Yk = torch.full_like(X, float("nan"))
        picuda.apply_element_major_(Yk, compiled, X)
        torch.cuda.synchronize()
        assert torch.equal(Yk, Y), (name, kernel, r)


def test_element_major_apply_padded_stride_and_errors(torch_cuda):
    torch = torch_cuda
    model = M.ensemble_c2(20)
    compiled = picuda.compile(model)
    n = len(model.basis)
    base = torch.randn((n, 10), dtype=torch.complex64, device="cuda")
    X = base[:, :8]  # row stride 10, 8 columns
    Yb = torch.zeros((n, 10), dtype=torch.complex64, device="cuda")
    Y = Yb[:, :8]
    picuda.apply_element_major_(Y, compiled, X)
    ref = torch.empty_like(X.t().contiguous())
    picuda.apply_(ref, compiled, X.t().contiguous(), precision="fp32", coords="population")
    torch.cuda.synchronize()
    assert (Y.t() - ref).abs().max().item() <= 2e-6 * ref.abs().max().item()
    assert torch.count_nonzero(Yb[:, 8:]).item() == 0  # padding columns untouched
    with pytest.raises(picuda.PiArgumentError):
        picuda.apply_element_major_(torch.empty((n, 7), dtype=torch.complex64, device="cuda")[:, :7], compiled,
                                    torch.empty((n, 7), dtype=torch.complex64, device="cuda"))
    general = picuda.compile(M.general(6, 2))
    ng = len(general.basis)
    with pytest.raises(picuda.PiArgumentError):
        picuda.apply_element_major_(torch.empty((ng, 2), dtype=torch.complex64, device="cuda"), general,
                                    torch.empty((ng, 2), dtype=torch.complex64, device="cuda"))


def test_apply_largest_served_size_properties(torch_cuda):
    """The largest served request size (N = 300, dim 4,590,551), checked through properties
    that hold at any size: trace preservation t^H (L x) = 0, duality <y, L x> = <L^H y, x>,
    and the FP32 population-coordinate apply agreeing with the FP64 apply."""
    torch = torch_cuda
    model = M.ensemble_c2(300)
    c = picuda.compile(model)
    n = len(model.basis)
    assert n == 4590551
    x = torch.from_numpy(M.random_state_vector(n, 5)).cuda()
    y = torch.from_numpy(M.random_state_vector(n, 6)).cuda()
    Lx, LHy = torch.empty_like(x), torch.empty_like(y)
    picuda.apply_(Lx, c, x)
    picuda.apply_adjoint_(LHy, c, y)
    idx, val = c.library_trace_functional()
    idx_d = torch.from_numpy(idx).cuda()
    val_d = torch.from_numpy(val).cuda().to(torch.complex128)
    tr = (val_d * Lx[idx_d]).sum()
    assert abs(complex(tr.item())) <= 1e-11 * float((val_d.abs() * Lx[idx_d].abs()).sum())
    lhs, rhs = complex(torch.vdot(y, Lx).item()), complex(torch.vdot(LHy, x).item())
    assert abs(lhs - rhs) <= 1e-12 * float(torch.linalg.norm(Lx)) * float(torch.linalg.norm(y))
    # population coordinates z = sqrt(f) x are O(1) for physical states while sqrt(f) reaches
    # ~1e44 at N = 300: draw z, then x = z / sqrt(f)
    scale = torch.from_numpy(np.repeat(c.sector_scales(), np.array(model.basis.dims) ** 2)).cuda()
    z64 = torch.from_numpy(M.random_state_vector(n, 7)).cuda()
    xz = z64 / scale
    Lxz = torch.empty_like(xz)
    picuda.apply_(Lxz, c, xz)
    z = z64.to(torch.complex64)
    Lz = torch.empty_like(z)
    picuda.apply_(Lz, c, z, precision="fp32", coords="population")
    ref = Lxz * scale
    assert float((Lz.to(torch.complex128) - ref).abs().max()) <= 1e-5 * float(ref.abs().max())
