// Batched apply on element-major batches: y[e * ld + c] = (L x_c)[e] for c < ncols.
//
// The multi-right-hand-side apply of the reference (liouvillian.jl:3232-3251) takes the
// batch as a dim x ncols matrix; when the batch is stored element-major (ncols consecutive
// values per PI coordinate, a (dim, ncols) row-major array), every stencil source of an
// output entry is one contiguous row of the batch.  Then:
//   - a warp owns one output column b of one sector and walks its rows a; lane l reads the
//     right-hand-side pair (2l, 2l+1) of a source row with one 16-byte load, so every load
//     is fully coalesced and no shared-memory staging is needed;
//   - the stencil terms of the qubit families with real one-body operators sit at a few
//     canonical positions (own sector: centre, row shifts +-1, column shifts +-1, the
//     (-1,-1) diagonal; neighbouring sectors: two diagonal shifts each, three with pumping).
//     Terms at one position are merged into one complex coefficient per output entry,
//     precomputed once per plan into a coefficient plane [dim][kEmPos] (about 80 bytes per
//     entry against 16 bytes per entry and right-hand side of x and y); a warp copies the
//     coefficients of all its rows to shared memory once (cp.async) and reads them there;
//   - the own-sector sources of rows a-1, a, a+1 and columns b-1, b, b+1 stay in registers
//     as a sliding window, so each output row costs three new own-sector loads plus two per
//     neighbouring sector.
//
// Two kernels implement this:
//   - k_apply_em_tma: the sources are staged in shared memory by the Tensor Memory
//     Accelerator.  Every sector block of the batch is a 3-D tensor (right-hand side, row,
//     column) with its own tensor map, so one cp.async.bulk.tensor per row step and source
//     sector brings the 10 staged columns of a block's 8 output columns, and rows or columns
//     outside the sector block arrive as zeros from the hardware (no bounds checks).  A
//     producer thread keeps a ring of row steps in flight ahead of the 8 consumer warps
//     (full/empty mbarriers), so no warp holds loads in registers to hide memory latency.
//     Tiles of 16, 32 or 64 rows.
//   - k_apply_em_f32: the same stencil with plain coalesced loads from global memory; the
//     only kernel for plans with more sectors than the kernel-parameter map table holds.
// Every candidate computes each output entry with the same operations in the same order, so
// the autotuner (em_tune) may pick any of them per batch width by timing: the first call
// times them on the caller's batch and later calls launch the fastest.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "../../include/picuda.h"
#include "pi_apply_impl.cuh"
#include "pi_handle.hpp"

namespace picuda {
namespace {

constexpr int kEmRows = 32;   // rows per warp task
constexpr int kEmWarps = 8;   // columns per block
constexpr int kEmPos = 10;    // canonical positions without +1 diagonal shifts
constexpr int kEmPosPlus = 14;  // with them (13, padded to an even count)

// Plane position index -> canonical table entry.  Positions:
//  0 own centre (ADD + own (0,0) sandwich), 1 LEFT -1, 2 LEFT +1, 3 RIGHT -1, 4 RIGHT +1,
//  5 own (-1,-1), 6 smaller sector (-2,-2), 7 smaller (-1,-1), 8 larger (0,0), 9 larger (1,1),
//  10 own (1,1), 11 smaller (0,0), 12 larger (2,2), 13 padding.
// Sandwich entries of the canonical table are indexed slot * 3 + (p + 1), p = q the window
// shift; the smaller source sector is slot 0 (e = -1), the larger slot 2 (e = +1).
__device__ __forceinline__ int sand_pos(int plane) {
  switch (plane) {
    case 5: return 3;   // own, p = -1
    case 6: return 0;   // slot 0, p = -1
    case 7: return 1;   // slot 0, p = 0
    case 8: return 6;   // slot 2, p = -1
    case 9: return 7;   // slot 2, p = 0
    case 10: return 5;  // own, p = +1
    case 11: return 2;  // slot 0, p = +1
    case 12: return 8;  // slot 2, p = +1
    default: return -1;
  }
}

// Merged coefficient of plane position k at entry (a, b) of a sector (canonical table ct).
template <typename T2>
__device__ __forceinline__ T2 em_coef(int k, const int4* __restrict__ ct, const T2* __restrict__ coef, int a, int b) {
  using T = decltype(T2{}.x);
  T re = 0, im = 0;
  if (k == 0) {
    const T2 al = coef[ct[0].x + a], be = coef[ct[0].y + b];
    re = al.x + be.x;
    im = al.y + be.y;
    for (int t = 0; t < kCanonPerPos; ++t) {
      const int4 e = ct[5 + 4 * kCanonPerPos + t];  // own centre sandwich (slot 1, p = 0)
      re += coef[e.x + a].x * coef[e.y + b].x;
    }
  } else if (k <= 2) {
    const T2 al = coef[ct[k].x + a];  // LEFT: alpha only
    re = al.x;
    im = al.y;
  } else if (k <= 4) {
    const T2 be = coef[ct[k].y + b];  // RIGHT: beta only
    re = be.x;
    im = be.y;
  } else {
    const int pos = sand_pos(k);
    if (pos >= 0)
      for (int t = 0; t < kCanonPerPos; ++t) {
        const int4 e = ct[5 + pos * kCanonPerPos + t];
        re += coef[e.x + a].x * coef[e.y + b].x;
      }
  }
  T2 v;
  v.x = re;
  v.y = im;
  return v;
}

// planes[e * np + k] for every entry e of sector blockIdx.y.
template <typename T>
__global__ void k_em_planes(const DevSector* __restrict__ sectors, const int4* __restrict__ canon,
                            const typename Vec2<T>::type* __restrict__ coef, int np,
                            typename Vec2<T>::type* __restrict__ planes) {
  using T2 = typename Vec2<T>::type;
  const int s = blockIdx.y;
  const DevSector sec = sectors[s];
  const int n = sec.n;
  const long long cnt = (long long)n * n;
  const int4* ct = canon + (long long)s * kCanonEntries;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(i % n), b = (int)(i / n);
    T2* out = planes + (sec.offset + i) * np;
    for (int k = 0; k < np; ++k) out[k] = em_coef<T2>(k, ct, coef, a, b);
  }
}

// The same coefficients split by what they depend on, for the TMA-staged kernel:
//   entry plane, per entry (a, b) (ne float4): (centre re, centre im, own (-1,-1), smaller
//     (-2,-2)), (smaller (-1,-1), larger (0,0), larger (1,1), own (1,1)) [, (smaller (0,0),
//     larger (2,2), 0, 0)] -- the real positions only carry a real part;
//   row plane, per row a of a sector: (LEFT -1, LEFT +1) -- alpha only, shared by all columns;
//   column plane, per column b: (RIGHT -1, RIGHT +1) -- beta only, constant along a column.
// Row and column planes of sector s start at line_off[s] (the sum of the smaller n).
__global__ void k_em_split_planes(const DevSector* __restrict__ sectors, const int4* __restrict__ canon,
                                  const float2* __restrict__ coef, const int* __restrict__ line_off, int ne,
                                  float4* __restrict__ eplane, float4* __restrict__ lrow, float4* __restrict__ rcol) {
  const int s = blockIdx.y;
  const DevSector sec = sectors[s];
  const int n = sec.n;
  const long long cnt = (long long)n * n;
  const int4* ct = canon + (long long)s * kCanonEntries;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(i % n), b = (int)(i / n);
    const float2 c0 = em_coef<float2>(0, ct, coef, a, b);
    float4* out = eplane + (sec.offset + i) * ne;
    out[0] = make_float4(c0.x, c0.y, em_coef<float2>(5, ct, coef, a, b).x, em_coef<float2>(6, ct, coef, a, b).x);
    out[1] = make_float4(em_coef<float2>(7, ct, coef, a, b).x, em_coef<float2>(8, ct, coef, a, b).x,
                         em_coef<float2>(9, ct, coef, a, b).x, ne > 2 ? em_coef<float2>(10, ct, coef, a, b).x : 0.f);
    if (ne > 2)
      out[2] = make_float4(em_coef<float2>(11, ct, coef, a, b).x, em_coef<float2>(12, ct, coef, a, b).x, 0.f, 0.f);
  }
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const float2 l0 = em_coef<float2>(1, ct, coef, i, 0), l1 = em_coef<float2>(2, ct, coef, i, 0);
      const float2 r0 = em_coef<float2>(3, ct, coef, 0, i), r1 = em_coef<float2>(4, ct, coef, 0, i);
      lrow[line_off[s] + i] = make_float4(l0.x, l0.y, l1.x, l1.y);
      rcol[line_off[s] + i] = make_float4(r0.x, r0.y, r1.x, r1.y);
    }
}

// Separable line planes (SplitPlanes::srow / scol): per row a and per column b of sector
// blockIdx.y, the factors of every merged coefficient in the order em_coef combines them.
__global__ void k_sep_planes(const DevSector* __restrict__ sectors, const int4* __restrict__ canon,
                             const float2* __restrict__ coef, const int* __restrict__ line_off, int nf4,
                             float4* __restrict__ srow, float4* __restrict__ scol) {
  // sandwich positions of the canonical table (slot * 3 + p + 1) in plane order
  constexpr int kPos[9] = {4, 3, 0, 1, 6, 7, 5, 2, 8};
  const int s = blockIdx.y;
  const DevSector sec = sectors[s];
  const int n = sec.n;
  const int4* ct = canon + (long long)s * kCanonEntries;
  const int npos = nf4 == kSepF4Plus ? 9 : 6;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float r[4 * kSepF4Plus], c[4 * kSepF4Plus];
    for (int k = 0; k < 4 * nf4; ++k) r[k] = c[k] = 0.f;
    const float2 aa = coef[ct[0].x + i], bb = coef[ct[0].y + i];
    const float2 l0 = coef[ct[1].x + i], l1 = coef[ct[2].x + i];
    const float2 r0 = coef[ct[3].y + i], r1 = coef[ct[4].y + i];
    r[0] = aa.x; r[1] = aa.y; r[2] = l0.x; r[3] = l0.y; r[4] = l1.x; r[5] = l1.y;
    c[0] = bb.x; c[1] = bb.y; c[2] = r0.x; c[3] = r0.y; c[4] = r1.x; c[5] = r1.y;
    for (int p = 0; p < npos; ++p)
      for (int t = 0; t < kCanonPerPos; ++t) {
        const int4 e = ct[5 + kPos[p] * kCanonPerPos + t];
        r[6 + 3 * p + t] = coef[e.x + i].x;
        c[6 + 3 * p + t] = coef[e.y + i].x;
      }
    float4* ro = srow + (long long)(line_off[s] + i) * nf4;
    float4* co = scol + (long long)(line_off[s] + i) * nf4;
    for (int k = 0; k < nf4; ++k) {
      ro[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
      co[k] = make_float4(c[4 * k], c[4 * k + 1], c[4 * k + 2], c[4 * k + 3]);
    }
  }
}

__device__ __forceinline__ void cmac2(float4& acc, const float cr, const float ci, const float4 v) {
  // acc.(xy) += c * v.(xy), acc.(zw) += c * v.(zw) (complex c = cr + i ci)
  acc.x = fmaf(cr, v.x, acc.x);
  acc.x = fmaf(-ci, v.y, acc.x);
  acc.y = fmaf(cr, v.y, acc.y);
  acc.y = fmaf(ci, v.x, acc.y);
  acc.z = fmaf(cr, v.z, acc.z);
  acc.z = fmaf(-ci, v.w, acc.z);
  acc.w = fmaf(cr, v.w, acc.w);
  acc.w = fmaf(ci, v.z, acc.w);
}
__device__ __forceinline__ void rmac2(float4& acc, const float c, const float4 v) {
  acc.x = fmaf(c, v.x, acc.x);
  acc.y = fmaf(c, v.y, acc.y);
  acc.z = fmaf(c, v.z, acc.z);
  acc.w = fmaf(c, v.w, acc.w);
}

// A source stream: one column of one source block, walked row by row as the warp walks its
// output rows.  Positions are 32-bit indices in float4 units (dim * ld/2 < 2^32, checked on
// the host), advanced by the row stride with one 32-bit add per row.
struct Stream {
  unsigned idx;  // float4 index of row `row` (meaningful when the row and column are valid)
  int row;
  int m;
  bool col_ok;
};

__device__ __forceinline__ Stream make_stream(unsigned ld4, int off, int m, int r, int c, int q) {
  Stream s;
  s.col_ok = (unsigned)c < (unsigned)m;
  s.m = m;
  s.row = r;
  s.idx = (unsigned)(off + r + (s.col_ok ? c : 0) * m) * ld4 + (unsigned)q;
  return s;
}
__device__ __forceinline__ void advance(Stream& s, unsigned ld4) {
  s.idx += ld4;
  ++s.row;
}

// Q right-hand-side pairs per lane (Q = 1: lane l holds pair l of its 32-pair chunk; Q = 2:
// pairs l and l + 32 of a 64-pair chunk), so coefficient loads and index updates are shared
// by 2Q right-hand sides.
template <int Q>
struct Pack {
  float4 v[Q];
};

// Loads pair i only for lanes whose pair i lies inside the batch (lane_ok[i]); pair 0 of a
// lane past the batch is redirected to pair 0 by the caller, so every read is in bounds.
template <int Q>
__device__ __forceinline__ Pack<Q> takeq(const float4* __restrict__ x, const Stream& s, const bool (&lane_ok)[Q]) {
  Pack<Q> r;
  const bool ok = s.col_ok && (unsigned)s.row < (unsigned)s.m;
#pragma unroll
  for (int i = 0; i < Q; ++i)
    r.v[i] = (ok && (i == 0 || lane_ok[i])) ? __ldg(x + s.idx + 32 * i) : make_float4(0.f, 0.f, 0.f, 0.f);
  return r;
}
template <int Q>
__device__ __forceinline__ void cmacq(Pack<Q>& acc, const float cr, const float ci, const Pack<Q>& v) {
#pragma unroll
  for (int i = 0; i < Q; ++i) cmac2(acc.v[i], cr, ci, v.v[i]);
}
template <int Q>
__device__ __forceinline__ void rmacq(Pack<Q>& acc, const float c, const Pack<Q>& v) {
#pragma unroll
  for (int i = 0; i < Q; ++i) rmac2(acc.v[i], c, v.v[i]);
}

template <bool PLUS, int Q>
__global__ void __launch_bounds__(32 * kEmWarps, 4)
    k_apply_em_f32(const DevSector* __restrict__ sectors, const DevTile* __restrict__ tiles,
                   const float2* __restrict__ planes, const float4* __restrict__ x, float4* __restrict__ y,
                   unsigned ld4, int npairs, BorderArgs border) {
  constexpr int NP = PLUS ? kEmPosPlus : kEmPos;
  const DevTile tile = tiles[blockIdx.x];
  const int lane = threadIdx.x & 31;
  const int q0 = blockIdx.y * 32 * Q + lane;  // first right-hand-side pair of this lane
  const DevSector sec = sectors[tile.sector];
  const int n = sec.n;
  const int b = tile.b0 + (threadIdx.x >> 5);
  if (b >= n) return;  // warp-uniform
  const int a0 = tile.a0;
  const int a_end = min(a0 + kEmRows, n);
  const int own = (int)sec.offset;
  const int s0 = sec.src[0], s2 = sec.src[2];
  const int off0 = s0 >= 0 ? (int)sectors[s0].offset : 0, off2 = s2 >= 0 ? (int)sectors[s2].offset : 0;
  const int m0 = s0 >= 0 ? sectors[s0].n : 0, m2 = s2 >= 0 ? sectors[s2].n : 0;
  // Everything FP64 is evaluated here, once per warp: inside the row loop the compiler would
  // if-convert it and every row would issue it to GB300's narrow FP64 pipe.
  const float scale = (float)border.scale;
  const bool do_scale = scale != 1.0f;
  bool ok[Q];
  Pack<Q> badd;  // trace-border addend of the diagonal entry (a == b)
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const int q = q0 + 32 * i;
    ok[i] = q < npairs;
    badd.v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (border.alpha != nullptr && ok[i] && b >= a0 && b < a_end) {
      const double v = border.coords ? sec.border_z : sec.border_x;
      const double2 al0 = border.alpha[2 * q], al1 = border.alpha[2 * q + 1];
      badd.v[i] = make_float4((float)(al0.x * v), (float)(al0.y * v), (float)(al1.x * v), (float)(al1.y * v));
    }
  }
  const int qq = ok[0] ? q0 : 0;  // lanes past the batch read pair 0 (in bounds) and store nothing
  // own-sector window rows a-1, a, a+1 of columns b-1, b, b+1; the streams point at row a+2
  Pack<Q> w[3][3];
  Stream so[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    Stream t = make_stream(ld4, own, n, a0 - 1, b - 1 + c, qq);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      w[r][c] = takeq<Q>(x, t, ok);
      advance(t, ld4);
    }
    so[c] = t;
  }
  // neighbouring sectors: smaller (a-2, b-2), (a-1, b-1) [, (a, b)]; larger (a, b),
  // (a+1, b+1) [, (a+2, b+2)]; a zero-size block when the neighbour does not exist
  Stream sm[3], sl[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    sm[d] = make_stream(ld4, off0, m0, a0 - 2 + d, b - 2 + d, qq);
    sl[d] = make_stream(ld4, off2, m2, a0 + d, b + d, qq);
  }
  constexpr int NX = PLUS ? 3 : 2;  // cross-sector streams per neighbour
  // The warp's merged coefficients for all its rows (contiguous in the planes: rows a0..
  // a_end-1 of column b) go to shared memory with one round of asynchronous copies, so no
  // row waits on a coefficient load from memory (the planes are read once per launch and
  // miss in L2; loaded row by row they put a full memory latency into every iteration).
  __shared__ __align__(16) float4 coef_sm[kEmWarps][kEmRows * (NP / 2)];
  float4* cw = coef_sm[threadIdx.x >> 5];
  {
    const float4* src = reinterpret_cast<const float4*>(planes) + (size_t)(unsigned)(own + a0 + b * n) * (NP / 2);
    const int cnt = (a_end - a0) * (NP / 2);
    for (int i = lane; i < cnt; i += 32) cp_async_zfill<16>(cw + i, src + i, true);
    cp_async_commit();
  }
  unsigned yi = (unsigned)(own + a0 + b * n) * ld4 + (unsigned)qq;
  cp_async_wait<0>();
  __syncwarp();
  for (int a = a0; a < a_end; ++a) {
    // coefficient pairs: cv[k] = (c_{2k}, c_{2k+1}), used component-wise
    float4 cv[NP / 2];
#pragma unroll
    for (int k = 0; k < NP / 2; ++k) cv[k] = cw[(a - a0) * (NP / 2) + k];
    Pack<Q> acc;
#pragma unroll
    for (int i = 0; i < Q; ++i) acc.v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    cmacq<Q>(acc, cv[0].x, cv[0].y, w[1][1]);  // 0 centre
    cmacq<Q>(acc, cv[0].z, cv[0].w, w[0][1]);  // 1 LEFT -1
    cmacq<Q>(acc, cv[1].x, cv[1].y, w[2][1]);  // 2 LEFT +1
    cmacq<Q>(acc, cv[1].z, cv[1].w, w[1][0]);  // 3 RIGHT -1
    cmacq<Q>(acc, cv[2].x, cv[2].y, w[1][2]);  // 4 RIGHT +1
    rmacq<Q>(acc, cv[2].z, w[0][0]);           // 5 own (-1,-1)
    Pack<Q> xs[NX], xl[NX];
#pragma unroll
    for (int d = 0; d < NX; ++d) {
      xs[d] = takeq<Q>(x, sm[d], ok);
      xl[d] = takeq<Q>(x, sl[d], ok);
    }
    rmacq<Q>(acc, cv[3].x, xs[0]);  // 6 smaller (-2,-2)
    rmacq<Q>(acc, cv[3].z, xs[1]);  // 7 smaller (-1,-1)
    rmacq<Q>(acc, cv[4].x, xl[0]);  // 8 larger (0,0)
    rmacq<Q>(acc, cv[4].z, xl[1]);  // 9 larger (1,1)
    if (PLUS) {
      rmacq<Q>(acc, cv[5].x, w[2][2]);  // 10 own (1,1)
      rmacq<Q>(acc, cv[5].z, xs[NX - 1]);  // 11 smaller (0,0)
      rmacq<Q>(acc, cv[6].x, xl[NX - 1]);  // 12 larger (2,2)
    }
#pragma unroll
    for (int d = 0; d < NX; ++d) {
      advance(sm[d], ld4);
      advance(sl[d], ld4);
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      float4 o = acc.v[i];
      if (do_scale) {
        o.x *= scale;
        o.y *= scale;
        o.z *= scale;
        o.w *= scale;
      }
      if (a == b) {
        o.x += badd.v[i].x;
        o.y += badd.v[i].y;
        o.z += badd.v[i].z;
        o.w += badd.v[i].w;
      }
      if (ok[i]) y[yi + 32 * i] = o;
    }
    yi += ld4;
    // slide the window down one row
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      w[0][cc] = w[1][cc];
      w[1][cc] = w[2][cc];
      w[2][cc] = takeq<Q>(x, so[cc], ok);
      advance(so[cc], ld4);
    }
  }
}

// ---------------------------------------------------------------------------------------
// TMA-staged kernel.
//
// Block = one tile (16, 32 or 64 rows x 8 columns of one sector block) and one half of the
// batch row (64 complex right-hand sides = 512 bytes).  Row step k stages, in one ring slot:
//   source 0: smaller sector, row k-1, columns b0-2 .. b0+7
//   source 1: own sector,     row k,   columns b0-1 .. b0+8
//   source 2: larger sector,  row k+1, columns b0   .. b0+9
// so output row a reads the slots of steps a-1, a and a+1; a consumer warp reads each step's
// own row when it lands and its neighbour columns one row later, then releases the slot.  A
// tile of R rows takes R + 2 steps (a0-1 .. a0+R).
constexpr int kTmW = kEmWarps;                      // consumer warps = output columns
constexpr int kTmCols = kTmW + 2;                   // staged columns per source sector
constexpr int kTmHalf = 64;                         // complex right-hand sides per block
constexpr int kTmColBytes = kTmHalf * 8;            // one staged column of one row
constexpr int kTmSrcBytes = kTmCols * kTmColBytes;  // one source sector of one step
constexpr int kTmSlotBytes = 3 * kTmSrcBytes;       // one ring slot
constexpr int kTmThreads = 32 * (kTmW + 1);         // + one producer warp
constexpr int kTmWaitLimit = 1 << 22;               // mbarrier polls before a wait gives up

template <int MAXS>
struct EmMaps {
  CUtensorMap m[MAXS];
};

// Tile record of the TMA-staged kernel: everything a block needs about its tile and sector in
// one 48-byte load (no dependent loads at block start).
struct alignas(16) TmTile {
  long long offset;  // sector block offset
  int sector, a0, b0, n;
  int s0, s2;        // smaller / larger neighbour sector (-1: none)
  int loff;          // start of the sector's row and column planes
  int pad[3];
};
static_assert(sizeof(TmTile) == 48, "tile record layout");

template <bool PLUS, int ROWS>
struct TmCfg {
  static constexpr int NE = PLUS ? 3 : 2;  // float4 of the entry plane per entry
  static constexpr int RING = 6;           // two blocks of 8+1 warps per SM
  static constexpr int ENTRY_BYTES = kTmW * ROWS * NE * 16;  // entry-plane runs of the warps
  static constexpr int ROW_BYTES = ROWS * 16;                // row-plane run of the tile
  static constexpr int COL_BYTES = kTmW * 16;                   // column-plane values of the tile
  static constexpr int SMEM = RING * kTmSlotBytes + ENTRY_BYTES + ROW_BYTES + COL_BYTES + 2 * RING * 8;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
// Bounded wait for the completion of the phase with the given parity: false after
// kTmWaitLimit polls (each poll may suspend the thread for a short, hardware-defined time).
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity) {
  for (int it = 0; it < kTmWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

template <bool PLUS, int MAXS, int ROWS>
__global__ void __launch_bounds__(kTmThreads, 2)
    k_apply_em_tma(const __grid_constant__ EmMaps<MAXS> maps, const TmTile* __restrict__ tiles,
                   const float4* __restrict__ eplane, const float4* __restrict__ lrow,
                   const float4* __restrict__ rcol, float4* __restrict__ y, unsigned ld4, int npairs) {
  using C = TmCfg<PLUS, ROWS>;
  constexpr int NE = C::NE;
  constexpr int RING = C::RING;
  static_assert(RING % 3 == 0, "own rows are kept in registers indexed by step modulo three");
  extern __shared__ __align__(1024) unsigned char smem[];
  const float4* ring = reinterpret_cast<const float4*>(smem);
  const float4* ent = reinterpret_cast<const float4*>(smem + RING * kTmSlotBytes);
  const float4* lrw = reinterpret_cast<const float4*>(smem + RING * kTmSlotBytes + C::ENTRY_BYTES);
  const uint32_t ring_u32 = smem_u32(smem);
  const uint32_t ent_u32 = ring_u32 + RING * kTmSlotBytes;
  const uint32_t row_u32 = ent_u32 + C::ENTRY_BYTES;
  const uint32_t col_u32 = row_u32 + C::ROW_BYTES;
  const uint32_t full0 = col_u32 + C::COL_BYTES;  // full[i] at full0 + 8 i
  const uint32_t empty0 = full0 + 8 * RING;        // empty[i] at empty0 + 8 i

  const TmTile tile = tiles[blockIdx.x];
  const int n = tile.n;
  const int a0 = tile.a0, b0 = tile.b0;
  const int rows = min(ROWS, n - a0);
  const int s0 = tile.s0, s2 = tile.s2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int i = 0; i < RING; ++i) {
      mbar_init(full0 + 8 * i, 1);
      mbar_init(empty0 + 8 * i, kTmW);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // A missing neighbour sector (first or last sector) is never loaded: its part of every
  // slot is zeroed once here, so the consumers read zeros without a test per load.
  if (s0 < 0 || s2 < 0) {
    float4* rw = reinterpret_cast<float4*>(smem);
    constexpr int per_src = kTmSrcBytes / 16;
    for (int i = threadIdx.x; i < RING * per_src; i += blockDim.x) {
      const int slot = i / per_src, e = i - slot * per_src;
      if (s0 < 0) rw[(slot * 3 + 0) * per_src + e] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (s2 < 0) rw[(slot * 3 + 2) * per_src + e] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  __syncthreads();

  if (warp == kTmW) {  // producer: one thread issues every copy of the block
    if (lane != 0) return;
    // Step i (relative row a0-1+i): own row, smaller row - 1, larger row + 1, and at step 0
    // every consumer warp's merged coefficients for all its rows (contiguous in the planes).
    // Step i reuses the slot of step i - RING once every consumer warp has released it.
    const CUtensorMap* m_own = &maps.m[tile.sector];
    const CUtensorMap* m_sm = s0 >= 0 ? &maps.m[s0] : nullptr;
    const CUtensorMap* m_lg = s2 >= 0 ? &maps.m[s2] : nullptr;
    const int xq = blockIdx.y * kTmHalf;
    const uint32_t step_bytes = kTmSrcBytes * (1u + (m_sm != nullptr) + (m_lg != nullptr));
    const int nact = min(kTmW, n - b0);
    const uint32_t run_bytes = (uint32_t)rows * NE * 16, row_bytes = (uint32_t)rows * 16;
    const int nsteps = rows + 2;
    for (int i = 0; i < nsteps; ++i) {
      const int slot = i % RING;
      const uint32_t full = full0 + 8 * slot;
      if (i >= RING && !mbar_wait(empty0 + 8 * slot, (uint32_t)((i / RING) - 1) & 1u)) return;
      mbar_expect_tx(full, step_bytes + (i == 0 ? (run_bytes + 16u) * (uint32_t)nact + row_bytes : 0u));
      const int k = a0 - 1 + i;
      const uint32_t dst = ring_u32 + slot * kTmSlotBytes;
      tma_load_3d(dst + kTmSrcBytes, m_own, xq, k, b0 - 1, full);
      if (m_sm) tma_load_3d(dst, m_sm, xq, k - 1, b0 - 2, full);
      if (m_lg) tma_load_3d(dst + 2 * kTmSrcBytes, m_lg, xq, k + 1, b0, full);
      if (i == 0) {  // the warps' entry-plane runs (contiguous down a column), row and column planes
        for (int w = 0; w < nact; ++w)
          bulk_load(ent_u32 + w * (ROWS * NE * 16), eplane + (size_t)(tile.offset + a0 + (long long)(b0 + w) * n) * NE,
                    run_bytes, full);
        bulk_load(row_u32, lrow + tile.loff + a0, row_bytes, full);
        bulk_load(col_u32, rcol + tile.loff + b0, (uint32_t)nact * 16, full);
      }
    }
    return;
  }

  // consumers: warp w owns output column b = b0 + w, lane l the right-hand-side pair q
  const int b = b0 + warp;
  const bool active = b < n;
  const int q = blockIdx.y * 32 + lane;
  const bool ok = active && q < npairs;
  // This lane's float4 in staged column c of source src of slot i is rl[SLOT_F4 i + SRC_F4 src
  // + COL_F4 c]: with the row loop unrolled over the ring, every offset is a constant.
  constexpr int COL_F4 = kTmColBytes / 16, SRC_F4 = kTmSrcBytes / 16, SLOT_F4 = kTmSlotBytes / 16;
  const float4* rl = ring + warp * COL_F4 + lane;
  const float4* ew = ent + warp * (ROWS * NE);
  unsigned yi = (unsigned)(tile.offset + a0 + (long long)(active ? b : 0) * n) * ld4 + (unsigned)(ok ? q : 0);
  int r = 0;
  // Step s carries own row s-1 (relative to a0), used by output rows s-2 .. s, and the
  // neighbour sectors' columns w+2 (row s-2, pumping terms only), w+1 (row s-1) and w (row s).
  // A warp reads the own row and column w+2 when the step lands (row s-2), columns w+1 and w
  // one row later, keeps column w in registers for one more row and then releases the slot:
  // each slot is held for one output row, so RING-1 steps stay in flight ahead of the reads.
  // Own rows live in win[t % 3] (t = the step): with a ring of a multiple of three slots the
  // index is a constant in every unrolled copy.
  float4 win[3][3];  // own rows a-1, a, a+1 at columns b-1, b, b+1
  auto take_own = [&](int slot, int qi) {
#pragma unroll
    for (int c = 0; c < 3; ++c) win[qi][c] = rl[slot * SLOT_F4 + 1 * SRC_F4 + c * COL_F4];
  };
  auto release = [&](int slot) {
    __syncwarp();
    if (lane == 0) mbar_arrive(empty0 + 8 * slot);
  };
  float4 hs, hl;  // smaller / larger column w of step r, read one row early
  bool good = mbar_wait(full0, 0) && mbar_wait(full0 + 8, 0);
  // RIGHT -1, +1 of column b (staged with step 0)
  const float4 rc = reinterpret_cast<const float4*>(smem + RING * kTmSlotBytes + C::ENTRY_BYTES + C::ROW_BYTES)[active ? warp : 0];
  if (good) {
    take_own(0, 0);
    take_own(1, 1);
    hs = rl[0 * SLOT_F4 + 0 * SRC_F4 + 0 * COL_F4];
    hl = rl[0 * SLOT_F4 + 2 * SRC_F4 + 0 * COL_F4];
    release(0);
  }
  uint32_t phase = 0;  // parity of ring pass base / RING
  for (int base = 0; good && base < rows; base += RING, phase ^= 1u) {
#pragma unroll
    for (int k = 0; k < RING; ++k) {
      r = base + k;
      if (r >= rows) break;
      const int sl1 = (k + 1) % RING, sl2 = (k + 2) % RING;  // ring slots of steps r+1, r+2
      if (!mbar_wait(full0 + 8 * sl2, phase ^ (k + 2 >= RING ? 1u : 0u))) {
        good = false;
        break;
      }
      // window indices of steps r, r+1, r+2 (base is a multiple of three)
      const int q0 = k % 3, q1 = (k + 1) % 3, q2 = (k + 2) % 3;
      take_own(sl2, q2);
      float4 xs2, xl2;
      if (PLUS) {
        xs2 = rl[sl2 * SLOT_F4 + 0 * SRC_F4 + 2 * COL_F4];
        xl2 = rl[sl2 * SLOT_F4 + 2 * SRC_F4 + 2 * COL_F4];
      }
      const float4 xs1 = rl[sl1 * SLOT_F4 + 0 * SRC_F4 + 1 * COL_F4];
      const float4 xl1 = rl[sl1 * SLOT_F4 + 2 * SRC_F4 + 1 * COL_F4];
      const float4 ns = rl[sl1 * SLOT_F4 + 0 * SRC_F4 + 0 * COL_F4];
      const float4 nl = rl[sl1 * SLOT_F4 + 2 * SRC_F4 + 0 * COL_F4];
      release(sl1);  // step r+1 is not read again
      const float4 e0 = ew[r * NE], e1 = ew[r * NE + 1];
      const float4 lv = lrw[r];  // LEFT -1, +1 of row a
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      cmac2(acc, e0.x, e0.y, win[q1][1]);  // 0 centre
      cmac2(acc, lv.x, lv.y, win[q0][1]);  // 1 LEFT -1
      cmac2(acc, lv.z, lv.w, win[q2][1]);  // 2 LEFT +1
      cmac2(acc, rc.x, rc.y, win[q1][0]);  // 3 RIGHT -1
      cmac2(acc, rc.z, rc.w, win[q1][2]);  // 4 RIGHT +1
      rmac2(acc, e0.z, win[q0][0]);        // 5 own (-1,-1)
      rmac2(acc, e0.w, hs);                // 6 smaller (-2,-2): step r, column w
      rmac2(acc, e1.x, xs1);               // 7 smaller (-1,-1): step r+1, column w+1
      rmac2(acc, e1.y, hl);                // 8 larger (0,0): step r, column w
      rmac2(acc, e1.z, xl1);               // 9 larger (1,1): step r+1, column w+1
      if (PLUS) {
        const float4 e2 = ew[r * NE + 2];
        rmac2(acc, e1.w, win[q2][2]);  // 10 own (1,1)
        rmac2(acc, e2.x, xs2);         // 11 smaller (0,0): step r+2, column w+2
        rmac2(acc, e2.y, xl2);         // 12 larger (2,2): step r+2, column w+2
      }
      if (ok) __stcs(y + yi, acc);  // streamed out: keeps L2 for the rows neighbouring sectors reread
      yi += ld4;
      hs = ns;
      hl = nl;
      r = base + k + 1;
    }
  }
  if (!good && ok) {  // a wait gave up: mark the rows this warp did not compute
    const float nan = __int_as_float(0x7fc00000);
    for (; r < rows; ++r, yi += ld4) y[yi] = make_float4(nan, nan, nan, nan);
  }
}

}  // namespace

// Builds (once per plan) the element-major tile list.  Caller holds plan->em_mu.
static int em_tiles(pi_plan* plan) {
  const DevicePlan& dp = plan->dev;
  if (!dp.canon)
    return fail(PI_ERR_UNSUPPORTED,
                "element-major batched apply needs a plan whose stencil sits at the canonical positions "
                "(qubit models with real one-body operators)");
  if (!plan->em_tiles) {
    std::vector<DevTile> tiles;
    for (int s = 0; s < (int)plan->host.sectors.size(); ++s) {
      const int n = plan->host.sectors[s].n;
      for (int a0 = 0; a0 < n; a0 += kEmRows)
        for (int b0 = 0; b0 < n; b0 += kEmWarps) tiles.push_back(DevTile{s, a0, b0, 0});
    }
    void* d = plan_alloc(plan, sizeof(DevTile) * tiles.size());
    if (!d) return fail(PI_ERR_OUT_OF_MEMORY, "element-major tile list");
    cudaError_t e = cudaMemcpy(d, tiles.data(), sizeof(DevTile) * tiles.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "element-major tile list");
    plan->em_tiles = (const DevTile*)d;
    plan->em_ntiles = (int)tiles.size();
  }
  return PI_OK;
}

// Builds (once per plan and coefficient set) the merged coefficient planes of the kernel
// with plain loads.  which: 0 FP32 reference coordinates, 1 FP32 population coordinates.
static int em_prepare(pi_plan* plan, int which, const float2** planes_out) {
  std::lock_guard<std::mutex> lk(plan->em_mu);
  const DevicePlan& dp = plan->dev;
  int rc = em_tiles(plan);
  if (rc) return rc;
  if (!plan->em_planes32[which]) {
    const int np = dp.canon_plus ? kEmPosPlus : kEmPos;
    void* d = plan_alloc(plan, sizeof(float2) * (size_t)dp.dim * np);
    if (!d) return fail(PI_ERR_OUT_OF_MEMORY, "element-major coefficient planes");
    dim3 grid(64, (unsigned)dp.nsectors);
    k_em_planes<float><<<grid, 256, 0, plan->stream>>>(dp.sectors, dp.canon, which ? dp.coef32z : dp.coef32x, np,
                                                       (float2*)d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(plan->stream);
    if (e != cudaSuccess) return cuda_fail(e, "element-major coefficient planes");
    plan->em_planes32[which] = (const float2*)d;
  }
  *planes_out = plan->em_planes32[which];
  return PI_OK;
}

// Tile records of the TMA-staged kernel for tiles of rows x kTmW (one load per block),
// built once per plan and tile height.  Caller holds plan->em_mu.
static int em_tma_tiles(pi_plan* plan, int ri, const TmTile** tiles_out, int* ntiles_out) {
  static constexpr int kRows[3] = {16, 32, 64};
  const DevicePlan& dp = plan->dev;
  if (!plan->em_tma_tiles[ri]) {
    std::vector<DevSector> secs(dp.nsectors);
    cudaError_t e = cudaMemcpy(secs.data(), dp.sectors, sizeof(DevSector) * secs.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "element-major tile list");
    std::vector<TmTile> tiles;
    int loff = 0;
    for (int s = 0; s < dp.nsectors; ++s) {
      const int n = secs[s].n;
      for (int a0 = 0; a0 < n; a0 += kRows[ri])
        for (int b0 = 0; b0 < n; b0 += kTmW) {
          TmTile t{};
          t.offset = secs[s].offset;
          t.sector = s;
          t.a0 = a0;
          t.b0 = b0;
          t.n = n;
          t.s0 = secs[s].src[0];
          t.s2 = secs[s].src[2];
          t.loff = loff;
          tiles.push_back(t);
        }
      loff += n;
    }
    void* d = plan_alloc(plan, sizeof(TmTile) * tiles.size());
    if (!d) return fail(PI_ERR_OUT_OF_MEMORY, "element-major tile list");
    e = cudaMemcpy(d, tiles.data(), sizeof(TmTile) * tiles.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "element-major tile list");
    plan->em_tma_tiles[ri] = d;
    plan->em_tma_ntiles[ri] = (int)tiles.size();
  }
  *tiles_out = (const TmTile*)plan->em_tma_tiles[ri];
  *ntiles_out = plan->em_tma_ntiles[ri];
  return PI_OK;
}

// Builds (once per plan and coefficient set) the split coefficient planes of the TMA-staged
// kernel and the per-sector line offsets of its row and column planes.
static int em_prepare_split(pi_plan* plan, int which, pi_plan::EmSplit* out) {
  std::lock_guard<std::mutex> lk(plan->em_mu);
  const DevicePlan& dp = plan->dev;
  int rc = em_tiles(plan);
  if (rc) return rc;
  if (!plan->em_line_off) {
    std::vector<int> off(plan->host.sectors.size());
    int acc = 0;
    for (size_t s = 0; s < off.size(); ++s) {
      off[s] = acc;
      acc += plan->host.sectors[s].n;
    }
    void* d = plan_alloc(plan, sizeof(int) * off.size());
    if (!d) return fail(PI_ERR_OUT_OF_MEMORY, "element-major line offsets");
    cudaError_t e = cudaMemcpy(d, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "element-major line offsets");
    plan->em_line_off = (const int*)d;
    plan->em_nlines = acc;
  }
  pi_plan::EmSplit& sp = plan->em_split[which];
  if (!sp.eplane) {
    const int ne = dp.canon_plus ? TmCfg<true, 32>::NE : TmCfg<false, 32>::NE;
    void* e_d = plan_alloc(plan, sizeof(float4) * (size_t)dp.dim * ne);
    void* l_d = plan_alloc(plan, sizeof(float4) * (size_t)plan->em_nlines);
    void* r_d = plan_alloc(plan, sizeof(float4) * (size_t)plan->em_nlines);
    if (!e_d || !l_d || !r_d) return fail(PI_ERR_OUT_OF_MEMORY, "element-major coefficient planes");
    dim3 grid(64, (unsigned)dp.nsectors);
    k_em_split_planes<<<grid, 256, 0, plan->stream>>>(dp.sectors, dp.canon, which ? dp.coef32z : dp.coef32x,
                                                      plan->em_line_off, ne, (float4*)e_d, (float4*)l_d, (float4*)r_d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(plan->stream);
    if (e != cudaSuccess) return cuda_fail(e, "element-major coefficient planes");
    sp.eplane = (const float4*)e_d;
    sp.lrow = (const float4*)l_d;
    sp.rcol = (const float4*)r_d;
  }
  if (!sp.srow) {
    const int nf4 = dp.canon_plus ? kSepF4Plus : kSepF4;
    void* sr = plan_alloc(plan, sizeof(float4) * (size_t)plan->em_nlines * nf4);
    void* sc = plan_alloc(plan, sizeof(float4) * (size_t)plan->em_nlines * nf4);
    if (!sr || !sc) return fail(PI_ERR_OUT_OF_MEMORY, "separable line planes");
    dim3 grid(4, (unsigned)dp.nsectors);
    k_sep_planes<<<grid, 128, 0, plan->stream>>>(dp.sectors, dp.canon, which ? dp.coef32z : dp.coef32x,
                                                 plan->em_line_off, nf4, (float4*)sr, (float4*)sc);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(plan->stream);
    if (e != cudaSuccess) return cuda_fail(e, "separable line planes");
    sp.srow = (const float4*)sr;
    sp.scol = (const float4*)sc;
  }
  *out = sp;
  return PI_OK;
}

int em_split_planes(pi_plan* plan, int which, SplitPlanes* out) {
  pi_plan::EmSplit sp;
  const int rc = em_prepare_split(plan, which, &sp);
  if (rc) return rc;
  out->eplane = sp.eplane;
  out->lrow = sp.lrow;
  out->rcol = sp.rcol;
  out->line_off = plan->em_line_off;
  out->plus = plan->dev.canon_plus ? 1 : 0;
  out->srow = sp.srow;
  out->scol = sp.scol;
  return PI_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link-time dependency on
// the driver library); nullptr when the driver does not provide it.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)p;
  }();
  return fn;
}

constexpr int kTmMapsSmall = 64;   // sectors of N <= 126
constexpr int kTmMapsLarge = 160;  // sectors of N <= 318
constexpr size_t kTmMapCache = 4;  // source batches whose maps are kept per plan

// Per-sector tensor maps over the batch x: sector s is the 3-D tensor (right-hand side c <
// ncols, row a < n, column b < n) at x + offset_s * ld with strides (8, 8 ld, 8 ld n) bytes;
// the box is 64 right-hand sides x 1 row x kTmCols columns.  Encoded on the host once per
// (x, ld, ncols) and kept for the last few batches.  Returns nullptr when a map cannot be
// encoded (the caller then uses the kernel with plain loads).
static const unsigned char* em_tensor_maps(pi_plan* plan, const void* x, long long ld, int ncols) {
  std::lock_guard<std::mutex> lk(plan->em_mu);
  for (auto& e : plan->em_maps)
    if (e.x == x && e.ld == ld && e.ncols == ncols) return e.maps.data();
  const auto encode = tensor_map_encoder();
  if (!encode) return nullptr;
  const auto& secs = plan->host.sectors;
  std::vector<unsigned char> blob(secs.size() * sizeof(CUtensorMap));
  for (size_t s = 0; s < secs.size(); ++s) {
    const unsigned long long n = (unsigned long long)secs[s].n;
    const cuuint64_t dims[3] = {(cuuint64_t)ncols, n, n};
    const cuuint64_t strides[2] = {(cuuint64_t)ld * 8, (cuuint64_t)ld * 8 * n};
    const cuuint32_t box[3] = {kTmHalf, 1, kTmCols};
    const cuuint32_t elem[3] = {1, 1, 1};
    CUtensorMap m;
    void* base = (void*)((const char*)x + (size_t)secs[s].offset * (size_t)ld * 8);
    if (encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return nullptr;
    std::memcpy(blob.data() + s * sizeof(CUtensorMap), &m, sizeof(CUtensorMap));
  }
  if (plan->em_maps.size() >= kTmMapCache) plan->em_maps.erase(plan->em_maps.begin());
  plan->em_maps.push_back(pi_plan::EmMapSet{x, ld, ncols, std::move(blob)});
  return plan->em_maps.back().maps.data();
}

template <bool PLUS, int MAXS, int ROWS>
static cudaError_t launch_em_tma(const unsigned char* blob, int nsectors, const TmTile* tiles, int ntiles,
                                 const pi_plan::EmSplit& sp, float4* y, unsigned ld4, int npairs, cudaStream_t s) {
  EmMaps<MAXS> maps;
  std::memset(&maps, 0, sizeof(maps));
  std::memcpy(maps.m, blob, (size_t)nsectors * sizeof(CUtensorMap));
  auto kern = k_apply_em_tma<PLUS, MAXS, ROWS>;
  constexpr int smem = TmCfg<PLUS, ROWS>::SMEM;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)ntiles, (unsigned)((npairs + 31) / 32));
  kern<<<grid, kTmThreads, smem, s>>>(maps, tiles, sp.eplane, sp.lrow, sp.rcol, y, ld4, npairs);
  return cudaGetLastError();
}

template <int MAXS, int ROWS>
static cudaError_t launch_em_tma_rows(bool plus, const unsigned char* blob, int nsectors, const TmTile* tiles,
                                      int ntiles, const pi_plan::EmSplit& sp, float4* y, unsigned ld4, int npairs,
                                      cudaStream_t s) {
  if (plus) {
    if constexpr (ROWS <= 32)  // the pumping variant's entry plane leaves no room for 64-row runs
      return launch_em_tma<true, MAXS, ROWS>(blob, nsectors, tiles, ntiles, sp, y, ld4, npairs, s);
    return cudaErrorInvalidValue;
  }
  return launch_em_tma<false, MAXS, ROWS>(blob, nsectors, tiles, ntiles, sp, y, ld4, npairs, s);
}

// One element-major kernel choice: TMA-staged with tiles of `rows` rows (kind 0), or plain
// loads (kind 1).
struct EmCand {
  int kind;
  int rows;
};

// Runs one candidate.  Returns a PI status.
static int em_run(pi_plan* plan, EmCand c, float* y_dev, const float* x_dev, int ncols, long long ld, int coords,
                  cudaStream_t s) {
  const DevicePlan& dp = plan->dev;
  const int npairs = ncols / 2;
  const unsigned ld4 = (unsigned)(ld / 2);
  float4* y4 = (float4*)y_dev;
  if (c.kind == 0) {
    const unsigned char* maps = em_tensor_maps(plan, x_dev, ld, ncols);
    if (!maps) return fail(PI_ERR_UNSUPPORTED, "element-major tensor maps could not be encoded");
    pi_plan::EmSplit sp;
    int rc = em_prepare_split(plan, coords, &sp);
    if (rc) return rc;
    const int ri = c.rows == 16 ? 0 : c.rows == 32 ? 1 : 2;
    const TmTile* tiles = nullptr;
    int ntiles = 0;
    {
      std::lock_guard<std::mutex> lk(plan->em_mu);
      rc = em_tma_tiles(plan, ri, &tiles, &ntiles);
    }
    if (rc) return rc;
    const bool plus = dp.canon_plus != 0, small = dp.nsectors <= kTmMapsSmall;
    cudaError_t e;
    switch (ri) {
      case 0:
        e = small ? launch_em_tma_rows<kTmMapsSmall, 16>(plus, maps, dp.nsectors, tiles, ntiles, sp, y4, ld4, npairs, s)
                  : launch_em_tma_rows<kTmMapsLarge, 16>(plus, maps, dp.nsectors, tiles, ntiles, sp, y4, ld4, npairs, s);
        break;
      case 1:
        e = small ? launch_em_tma_rows<kTmMapsSmall, 32>(plus, maps, dp.nsectors, tiles, ntiles, sp, y4, ld4, npairs, s)
                  : launch_em_tma_rows<kTmMapsLarge, 32>(plus, maps, dp.nsectors, tiles, ntiles, sp, y4, ld4, npairs, s);
        break;
      default:
        e = small ? launch_em_tma_rows<kTmMapsSmall, 64>(plus, maps, dp.nsectors, tiles, ntiles, sp, y4, ld4, npairs, s)
                  : launch_em_tma_rows<kTmMapsLarge, 64>(plus, maps, dp.nsectors, tiles, ntiles, sp, y4, ld4, npairs, s);
    }
    if (e != cudaSuccess) return cuda_fail(e, "element-major apply launch (TMA)");
    return PI_OK;
  }
  const float2* planes = nullptr;
  int rc = em_prepare(plan, coords, &planes);
  if (rc) return rc;
  BorderArgs border{1.0, nullptr, coords};
  // One right-hand-side pair per lane, 8-warp blocks, 64 registers (4 blocks per SM):
  // measured fastest for plain loads on GB300 for 64..256-column batches.  Two pairs per
  // lane, one pair per lane with 8-byte loads, wider blocks, L2 bulk prefetch and source
  // loads pipelined a row ahead were all slower (the last raises the register count past 64
  // and costs more in occupancy than it saves in latency).
  dim3 grid((unsigned)plan->em_ntiles, (unsigned)((npairs + 31) / 32));
  const float4* x4 = (const float4*)x_dev;
  if (dp.canon_plus)
    k_apply_em_f32<true, 1><<<grid, 32 * kEmWarps, 0, s>>>(dp.sectors, plan->em_tiles, planes, x4, y4, ld4, npairs, border);
  else
    k_apply_em_f32<false, 1><<<grid, 32 * kEmWarps, 0, s>>>(dp.sectors, plan->em_tiles, planes, x4, y4, ld4, npairs, border);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "element-major apply launch");
  return PI_OK;
}

// The candidates for a plan: TMA-staged tiles of 16, 32 and (without pumping terms) 64 rows
// when the plan's tensor maps fit the kernel-parameter table, and plain loads.
static std::vector<EmCand> em_candidates(const pi_plan* plan) {
  std::vector<EmCand> c;
  if (plan->dev.nsectors <= kTmMapsLarge && tensor_map_encoder()) {
    c.push_back({0, 32});
    c.push_back({0, 16});
    if (!plan->dev.canon_plus) c.push_back({0, 64});
  }
  c.push_back({1, 32});
  return c;
}

// Autotuner: the first call for a batch width and coordinate system runs every candidate on
// the caller's batch (all compute each output entry with the same operations, so y is the
// same whichever runs; a candidate that fails to launch drops out), times two rounds of the
// rest with CUDA events on the caller's stream, waits for that stream once, and keeps the
// fastest for later calls.
static int em_tune(pi_plan* plan, float* y_dev, const float* x_dev, int ncols, long long ld, int coords,
                   cudaStream_t s, pi_plan::EmChoice* out) {
  // a candidate that cannot run on this batch (its tensor maps do not encode, say) drops out
  std::vector<EmCand> cands;
  int first_rc = PI_OK;
  for (const EmCand& c : em_candidates(plan)) {
    const int rc = em_run(plan, c, y_dev, x_dev, ncols, ld, coords, s);
    if (rc == PI_OK)
      cands.push_back(c);
    else if (first_rc == PI_OK)
      first_rc = rc;
  }
  if (cands.empty()) return first_rc;
  std::vector<cudaEvent_t> ev(2 * cands.size() * 2, nullptr);
  for (auto& e : ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      for (auto& f : ev)
        if (f) cudaEventDestroy(f);
      return cuda_fail(cudaGetLastError(), "autotuner events");
    }
  int rc = PI_OK;
  for (int round = 0; round < 2 && !rc; ++round)
    for (size_t i = 0; i < cands.size() && !rc; ++i) {
      cudaEventRecord(ev[(round * cands.size() + i) * 2], s);
      rc = em_run(plan, cands[i], y_dev, x_dev, ncols, ld, coords, s);
      cudaEventRecord(ev[(round * cands.size() + i) * 2 + 1], s);
    }
  cudaError_t e = rc ? cudaSuccess : cudaEventSynchronize(ev.back());
  pi_plan::EmChoice best{ncols, coords, 1, 32, 0.0};
  float best_ms = 3.4e38f;
  if (!rc && e == cudaSuccess)
    for (size_t i = 0; i < cands.size(); ++i) {
      float ms = 3.4e38f;
      for (int round = 0; round < 2; ++round) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, ev[(round * cands.size() + i) * 2], ev[(round * cands.size() + i) * 2 + 1]) ==
            cudaSuccess)
          ms = std::min(ms, t);
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = {ncols, coords, cands[i].kind, cands[i].rows, (double)ms};
      }
    }
  for (auto& f : ev) cudaEventDestroy(f);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "autotuner timing");
  *out = best;
  return PI_OK;
}

}  // namespace picuda

using namespace picuda;

extern "C" int pi_apply_f32_em(pi_plan* plan, float* y_dev, const float* x_dev, int ncols, long long ld, int coords,
                               void* stream) {
  if (!plan || !y_dev || !x_dev) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (ncols < 2 || (ncols & 1)) return fail(PI_ERR_INVALID_ARGUMENT, "ncols must be even and at least 2");
  if (ld < ncols || (ld & 1) || ld / 2 > 0x7fffffffLL)
    return fail(PI_ERR_INVALID_ARGUMENT, "ld must be even, at least ncols and below 2^32");
  if (((uintptr_t)x_dev | (uintptr_t)y_dev) & 15)
    return fail(PI_ERR_INVALID_ARGUMENT, "element-major batches must start on a 16-byte boundary");
  if (coords != PI_COORDS_REFERENCE && coords != PI_COORDS_POPULATION)
    return fail(PI_ERR_INVALID_ARGUMENT, "coords must be PI_COORDS_REFERENCE or PI_COORDS_POPULATION");
  const long long span = plan->host.dim * ld * (long long)sizeof(float2);
  const char* xb = (const char*)x_dev;
  const char* yb = (const char*)y_dev;
  if (xb < yb + span && yb < xb + span)
    return fail(PI_ERR_INVALID_ARGUMENT, "source and destination must not share storage");
  if ((unsigned long long)plan->host.dim * (unsigned long long)(ld / 2) >= (1ULL << 32))
    return fail(PI_ERR_UNSUPPORTED, "element-major batch larger than 2^32 16-byte rows; split the batch");
  if (!plan->dev.canon)
    return fail(PI_ERR_UNSUPPORTED,
                "element-major batched apply needs a plan whose stencil sits at the canonical positions "
                "(qubit models with real one-body operators)");
  cudaStream_t s = (cudaStream_t)stream;
  pi_plan::EmChoice ch{};
  bool known = false;
  {
    std::lock_guard<std::mutex> lk(plan->em_mu);
    for (const auto& c : plan->em_choices)
      if (c.ncols == ncols && c.coords == coords) {
        ch = c;
        known = true;
      }
  }
  if (!known) {
    std::lock_guard<std::mutex> tl(plan->em_tune_mu);  // one tuning pass per key
    {
      std::lock_guard<std::mutex> lk(plan->em_mu);
      for (const auto& c : plan->em_choices)
        if (c.ncols == ncols && c.coords == coords) {
          ch = c;
          known = true;
        }
    }
    if (!known) {
      int rc = em_tune(plan, y_dev, x_dev, ncols, ld, coords, s, &ch);
      if (rc) return rc;
      std::lock_guard<std::mutex> lk(plan->em_mu);
      plan->em_choices.push_back(ch);
      return PI_OK;  // y already holds L x from the timed runs
    }
  }
  return em_run(plan, EmCand{ch.kind, ch.rows}, y_dev, x_dev, ncols, ld, coords, s);
}

extern "C" int pi_apply_f32_em_tuning(pi_plan* plan, int ncols, int coords, int* kind, int* rows, double* ms) {
  if (!plan || !kind || !rows || !ms) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(plan->em_mu);
  for (const auto& c : plan->em_choices)
    if (c.ncols == ncols && c.coords == coords) {
      *kind = c.kind;
      *rows = c.rows;
      *ms = c.ms;
      return PI_OK;
    }
  return fail(PI_ERR_INVALID_ARGUMENT, "no element-major apply with this width and coordinate system has run yet");
}

extern "C" int pi_apply_f32_em_select(pi_plan* plan, int ncols, int coords, int kind, int rows) {
  if (!plan) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (coords != PI_COORDS_REFERENCE && coords != PI_COORDS_POPULATION)
    return fail(PI_ERR_INVALID_ARGUMENT, "coords must be PI_COORDS_REFERENCE or PI_COORDS_POPULATION");
  bool listed = false;
  for (const EmCand& c : em_candidates(plan)) listed = listed || (c.kind == kind && (kind == 1 || c.rows == rows));
  if (!listed) return fail(PI_ERR_INVALID_ARGUMENT, "this element-major kernel choice is not available for the plan");
  std::lock_guard<std::mutex> lk(plan->em_mu);
  pi_plan::EmChoice ch{ncols, coords, kind, kind == 1 ? 32 : rows, 0.0};
  for (auto& c : plan->em_choices)
    if (c.ncols == ncols && c.coords == coords) {
      c = ch;
      return PI_OK;
    }
  plan->em_choices.push_back(ch);
  return PI_OK;
}
