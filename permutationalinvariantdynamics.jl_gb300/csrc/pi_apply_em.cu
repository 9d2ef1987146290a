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
    for (int k = 0; k < np; ++k) {
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
      out[k] = v;
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
__device__ __forceinline__ float4 take(const float4* __restrict__ x, const Stream& s) {
  if (s.col_ok && (unsigned)s.row < (unsigned)s.m) return __ldg(x + s.idx);
  return make_float4(0.f, 0.f, 0.f, 0.f);
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

}  // namespace

// Builds (once per plan and coefficient set) the element-major tile list and the merged
// coefficient planes.  which: 0 FP32 reference coordinates, 1 FP32 population coordinates.
static int em_prepare(pi_plan* plan, int which, const float2** planes_out) {
  std::lock_guard<std::mutex> lk(plan->em_mu);
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
  const float2* planes = nullptr;
  int rc = em_prepare(plan, coords, &planes);
  if (rc) return rc;
  const DevicePlan& dp = plan->dev;
  const int npairs = ncols / 2;
  BorderArgs border{1.0, nullptr, coords};
  cudaStream_t s = (cudaStream_t)stream;
  // One right-hand-side pair per lane, 8-warp blocks, 64 registers (4 blocks per SM):
  // measured fastest on GB300 for 64..256-column batches.  Two pairs per lane, one pair per
  // lane with 8-byte loads, wider blocks, L2 bulk prefetch and source loads pipelined a row
  // ahead were all slower (the last raises the register count past 64 and costs more in
  // occupancy than it saves in latency).
  dim3 grid((unsigned)plan->em_ntiles, (unsigned)((npairs + 31) / 32));
  const float4* x4 = (const float4*)x_dev;
  float4* y4 = (float4*)y_dev;
  const unsigned ld4 = (unsigned)(ld / 2);
  if (dp.canon_plus)
    k_apply_em_f32<true, 1><<<grid, 32 * kEmWarps, 0, s>>>(dp.sectors, plan->em_tiles, planes, x4, y4, ld4, npairs, border);
  else
    k_apply_em_f32<false, 1><<<grid, 32 * kEmWarps, 0, s>>>(dp.sectors, plan->em_tiles, planes, x4, y4, ld4, npairs, border);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "element-major apply launch");
  return PI_OK;
}
