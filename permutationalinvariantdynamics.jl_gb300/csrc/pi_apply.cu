// Fused Schur-block Liouvillian action y = L x on sm_103a.
//
// Replaces the reference's fused static kernel apply (src/liouvillian.jl:3070-3105), which
// copies every sector into dense scratch (:2952-2958) and runs sparse x dense products for
// the Hamiltonian commutator, the loss anticommutator and the collective gains plus the
// support-path sandwich loops of the one-body gains (:2486-2561).  Here every output entry
// (j, m, m') is produced once, as a gather over the separable stencil terms of its sector:
// no scratch copies, one read stream of x (the neighbouring sectors j +- 1 are served from
// L1/L2) and one write of y.
//
// Work layout: a block owns a 32 x 32 tile of one sector block; lane = row (coalesced,
// column-major blocks), warp = 4 consecutive columns.  The block first stages, for each of
// the (at most three) source sectors j, j +- 1, the zero-padded 36 x 36 window of x that
// the tile's stencil reaches, plus the sector's term list grouped by (kind, class); every
// term then reads shared memory without bounds checks in one branch-free loop per group,
// and the alpha[a] coefficient of a term is reused across the thread's 4 columns.  The
// same kernel serves the plain FP64 path and the FP32 path (reference or population
// coordinates).  TMA is not used for the staging: the reference's packed column-major
// blocks have odd leading dimensions (n = N - 2k + 1), so FP32 rows are not 16-byte
// strided as tensor maps require.
#include <algorithm>

#include "pi_device.cuh"
#include "pi_internal.hpp"

namespace picuda {

template <typename T>
struct Vec2;
template <>
struct Vec2<double> {
  using type = double2;
};
template <>
struct Vec2<float> {
  using type = float2;
};

enum Kind { K_ADD, K_LEFT, K_RIGHT, K_SAND };
enum Cls { C_RE, C_IM, C_CX };

template <typename T>
struct Acc {
  T re[kColsPerThread];
  T im[kColsPerThread];
};

// beta[b0 .. b0+3] of one term: b0 and every beta array start are multiples of 4, so the
// four coefficients are read with aligned vector loads.
__device__ __forceinline__ void load4(const float2* p, float2 (&v)[4]) {
  const float4 u0 = __ldg(reinterpret_cast<const float4*>(p));
  const float4 u1 = __ldg(reinterpret_cast<const float4*>(p) + 1);
  v[0] = make_float2(u0.x, u0.y);
  v[1] = make_float2(u0.z, u0.w);
  v[2] = make_float2(u1.x, u1.y);
  v[3] = make_float2(u1.z, u1.w);
}
__device__ __forceinline__ void load4(const double2* p, double2 (&v)[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = __ldg(p + k);
}

// One stencil term for the thread's row and 4 columns, reading the zero-padded source
// windows in shared memory (no bounds checks).  ca points at coef + a, cb at coef + b0.
template <typename T, typename T2, int KIND, int CLS>
__device__ __forceinline__ void term(const int4 tm, const T2* __restrict__ ca, const T2* __restrict__ cb,
                                     const T2* wbase, Acc<T>& acc) {
  T2 al;
  if (KIND != K_RIGHT) al = __ldg(ca + tm.y);
  T2 be[4];
  if (KIND != K_LEFT) load4(cb + tm.z, be);
  const T2* wp = wbase + tm.x;
#pragma unroll
  for (int k = 0; k < kColsPerThread; ++k) {
    const T2 xv = wp[k * kWinRows];
    T cr, ci;  // combined coefficient
    if (KIND == K_ADD) {
      cr = al.x + be[k].x;
      ci = al.y + be[k].y;
    } else if (KIND == K_LEFT) {
      cr = al.x;
      ci = al.y;
    } else if (KIND == K_RIGHT) {
      cr = be[k].x;
      ci = be[k].y;
    } else if (CLS == C_RE) {
      cr = al.x * be[k].x;
      ci = 0;
    } else {
      cr = al.x * be[k].x - al.y * be[k].y;
      ci = al.x * be[k].y + al.y * be[k].x;
    }
    if (CLS == C_RE && KIND != K_ADD) {
      acc.re[k] = fma(cr, xv.x, acc.re[k]);
      acc.im[k] = fma(cr, xv.y, acc.im[k]);
    } else if (CLS == C_IM && KIND != K_ADD) {
      acc.re[k] = fma(-ci, xv.y, acc.re[k]);
      acc.im[k] = fma(ci, xv.x, acc.im[k]);
    } else {
      acc.re[k] = fma(cr, xv.x, acc.re[k]);
      acc.re[k] = fma(-ci, xv.y, acc.re[k]);
      acc.im[k] = fma(cr, xv.y, acc.im[k]);
      acc.im[k] = fma(ci, xv.x, acc.im[k]);
    }
  }
}

template <typename T, typename T2, int KIND, int CLS>
__device__ __forceinline__ void group(const int4* st, int g0, int g1, const T2* __restrict__ ca,
                                      const T2* __restrict__ cb, const T2* wbase, Acc<T>& acc) {
  for (int t = g0; t < g1; ++t) term<T, T2, KIND, CLS>(st[t], ca, cb, wbase, acc);
}

// Asynchronous global -> shared copies (cp.async) with hardware zero fill: a source size of
// 0 writes zeros and reads nothing, which pads the halo and the block edges for free.
template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int sz = valid ? BYTES : 0;
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gmem), "n"(BYTES), "r"(sz)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Shared-memory state of one pipeline stage: the three source windows of a work item, its
// sector's grouped term list and group boundaries.
template <typename T2>
struct Stage {
  T2 win[3 * kWinElems];
  int4 st[kMaxSectorTerms];
  int ge[G_COUNT + 1];
};

// Issues the copies of work item `item` = (tile, column) into stage `S` (cp.async for the
// windows, plain loads for the term list) and commits one cp.async group.
template <typename T2>
__device__ __forceinline__ void issue_stage(Stage<T2>& S, const DevSector* __restrict__ sectors,
                                            const DevTerm* __restrict__ terms, const DevTile* __restrict__ tiles,
                                            const T2* __restrict__ x, long long ld, int ncols, int item) {
  const int tile_id = item / ncols;
  const int col = item - tile_id * ncols;
  const DevTile tile = tiles[tile_id];
  const DevSector& sec = sectors[tile.sector];
  const T2* xc = x + (long long)col * ld;
  const int la = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll 1
  for (int slot = 0; slot < 3; ++slot) {
    const int s2 = sec.src[slot];
    if (s2 < 0) continue;
    const int m = sectors[s2].n;
    const T2* xs = xc + sectors[s2].offset;
    const int r0 = tile.a0 + slot - 1 - kHalo, c0 = tile.b0 + slot - 1 - kHalo;
    T2* w = S.win + slot * kWinElems;
    const int R = r0 + la, R2 = r0 + 32 + la;
    const bool rv = (unsigned)R < (unsigned)m;
    const bool extra = la < kWinRows - 32;
    const bool rv2 = extra && (unsigned)R2 < (unsigned)m;
    for (int j = warp; j < kWinCols; j += kApplyWarps) {
      const int C = c0 + j;
      const bool cv = (unsigned)C < (unsigned)m;
      const bool v1 = rv && cv, v2 = rv2 && cv;
      cp_async_zfill<sizeof(T2)>(w + la + j * kWinRows, v1 ? xs + R + C * m : xs, v1);
      if (extra) cp_async_zfill<sizeof(T2)>(w + 32 + la + j * kWinRows, v2 ? xs + R2 + C * m : xs, v2);
    }
  }
  cp_async_commit();
  const int tb = sec.term_begin;
  const int nt = sec.group_end[G_COUNT - 1] - tb;
  for (int i = threadIdx.x; i < nt; i += blockDim.x) S.st[i] = reinterpret_cast<const int4*>(terms)[tb + i];
  if (threadIdx.x <= G_COUNT) S.ge[threadIdx.x] = threadIdx.x == 0 ? 0 : sec.group_end[threadIdx.x - 1] - tb;
}

// Persistent apply: each block walks a contiguous range of work items (tile-major, column
// minor, so one tile is reused across many right-hand sides) with a two-stage cp.async
// pipeline -- the windows of item i+1 are in flight while item i is computed.
template <typename T>
__global__ void __launch_bounds__(kApplyThreads)
    k_apply(const DevSector* __restrict__ sectors, const DevTerm* __restrict__ terms,
            const typename Vec2<T>::type* __restrict__ coef, const DevTile* __restrict__ tiles, int ntiles,
            int ncols, const typename Vec2<T>::type* __restrict__ x, typename Vec2<T>::type* __restrict__ y,
            long long ld, BorderArgs border) {
  using T2 = typename Vec2<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Stage<T2>* stages = reinterpret_cast<Stage<T2>*>(smem_raw);
  const long long total = (long long)ntiles * ncols;
  const int begin = (int)((long long)blockIdx.x * total / gridDim.x);
  const int end = (int)((long long)(blockIdx.x + 1) * total / gridDim.x);
  if (begin >= end) return;
  const int la = threadIdx.x & 31;
  const int lb = (threadIdx.x >> 5) * kColsPerThread;
  issue_stage<T2>(stages[0], sectors, terms, tiles, x, ld, ncols, begin);
  for (int item = begin; item < end; ++item) {
    const int buf = (item - begin) & 1;
    if (item + 1 < end)
      issue_stage<T2>(stages[buf ^ 1], sectors, terms, tiles, x, ld, ncols, item + 1);
    else
      cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const Stage<T2>& S = stages[buf];
    const int tile_id = item / ncols;
    const int col = item - tile_id * ncols;
    const DevTile tile = tiles[tile_id];
    const DevSector& sec = sectors[tile.sector];
    const int n = sec.n;
    const int a = tile.a0 + la;
    const int b0 = tile.b0 + lb;
    if (a < n && b0 < n) {
      const int ncol = min(kColsPerThread, n - b0);
      Acc<T> acc;
#pragma unroll
      for (int k = 0; k < kColsPerThread; ++k) acc.re[k] = acc.im[k] = 0;
      const T2* ca = coef + a;
      const T2* cb = coef + b0;
      const T2* wbase = S.win + (la + kHalo) + (lb + kHalo) * kWinRows;  // + woff selects slot, p, q
      const int4* st = S.st;
      group<T, T2, K_ADD, C_CX>(st, S.ge[G_ADD], S.ge[G_ADD + 1], ca, cb, wbase, acc);
      group<T, T2, K_LEFT, C_IM>(st, S.ge[G_LEFT_IM], S.ge[G_LEFT_IM + 1], ca, cb, wbase, acc);
      group<T, T2, K_LEFT, C_RE>(st, S.ge[G_LEFT_RE], S.ge[G_LEFT_RE + 1], ca, cb, wbase, acc);
      group<T, T2, K_LEFT, C_CX>(st, S.ge[G_LEFT_CX], S.ge[G_LEFT_CX + 1], ca, cb, wbase, acc);
      group<T, T2, K_RIGHT, C_IM>(st, S.ge[G_RIGHT_IM], S.ge[G_RIGHT_IM + 1], ca, cb, wbase, acc);
      group<T, T2, K_RIGHT, C_RE>(st, S.ge[G_RIGHT_RE], S.ge[G_RIGHT_RE + 1], ca, cb, wbase, acc);
      group<T, T2, K_RIGHT, C_CX>(st, S.ge[G_RIGHT_CX], S.ge[G_RIGHT_CX + 1], ca, cb, wbase, acc);
      group<T, T2, K_SAND, C_RE>(st, S.ge[G_SAND_RE], S.ge[G_SAND_RE + 1], ca, cb, wbase, acc);
      group<T, T2, K_SAND, C_CX>(st, S.ge[G_SAND_CX], S.ge[G_SAND_CX + 1], ca, cb, wbase, acc);
      if (border.scale != 1.0) {
        const T scale = (T)border.scale;
#pragma unroll
        for (int k = 0; k < kColsPerThread; ++k) {
          acc.re[k] *= scale;
          acc.im[k] *= scale;
        }
      }
      T2* yp = y + (long long)col * ld + sec.offset + a + (long long)b0 * n;
#pragma unroll
      for (int k = 0; k < kColsPerThread; ++k) {
        if (k >= ncol) break;
        T2 out;
        out.x = acc.re[k];
        out.y = acc.im[k];
        if (b0 + k == a && border.alpha != nullptr) {
          const double2 al = border.alpha[col];
          const double v = border.coords ? sec.border_z : sec.border_x;
          out.x += (T)(al.x * v);
          out.y += (T)(al.y * v);
        }
        yp[(long long)k * n] = out;
      }
    }
    __syncthreads();  // every thread is done with stage `buf` before it is refilled
  }
}

template <typename T>
cudaError_t launch_apply_t(const DevicePlan& dp, const void* coef, const void* x, void* y, int ncols,
                           long long ld, const BorderArgs& border, cudaStream_t stream) {
  using T2 = typename Vec2<T>::type;
  if (dp.ntiles == 0 || ncols == 0) return cudaSuccess;
  const size_t smem = 2 * sizeof(Stage<T2>);
  static int blocks_per_sm = 0;  // per template instance; the kernel and device are fixed
  static int sms = 0;
  if (blocks_per_sm == 0) {
    cudaError_t e = cudaFuncSetAttribute(k_apply<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int occ = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_apply<T>, kApplyThreads, smem);
    if (e != cudaSuccess) return e;
    blocks_per_sm = occ > 0 ? occ : 1;
  }
  const long long total = (long long)dp.ntiles * ncols;
  const long long grid = std::min<long long>(total, (long long)sms * blocks_per_sm);
  k_apply<T><<<(unsigned)grid, kApplyThreads, smem, stream>>>(dp.sectors, dp.terms, (const T2*)coef, dp.tiles,
                                                               dp.ntiles, ncols, (const T2*)x, (T2*)y, ld, border);
  return cudaGetLastError();
}

cudaError_t launch_apply_f64(const DevicePlan& dp, const double* x, double* y, int ncols, long long ld,
                             const BorderArgs& border, cudaStream_t stream) {
  return launch_apply_t<double>(dp, dp.coef64, x, y, ncols, ld, border, stream);
}

cudaError_t launch_apply_f32(const DevicePlan& dp, const float* x, float* y, int ncols, long long ld,
                             const BorderArgs& border, cudaStream_t stream) {
  return launch_apply_t<float>(dp, border.coords ? dp.coef32z : dp.coef32x, x, y, ncols, ld, border, stream);
}

}  // namespace picuda
