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

// One stencil term for the thread's row la and columns lb .. lb+3 of the tile, reading the
// zero-padded source window in shared memory (no bounds checks).
template <typename T, typename T2, int KIND, int CLS>
__device__ __forceinline__ void term(const DevTerm& tm, const T2* __restrict__ coef, const T2* win, int a,
                                     int la, int lb, int b0, int nm1, Acc<T>& acc) {
  T2 al;
  if (KIND != K_RIGHT) al = __ldg(coef + tm.alpha_off + a);
  const T2* wp = win + tm.slot * kWinElems + (la + tm.p + kHalo) + (lb + tm.q + kHalo) * kWinRows;
#pragma unroll
  for (int k = 0; k < kColsPerThread; ++k) {
    const T2 xv = wp[k * kWinRows];
    T2 be;
    if (KIND != K_LEFT) be = __ldg(coef + tm.beta_off + min(b0 + k, nm1));
    T cr, ci;  // combined coefficient
    if (KIND == K_ADD) {
      cr = al.x + be.x;
      ci = al.y + be.y;
    } else if (KIND == K_LEFT) {
      cr = al.x;
      ci = al.y;
    } else if (KIND == K_RIGHT) {
      cr = be.x;
      ci = be.y;
    } else if (CLS == C_RE) {
      cr = al.x * be.x;
      ci = 0;
    } else {
      cr = al.x * be.x - al.y * be.y;
      ci = al.x * be.y + al.y * be.x;
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
__device__ __forceinline__ void group(const DevTerm* st, int g0, int g1, const T2* __restrict__ coef, const T2* win,
                                      int a, int la, int lb, int b0, int nm1, Acc<T>& acc) {
  for (int t = g0; t < g1; ++t) term<T, T2, KIND, CLS>(st[t], coef, win, a, la, lb, b0, nm1, acc);
}

template <typename T>
__global__ void __launch_bounds__(kApplyThreads)
    k_apply(const DevSector* __restrict__ sectors, const DevTerm* __restrict__ terms,
            const typename Vec2<T>::type* __restrict__ coef, const DevTile* __restrict__ tiles,
            const typename Vec2<T>::type* __restrict__ x, typename Vec2<T>::type* __restrict__ y,
            long long ld, BorderArgs border) {
  using T2 = typename Vec2<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* win = reinterpret_cast<T2*>(smem_raw);  // [3][kWinElems] source windows
  __shared__ DevTerm st[kMaxSectorTerms];
  __shared__ int ge[G_COUNT + 1];
  const DevTile tile = tiles[blockIdx.x];
  const DevSector& sec = sectors[tile.sector];
  const long long col = blockIdx.y;
  x += col * ld;
  y += col * ld;
  const int tb = sec.term_begin;
  const int nt = sec.group_end[G_COUNT - 1] - tb;
  for (int i = threadIdx.x; i < nt; i += blockDim.x) st[i] = terms[tb + i];
  if (threadIdx.x <= G_COUNT) ge[threadIdx.x] = threadIdx.x == 0 ? 0 : sec.group_end[threadIdx.x - 1] - tb;
  // Stage the zero-padded windows x_src[a0+e-2 .. a0+e+33, b0+e-2 .. b0+e+33] of every
  // source sector (e = -1, 0, +1).
#pragma unroll 1
  for (int slot = 0; slot < 3; ++slot) {
    const int s2 = sec.src[slot];
    if (s2 < 0) continue;
    const int m = sectors[s2].n;
    const T2* xs = x + sectors[s2].offset;
    const int r0 = tile.a0 + slot - 1 - kHalo, c0 = tile.b0 + slot - 1 - kHalo;
    T2* w = win + slot * kWinElems;
    for (int idx = threadIdx.x; idx < kWinElems; idx += blockDim.x) {
      const int i = idx % kWinRows, j = idx / kWinRows;
      const int R = r0 + i, C = c0 + j;
      T2 v;
      v.x = 0;
      v.y = 0;
      if ((unsigned)R < (unsigned)m && (unsigned)C < (unsigned)m) v = __ldg(xs + R + C * m);
      w[idx] = v;
    }
  }
  __syncthreads();
  const int n = sec.n;
  const int la = threadIdx.x & 31;
  const int lb = (threadIdx.x >> 5) * kColsPerThread;
  const int a = tile.a0 + la;
  const int b0 = tile.b0 + lb;
  if (a >= n || b0 >= n) return;
  const int ncol = min(kColsPerThread, n - b0);
  const int nm1 = n - 1;
  Acc<T> acc;
#pragma unroll
  for (int k = 0; k < kColsPerThread; ++k) acc.re[k] = acc.im[k] = 0;
  group<T, T2, K_ADD, C_CX>(st, ge[G_ADD], ge[G_ADD + 1], coef, win, a, la, lb, b0, nm1, acc);
  group<T, T2, K_LEFT, C_IM>(st, ge[G_LEFT_IM], ge[G_LEFT_IM + 1], coef, win, a, la, lb, b0, nm1, acc);
  group<T, T2, K_LEFT, C_RE>(st, ge[G_LEFT_RE], ge[G_LEFT_RE + 1], coef, win, a, la, lb, b0, nm1, acc);
  group<T, T2, K_LEFT, C_CX>(st, ge[G_LEFT_CX], ge[G_LEFT_CX + 1], coef, win, a, la, lb, b0, nm1, acc);
  group<T, T2, K_RIGHT, C_IM>(st, ge[G_RIGHT_IM], ge[G_RIGHT_IM + 1], coef, win, a, la, lb, b0, nm1, acc);
  group<T, T2, K_RIGHT, C_RE>(st, ge[G_RIGHT_RE], ge[G_RIGHT_RE + 1], coef, win, a, la, lb, b0, nm1, acc);
  group<T, T2, K_RIGHT, C_CX>(st, ge[G_RIGHT_CX], ge[G_RIGHT_CX + 1], coef, win, a, la, lb, b0, nm1, acc);
  group<T, T2, K_SAND, C_RE>(st, ge[G_SAND_RE], ge[G_SAND_RE + 1], coef, win, a, la, lb, b0, nm1, acc);
  group<T, T2, K_SAND, C_CX>(st, ge[G_SAND_CX], ge[G_SAND_CX + 1], coef, win, a, la, lb, b0, nm1, acc);
  const T scale = (T)border.scale;
  T2* yp = y + sec.offset + a + (long long)b0 * n;
#pragma unroll
  for (int k = 0; k < kColsPerThread; ++k) {
    if (k >= ncol) break;
    T2 out;
    out.x = scale * acc.re[k];
    out.y = scale * acc.im[k];
    if (b0 + k == a && border.alpha != nullptr) {
      const double2 al = border.alpha[col];
      const double v = border.coords ? sec.border_z : sec.border_x;
      out.x += (T)(al.x * v);
      out.y += (T)(al.y * v);
    }
    yp[(long long)k * n] = out;
  }
}

template <typename T>
cudaError_t launch_apply_t(const DevicePlan& dp, const void* coef, const void* x, void* y, int ncols,
                           long long ld, const BorderArgs& border, cudaStream_t stream) {
  using T2 = typename Vec2<T>::type;
  if (dp.ntiles == 0 || ncols == 0) return cudaSuccess;
  const size_t smem = 3 * kWinElems * sizeof(T2);
  static bool configured = false;  // per template instance, host side
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_apply<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  dim3 grid((unsigned)dp.ntiles, (unsigned)ncols);
  k_apply<T><<<grid, kApplyThreads, smem, stream>>>(dp.sectors, dp.terms, (const T2*)coef, dp.tiles,
                                                    (const T2*)x, (T2*)y, ld, border);
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
