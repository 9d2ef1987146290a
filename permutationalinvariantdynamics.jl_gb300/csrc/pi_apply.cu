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

#include "pi_apply_impl.cuh"
#include "pi_device.cuh"
#include "pi_internal.hpp"

namespace picuda {

template <typename T>
__global__ void __launch_bounds__(kApplyThreads)
    k_apply(const DevSector* __restrict__ sectors, const DevTerm* __restrict__ terms,
            const typename Vec2<T>::type* __restrict__ coef, const DevTile* __restrict__ tiles,
            const typename Vec2<T>::type* __restrict__ x, typename Vec2<T>::type* __restrict__ y,
            long long ld, BorderArgs border) {
  using T2 = typename Vec2<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* win = reinterpret_cast<T2*>(smem_raw);  // [3][kWinElems] source windows
  __shared__ int4 st[kMaxSectorTerms];
  __shared__ int ge[G_COUNT + 1];
  const long long col = blockIdx.y;
  apply_tile<T>(sectors, terms, coef, tiles[blockIdx.x], x + col * ld, y + col * ld, border,
                border.alpha != nullptr ? border.alpha + col : nullptr, win, st, ge);
}

// ---------------------------------------------------------------------------------------
// Batched apply for stencils made of one ADD term, LEFT/RIGHT terms with imaginary
// coefficients (the Hamiltonian off-diagonals) and real sandwich terms (collective and local
// gains) -- every qubit model with real one-body operators and diagonal losses.  The term
// counts are compile-time (sectors with fewer terms are padded with zero terms on the host),
// so each thread keeps its coefficient products alpha[a]*beta[b] in registers and reuses them
// for a chunk of right-hand sides; only the x windows stream through a two-stage cp.async
// pipeline.  Per output entry and right-hand side this leaves one shared load and two FMAs
// per term.
// ---------------------------------------------------------------------------------------
template <typename T, int LI, int RI, int SR>
__global__ void __launch_bounds__(kApplyThreads, sizeof(T) == 4 ? 2 : 1)
    k_apply_rhs(const DevSector* __restrict__ sectors, const int4* __restrict__ fterms,
                const typename Vec2<T>::type* __restrict__ coef, const DevTile* __restrict__ tiles, int ntiles,
                int ncols, int rc, const typename Vec2<T>::type* __restrict__ x, typename Vec2<T>::type* __restrict__ y,
                long long ld, BorderArgs border) {
  using T2 = typename Vec2<T>::type;
  constexpr int NT = 1 + LI + RI + SR;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* win = reinterpret_cast<T2*>(smem_raw);  // [2][3 * kWinElems]
  const int chunk = blockIdx.x / ntiles;
  const int tile_id = blockIdx.x - chunk * ntiles;
  const int c0 = chunk * rc, c1 = min(c0 + rc, ncols);
  const DevTile tile = tiles[tile_id];
  const DevSector& sec = sectors[tile.sector];
  const int n = sec.n;
  const int la = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int lb = warp * kColsPerThread;
  const int a = tile.a0 + la;
  const int b0 = tile.b0 + lb;
  const bool active = a < n && b0 < n;
  const int ac = active ? a : 0, bq = active ? b0 : 0;

  // Coefficients of the sector's terms for this thread's entries, kept in registers.
  const int4* tt = fterms + (long long)tile.sector * NT;
  int woff[NT];
  T car[4], cai[4], lim[LI > 0 ? LI : 1], rim[RI > 0 ? RI : 1][4], sre[SR > 0 ? SR : 1][4];
  {
    const int4 t = tt[0];
    woff[0] = t.x;
    const T2 al = __ldg(coef + t.y + ac);
    T2 be[4];
    load4(coef + t.z + bq, be);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      car[k] = al.x + be[k].x;
      cai[k] = al.y + be[k].y;
    }
  }
#pragma unroll
  for (int i = 0; i < LI; ++i) {
    const int4 t = tt[1 + i];
    woff[1 + i] = t.x;
    lim[i] = __ldg(coef + t.y + ac).y;
  }
#pragma unroll
  for (int i = 0; i < RI; ++i) {
    const int4 t = tt[1 + LI + i];
    woff[1 + LI + i] = t.x;
    T2 be[4];
    load4(coef + t.z + bq, be);
#pragma unroll
    for (int k = 0; k < 4; ++k) rim[i][k] = be[k].y;
  }
#pragma unroll
  for (int i = 0; i < SR; ++i) {
    const int4 t = tt[1 + LI + RI + i];
    woff[1 + LI + RI + i] = t.x;
    const T al = __ldg(coef + t.y + ac).x;
    T2 be[4];
    load4(coef + t.z + bq, be);
#pragma unroll
    for (int k = 0; k < 4; ++k) sre[i][k] = al * be[k].x;
  }

  // Staging plan of this thread, fixed for the tile: rows la and 32 + la of window columns
  // warp, warp + 8, ..., of each source window.  Validity is a bitmask and the source
  // pointers advance by a constant per column, so staging one right-hand side costs a
  // pointer bump and one cp.async per element.
  constexpr int kIters = (kWinCols + kApplyWarps - 1) / kApplyWarps;  // 5
  const bool extra = la < kWinRows - 32;
  unsigned long long vmask = 0;
  long long gbase[3];
  int gstep[3];
  bool have[3];
#pragma unroll
  for (int slot = 0; slot < 3; ++slot) {
    const int s2 = sec.src[slot];
    have[slot] = s2 >= 0;
    const int m = have[slot] ? sectors[s2].n : 0;
    const int R = tile.a0 + slot - 1 - kHalo + la;
    const int C0 = tile.b0 + slot - 1 - kHalo + warp;
    gbase[slot] = (have[slot] ? sectors[s2].offset : 0) + R + (long long)C0 * m;
    gstep[slot] = kApplyWarps * m;
    const bool rv = (unsigned)R < (unsigned)m, rv2 = extra && (unsigned)(R + 32) < (unsigned)m;
#pragma unroll
    for (int it = 0; it < kIters; ++it) {
      const int j = warp + it * kApplyWarps;
      const bool cv = j < kWinCols && (unsigned)(C0 + it * kApplyWarps) < (unsigned)m;
      if (rv && cv) vmask |= 1ull << (slot * 2 * kIters + 2 * it);
      if (rv2 && cv) vmask |= 1ull << (slot * 2 * kIters + 2 * it + 1);
    }
  }
  auto stage = [&](int col, T2* w) {
    const T2* xc = x + (long long)col * ld;
#pragma unroll
    for (int slot = 0; slot < 3; ++slot) {
      if (!have[slot]) continue;
      const T2* g = xc + gbase[slot];
      T2* ws = w + slot * kWinElems + la + warp * kWinRows;
#pragma unroll
      for (int it = 0; it < kIters; ++it) {
        if (warp + it * kApplyWarps < kWinCols) {
          const bool v1 = (vmask >> (slot * 2 * kIters + 2 * it)) & 1ull;
          const bool v2 = (vmask >> (slot * 2 * kIters + 2 * it + 1)) & 1ull;
          cp_async_zfill<sizeof(T2)>(ws, v1 ? g : xc, v1);
          if (extra) cp_async_zfill<sizeof(T2)>(ws + 32, v2 ? g + 32 : xc, v2);
        }
        g += gstep[slot];
        ws += kApplyWarps * kWinRows;
      }
    }
    cp_async_commit();
  };

  // FP64 comparisons and conversions run on GB300's narrow FP64 pipe: decide once per block
  const bool do_scale = border.scale != 1.0;
  const T scale = (T)border.scale;
  const bool has_border = border.alpha != nullptr;
  const bool diag_tile = tile.a0 == tile.b0;
  stage(c0, win);
  for (int col = c0; col < c1; ++col) {
    const int buf = (col - c0) & 1;
    if (col + 1 < c1)
      stage(col + 1, win + (buf ^ 1) * 3 * kWinElems);
    else
      cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    if (active) {
      const T2* wb = win + buf * 3 * kWinElems + (la + kHalo) + (lb + kHalo) * kWinRows;
      T accr[4], acci[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const T2 xv = wb[woff[0] + k * kWinRows];
        accr[k] = car[k] * xv.x - cai[k] * xv.y;
        acci[k] = car[k] * xv.y + cai[k] * xv.x;
      }
#pragma unroll
      for (int i = 0; i < LI; ++i) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const T2 xv = wb[woff[1 + i] + k * kWinRows];
          accr[k] = fma(-lim[i], xv.y, accr[k]);
          acci[k] = fma(lim[i], xv.x, acci[k]);
        }
      }
#pragma unroll
      for (int i = 0; i < RI; ++i) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const T2 xv = wb[woff[1 + LI + i] + k * kWinRows];
          accr[k] = fma(-rim[i][k], xv.y, accr[k]);
          acci[k] = fma(rim[i][k], xv.x, acci[k]);
        }
      }
#pragma unroll
      for (int i = 0; i < SR; ++i) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const T2 xv = wb[woff[1 + LI + RI + i] + k * kWinRows];
          accr[k] = fma(sre[i][k], xv.x, accr[k]);
          acci[k] = fma(sre[i][k], xv.y, acci[k]);
        }
      }
      if (do_scale) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          accr[k] *= scale;
          acci[k] *= scale;
        }
      }
      T2* yp = y + (long long)col * ld + sec.offset + a + (long long)b0 * n;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (b0 + k >= n) break;
        T2 out;
        out.x = accr[k];
        out.y = acci[k];
        if (has_border && diag_tile && b0 + k == a) {
          const double2 al = border.alpha[col];
          const double v = border.coords ? sec.border_z : sec.border_x;
          out.x += (T)(al.x * v);
          out.y += (T)(al.y * v);
        }
        yp[(long long)k * n] = out;
      }
    }
    __syncthreads();  // stage `buf` is refilled two columns later
  }
}

// ---------------------------------------------------------------------------------------
// Batched apply with register reuse over canonical stencil positions.  For the qubit
// models with real one-body operators every term of a sector sits at one of a few window
// positions: the ADD centre, imaginary LEFT at row shifts -1/+1, imaginary RIGHT at column
// shifts -1/+1, and real sandwich terms on the diagonal shifts -1, 0, +1 of the three source
// sectors.  Terms at one position are merged into one coefficient per thread entry at block
// start; during the right-hand-side loop every staged source value is loaded once into
// registers and shared by all the positions and columns that read it, which cuts the shared
// loads per output entry from one per term (14) to under 8 -- shared-memory bandwidth, not
// the FMA count, bounds the per-term design.
// ---------------------------------------------------------------------------------------
template <typename T, bool PLUS>
__global__ void __launch_bounds__(kApplyThreads, sizeof(T) == 4 ? 2 : 1)
    k_apply_canon(const DevSector* __restrict__ sectors, const int4* __restrict__ canon,
                  const typename Vec2<T>::type* __restrict__ coef, const DevTile* __restrict__ tiles, int ntiles,
                  int ncols, int rc, const typename Vec2<T>::type* __restrict__ x,
                  typename Vec2<T>::type* __restrict__ y, long long ld, BorderArgs border) {
  using T2 = typename Vec2<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* win = reinterpret_cast<T2*>(smem_raw);  // [2][3 * kWinElems]
  const int chunk = blockIdx.x / ntiles;
  const int tile_id = blockIdx.x - chunk * ntiles;
  const int c0 = chunk * rc, c1 = min(c0 + rc, ncols);
  const DevTile tile = tiles[tile_id];
  const DevSector& sec = sectors[tile.sector];
  const int n = sec.n;
  const int la = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int lb = warp * kColsPerThread;
  const int a = tile.a0 + la;
  const int b0 = tile.b0 + lb;
  const bool active = a < n && b0 < n;
  const int ac = active ? a : 0, bq = active ? b0 : 0;

  // Merged coefficients of this thread's entries (a, b0 + k).
  const int4* ct = canon + (long long)tile.sector * kCanonEntries;
  T car[4], cai[4], rm[4], rp[4];
  T sd[9][4];
  {
    const int4 t = ct[0];
    const T2 al = __ldg(coef + t.x + ac);
    T2 be[4];
    load4(coef + t.y + bq, be);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      car[k] = al.x + be[k].x;
      cai[k] = al.y + be[k].y;
    }
  }
  const T lm = __ldg(coef + ct[1].x + ac).y;
  const T lp = __ldg(coef + ct[2].x + ac).y;
  {
    T2 be[4];
    load4(coef + ct[3].y + bq, be);
#pragma unroll
    for (int k = 0; k < 4; ++k) rm[k] = be[k].y;
    load4(coef + ct[4].y + bq, be);
#pragma unroll
    for (int k = 0; k < 4; ++k) rp[k] = be[k].y;
  }
#pragma unroll
  for (int pos = 0; pos < 9; ++pos) {
#pragma unroll
    for (int k = 0; k < 4; ++k) sd[pos][k] = 0;
    if (!PLUS && pos % 3 == 2) continue;
#pragma unroll
    for (int t = 0; t < kCanonPerPos; ++t) {
      const int4 e = ct[5 + pos * kCanonPerPos + t];
      const T al = __ldg(coef + e.x + ac).x;
      T2 be[4];
      load4(coef + e.y + bq, be);
#pragma unroll
      for (int k = 0; k < 4; ++k) sd[pos][k] = fma(al, be[k].x, sd[pos][k]);
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) car[k] += sd[4][k];  // own-sector centre sandwich into the ADD term

  // Staging plan, as in k_apply_rhs.
  constexpr int kIters = (kWinCols + kApplyWarps - 1) / kApplyWarps;  // 5
  const bool extra = la < kWinRows - 32;
  unsigned long long vmask = 0;
  long long gbase[3];
  int gstep[3];
  bool have[3];
#pragma unroll
  for (int slot = 0; slot < 3; ++slot) {
    const int s2 = sec.src[slot];
    have[slot] = s2 >= 0;
    const int m = have[slot] ? sectors[s2].n : 0;
    const int R = tile.a0 + slot - 1 - kHalo + la;
    const int C0 = tile.b0 + slot - 1 - kHalo + warp;
    gbase[slot] = (have[slot] ? sectors[s2].offset : 0) + R + (long long)C0 * m;
    gstep[slot] = kApplyWarps * m;
    const bool rv = (unsigned)R < (unsigned)m, rv2 = extra && (unsigned)(R + 32) < (unsigned)m;
#pragma unroll
    for (int it = 0; it < kIters; ++it) {
      const int j = warp + it * kApplyWarps;
      const bool cv = j < kWinCols && (unsigned)(C0 + it * kApplyWarps) < (unsigned)m;
      if (rv && cv) vmask |= 1ull << (slot * 2 * kIters + 2 * it);
      if (rv2 && cv) vmask |= 1ull << (slot * 2 * kIters + 2 * it + 1);
    }
  }
  auto stage = [&](int col, T2* w) {
    const T2* xc = x + (long long)col * ld;
#pragma unroll
    for (int slot = 0; slot < 3; ++slot) {
      if (!have[slot]) continue;
      const T2* g = xc + gbase[slot];
      T2* ws = w + slot * kWinElems + la + warp * kWinRows;
#pragma unroll
      for (int it = 0; it < kIters; ++it) {
        if (warp + it * kApplyWarps < kWinCols) {
          const bool v1 = (vmask >> (slot * 2 * kIters + 2 * it)) & 1ull;
          const bool v2 = (vmask >> (slot * 2 * kIters + 2 * it + 1)) & 1ull;
          cp_async_zfill<sizeof(T2)>(ws, v1 ? g : xc, v1);
          if (extra) cp_async_zfill<sizeof(T2)>(ws + 32, v2 ? g + 32 : xc, v2);
        }
        g += gstep[slot];
        ws += kApplyWarps * kWinRows;
      }
    }
    cp_async_commit();
  };

  const bool do_scale = border.scale != 1.0;
  const T scale = (T)border.scale;
  const bool has_border = border.alpha != nullptr;
  const bool diag_tile = tile.a0 == tile.b0;
  stage(c0, win);
  for (int col = c0; col < c1; ++col) {
    const int buf = (col - c0) & 1;
    if (col + 1 < c1)
      stage(col + 1, win + (buf ^ 1) * 3 * kWinElems);
    else
      cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    if (active) {
      // window coordinates: the thread's entry (a, b0 + k) sits at row la + kHalo, column
      // lb + kHalo + k; X(slot, p, q) reads row shift p and column shift q from there
      const T2* wb = win + buf * 3 * kWinElems + (la + kHalo) + (lb + kHalo) * kWinRows;
      auto X = [&](int slot, int p, int q) -> T2 { return wb[slot * kWinElems + p + q * kWinRows]; };
      T ar[4], ai[4];
      {
        // own sector, row shift 0: columns -1 .. 4 (centre, RIGHT -1/+1)
        T2 r0[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) r0[c] = X(1, 0, c - 1);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const T2 xc = r0[k + 1], xl = r0[k], xr = r0[k + 2];
          ar[k] = car[k] * xc.x - cai[k] * xc.y;
          ai[k] = car[k] * xc.y + cai[k] * xc.x;
          ar[k] = fma(-rm[k], xl.y, ar[k]);
          ai[k] = fma(rm[k], xl.x, ai[k]);
          ar[k] = fma(-rp[k], xr.y, ar[k]);
          ai[k] = fma(rp[k], xr.x, ai[k]);
        }
      }
      {
        // own sector, row shift -1: columns -1 .. 3 (LEFT -1, sandwich (-1,-1))
        T2 r1[5];
#pragma unroll
        for (int c = 0; c < 5; ++c) r1[c] = X(1, -1, c - 1);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const T2 xv = r1[k + 1], xd = r1[k];
          ar[k] = fma(-lm, xv.y, ar[k]);
          ai[k] = fma(lm, xv.x, ai[k]);
          ar[k] = fma(sd[3][k], xd.x, ar[k]);
          ai[k] = fma(sd[3][k], xd.y, ai[k]);
        }
      }
      {
        // own sector, row shift +1: columns 0 .. 4 (LEFT +1, sandwich (1,1))
        T2 r2[5];
#pragma unroll
        for (int c = 0; c < (PLUS ? 5 : 4); ++c) r2[c] = X(1, 1, c);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const T2 xv = r2[k];
          ar[k] = fma(-lp, xv.y, ar[k]);
          ai[k] = fma(lp, xv.x, ai[k]);
          if (PLUS) {
            const T2 xd = r2[k + 1];
            ar[k] = fma(sd[5][k], xd.x, ar[k]);
            ai[k] = fma(sd[5][k], xd.y, ai[k]);
          }
        }
      }
#pragma unroll
      for (int slot = 0; slot < 3; slot += 2) {
        if (!have[slot]) continue;  // not staged; its coefficients are zero
#pragma unroll
        for (int d = -1; d <= (PLUS ? 1 : 0); ++d) {
          const int pos = slot * 3 + d + 1;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const T2 xd = X(slot, d, k + d);
            ar[k] = fma(sd[pos][k], xd.x, ar[k]);
            ai[k] = fma(sd[pos][k], xd.y, ai[k]);
          }
        }
      }
      if (do_scale) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          ar[k] *= scale;
          ai[k] *= scale;
        }
      }
      T2* yp = y + (long long)col * ld + sec.offset + a + (long long)b0 * n;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (b0 + k >= n) break;
        T2 out;
        out.x = ar[k];
        out.y = ai[k];
        if (has_border && diag_tile && b0 + k == a) {
          const double2 al = border.alpha[col];
          const double v = border.coords ? sec.border_z : sec.border_x;
          out.x += (T)(al.x * v);
          out.y += (T)(al.y * v);
        }
        yp[(long long)k * n] = out;
      }
    }
    __syncthreads();  // stage `buf` is refilled two columns later
  }
}

template <typename T, bool PLUS>
cudaError_t launch_apply_canon(const DevicePlan& dp, const void* coef, const void* x, void* y, int ncols,
                               long long ld, const BorderArgs& border, cudaStream_t stream) {
  using T2 = typename Vec2<T>::type;
  const size_t smem = 2 * 3 * kWinElems * sizeof(T2);
  static bool configured = false;
  if (!configured) {
    cudaError_t e =
        cudaFuncSetAttribute(k_apply_canon<T, PLUS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const int rc = ncols >= 64 ? 16 : (ncols >= 16 ? 8 : (ncols >= 4 ? 4 : 1));
  const long long chunks = (ncols + rc - 1) / rc;
  const long long grid = chunks * dp.ntiles;
  k_apply_canon<T, PLUS><<<(unsigned)grid, kApplyThreads, smem, stream>>>(
      dp.sectors, dp.canon, (const T2*)coef, dp.tiles, dp.ntiles, ncols, rc, (const T2*)x, (T2*)y, ld, border);
  return cudaGetLastError();
}

template <typename T, int LI, int RI, int SR>
cudaError_t launch_apply_rhs(const DevicePlan& dp, const void* coef, const void* x, void* y, int ncols,
                             long long ld, const BorderArgs& border, cudaStream_t stream) {
  using T2 = typename Vec2<T>::type;
  const size_t smem = 2 * 3 * kWinElems * sizeof(T2);
  static bool configured = false;
  if (!configured) {
    cudaError_t e =
        cudaFuncSetAttribute(k_apply_rhs<T, LI, RI, SR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  // chunks of right-hand sides per block: enough blocks to fill the GPU, many columns per
  // block to amortize the coefficient setup
  const int rc = ncols >= 64 ? 16 : (ncols >= 16 ? 8 : (ncols >= 4 ? 4 : 1));
  const long long chunks = (ncols + rc - 1) / rc;
  const long long grid = chunks * dp.ntiles;
  k_apply_rhs<T, LI, RI, SR><<<(unsigned)grid, kApplyThreads, smem, stream>>>(
      dp.sectors, (const int4*)dp.fterms, (const T2*)coef, dp.tiles, dp.ntiles, ncols, rc, (const T2*)x, (T2*)y,
      ld, border);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_apply_fast(const DevicePlan& dp, const void* coef, const void* x, void* y, int ncols,
                              long long ld, const BorderArgs& border, cudaStream_t stream) {
  if (dp.canon)
    return dp.canon_plus ? launch_apply_canon<T, true>(dp, coef, x, y, ncols, ld, border, stream)
                         : launch_apply_canon<T, false>(dp, coef, x, y, ncols, ld, border, stream);
  switch (dp.fast_sr) {
    case 5: return launch_apply_rhs<T, 2, 2, 5>(dp, coef, x, y, ncols, ld, border, stream);
    case 9: return launch_apply_rhs<T, 2, 2, 9>(dp, coef, x, y, ncols, ld, border, stream);
    default: return launch_apply_rhs<T, 2, 2, 13>(dp, coef, x, y, ncols, ld, border, stream);
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
  const void* coef = border.coords ? dp.coef64z : dp.coef64;
  if (dp.fast_sr > 0 && ncols >= kFastMinCols)
    return launch_apply_fast<double>(dp, coef, x, y, ncols, ld, border, stream);
  return launch_apply_t<double>(dp, coef, x, y, ncols, ld, border, stream);
}

cudaError_t launch_apply_f32(const DevicePlan& dp, const float* x, float* y, int ncols, long long ld,
                             const BorderArgs& border, cudaStream_t stream) {
  const void* coef = border.coords ? dp.coef32z : dp.coef32x;
  if (dp.fast_sr > 0 && ncols >= kFastMinCols) return launch_apply_fast<float>(dp, coef, x, y, ncols, ld, border, stream);
  return launch_apply_t<float>(dp, coef, x, y, ncols, ld, border, stream);
}

}  // namespace picuda
