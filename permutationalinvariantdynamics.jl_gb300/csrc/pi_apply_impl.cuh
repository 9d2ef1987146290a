// Device building blocks of the fused apply, shared by the single-plan kernels
// (pi_apply.cu) and the multi-instance kernels (pi_batch.cu).
#pragma once

#include "pi_device.cuh"

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

// Output sink of the tile loop that stores (L x)[e] into y[e].
template <typename T2>
struct StoreSink {
  T2* __restrict__ y;
  __device__ __forceinline__ void operator()(long long e, T2 v) const { y[e] = v; }
};

// Stages the zero-padded windows x_src[a0+e-2 .. a0+e+33, b0+e-2 .. b0+e+33] of every source
// sector (e = -1, 0, +1) of `tile` into win (slot e + 1): lane = window row (plus rows 32..35
// on lanes 0..3), warps stride over the 36 window columns.  Every element is one
// asynchronous copy with hardware zero fill (cp.async), so all of a thread's ~30 copies are
// in flight at once and the block waits for memory once, not once per window column.
template <typename T>
__device__ __forceinline__ void stage_windows(const DevSector* __restrict__ sectors, const DevSector& sec,
                                              const DevTile tile, const typename Vec2<T>::type* __restrict__ x,
                                              typename Vec2<T>::type* win) {
  using T2 = typename Vec2<T>::type;
  const int la = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const bool extra = la < kWinRows - 32;
#pragma unroll 1
  for (int slot = 0; slot < 3; ++slot) {
    const int s2 = sec.src[slot];
    if (s2 < 0) continue;
    const int m = sectors[s2].n;
    const T2* xs = x + sectors[s2].offset;
    const int r0 = tile.a0 + slot - 1 - kHalo, c0 = tile.b0 + slot - 1 - kHalo;
    T2* w = win + slot * kWinElems;
    const int R = r0 + la, R2 = r0 + 32 + la;
    const bool rv = (unsigned)R < (unsigned)m, rv2 = extra && (unsigned)R2 < (unsigned)m;
#pragma unroll
    for (int j = warp; j < kWinCols; j += kApplyWarps) {
      const int C = c0 + j;
      const bool cv = (unsigned)C < (unsigned)m;
      const bool v1 = rv && cv, v2 = rv2 && cv;
      cp_async_zfill<sizeof(T2)>(w + la + j * kWinRows, v1 ? xs + R + (long long)C * m : x, v1);
      if (extra) cp_async_zfill<sizeof(T2)>(w + 32 + la + j * kWinRows, v2 ? xs + R2 + (long long)C * m : x, v2);
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
}

// One 32 x 32 output tile of scale * (L x) (+ alpha * v on the diagonal) for the sector
// block `tile`: stage the source windows and the sector's grouped terms in shared memory,
// then evaluate every stencil term and hand each output entry, with its element index, to
// `sink` (a plain store, or a fused epilogue such as an RK4 stage update).  `alpha` is the
// device trace value of this column (or nullptr).  Shared by the single-plan and the
// multi-instance kernels.
template <typename T, typename Sink>
__device__ __forceinline__ void apply_tile_to(const DevSector* __restrict__ sectors, const DevTerm* __restrict__ terms,
                                              const typename Vec2<T>::type* __restrict__ coef, const DevTile tile,
                                              const typename Vec2<T>::type* __restrict__ x, const Sink& sink,
                                              const BorderArgs& border, const double2* alpha,
                                              typename Vec2<T>::type* win, int4* st, int* ge) {
  using T2 = typename Vec2<T>::type;
  const DevSector& sec = sectors[tile.sector];
  const int tb = sec.term_begin;
  const int nt = sec.group_end[G_COUNT - 1] - tb;
  for (int i = threadIdx.x; i < nt; i += blockDim.x) st[i] = reinterpret_cast<const int4*>(terms)[tb + i];
  if (threadIdx.x <= G_COUNT) ge[threadIdx.x] = threadIdx.x == 0 ? 0 : sec.group_end[threadIdx.x - 1] - tb;
  stage_windows<T>(sectors, sec, tile, x, win);
  const int la = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int n = sec.n;
  const int lb = warp * kColsPerThread;
  const int a = tile.a0 + la;
  const int b0 = tile.b0 + lb;
  if (a >= n || b0 >= n) return;
  const int ncol = min(kColsPerThread, n - b0);
  Acc<T> acc;
#pragma unroll
  for (int k = 0; k < kColsPerThread; ++k) acc.re[k] = acc.im[k] = 0;
  const T2* ca = coef + a;
  const T2* cb = coef + b0;
  const T2* wbase = win + (la + kHalo) + (lb + kHalo) * kWinRows;  // + woff selects slot, p, q
  group<T, T2, K_ADD, C_CX>(st, ge[G_ADD], ge[G_ADD + 1], ca, cb, wbase, acc);
  group<T, T2, K_LEFT, C_IM>(st, ge[G_LEFT_IM], ge[G_LEFT_IM + 1], ca, cb, wbase, acc);
  group<T, T2, K_LEFT, C_RE>(st, ge[G_LEFT_RE], ge[G_LEFT_RE + 1], ca, cb, wbase, acc);
  group<T, T2, K_LEFT, C_CX>(st, ge[G_LEFT_CX], ge[G_LEFT_CX + 1], ca, cb, wbase, acc);
  group<T, T2, K_RIGHT, C_IM>(st, ge[G_RIGHT_IM], ge[G_RIGHT_IM + 1], ca, cb, wbase, acc);
  group<T, T2, K_RIGHT, C_RE>(st, ge[G_RIGHT_RE], ge[G_RIGHT_RE + 1], ca, cb, wbase, acc);
  group<T, T2, K_RIGHT, C_CX>(st, ge[G_RIGHT_CX], ge[G_RIGHT_CX + 1], ca, cb, wbase, acc);
  group<T, T2, K_SAND, C_RE>(st, ge[G_SAND_RE], ge[G_SAND_RE + 1], ca, cb, wbase, acc);
  group<T, T2, K_SAND, C_CX>(st, ge[G_SAND_CX], ge[G_SAND_CX + 1], ca, cb, wbase, acc);
  if (border.scale != 1.0) {
    const T scale = (T)border.scale;
#pragma unroll
    for (int k = 0; k < kColsPerThread; ++k) {
      acc.re[k] *= scale;
      acc.im[k] *= scale;
    }
  }
  const long long e0 = sec.offset + a + (long long)b0 * n;
#pragma unroll
  for (int k = 0; k < kColsPerThread; ++k) {
    if (k >= ncol) break;
    T2 out;
    out.x = acc.re[k];
    out.y = acc.im[k];
    if (b0 + k == a && alpha != nullptr) {
      const double2 al = *alpha;
      const double v = border.coords ? sec.border_z : sec.border_x;
      out.x += (T)(al.x * v);
      out.y += (T)(al.y * v);
    }
    sink(e0 + (long long)k * n, out);
  }
}


__device__ __forceinline__ void pmac(float2& acc, float cr, float ci, float2 v) {
  acc.x = fmaf(cr, v.x, acc.x);
  acc.x = fmaf(-ci, v.y, acc.x);
  acc.y = fmaf(cr, v.y, acc.y);
  acc.y = fmaf(ci, v.x, acc.y);
}
__device__ __forceinline__ void prmac(float2& acc, float c, float2 v) {
  acc.x = fmaf(c, v.x, acc.x);
  acc.y = fmaf(c, v.y, acc.y);
}

// The 32 x 32 FP32 tile of apply_tile_to for a canonical plan with its merged coefficients
// read from the split planes: per output entry two coalesced 16-byte entry-plane loads (the
// row and column values are shared) and ten staged source reads, instead of forming every
// stencil term's coefficient product.  A merged position reads the staged window of slot
// e + 1 at offset p + 36 q (x_src[a + e + p, b + e + q]); the window of a missing neighbour
// sector is not staged (stale shared memory), so its positions are skipped, not multiplied
// by their zero coefficients.
template <bool PLUS, typename Sink>
__device__ __forceinline__ void apply_tile_planes_to(const DevSector* __restrict__ sectors, const DevTile tile,
                                                     const float2* __restrict__ x, const Sink& sink,
                                                     const BorderArgs& border, const double2* alpha,
                                                     const SplitPlanes& pl, float2* win) {
  constexpr int NE = PLUS ? 3 : 2;
  const DevSector& sec = sectors[tile.sector];
  stage_windows<float>(sectors, sec, tile, x, win);
  const int la = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int n = sec.n;
  const int lb = warp * kColsPerThread;
  const int a = tile.a0 + la;
  const int b0 = tile.b0 + lb;
  if (a >= n || b0 >= n) return;
  const int ncol = min(kColsPerThread, n - b0);
  const int loff = __ldg(pl.line_off + tile.sector);
  const float4 lv = __ldg(pl.lrow + loff + a);  // LEFT -1, +1 of row a
  const float2* wb = win + (la + kHalo) + (lb + kHalo) * kWinRows;
  const long long e0 = sec.offset + a + (long long)b0 * n;
  const float scale = (float)border.scale;
  const bool has_sm = sec.src[0] >= 0, has_lg = sec.src[2] >= 0;  // block-uniform
#pragma unroll
  for (int k = 0; k < kColsPerThread; ++k) {
    if (k >= ncol) break;
    const float4* ep = pl.eplane + (e0 + (long long)k * n) * NE;
    const float4 c0 = __ldg(ep), c1 = __ldg(ep + 1);
    const float4 rc = __ldg(pl.rcol + loff + b0 + k);  // RIGHT -1, +1 of column b
    const float2* w = wb + k * kWinRows;
    const float2* own = w + kWinElems;
    float2 acc = make_float2(0.f, 0.f);
    pmac(acc, c0.x, c0.y, own[0]);                      // centre
    pmac(acc, lv.x, lv.y, own[-1]);                     // LEFT -1
    pmac(acc, lv.z, lv.w, own[1]);                      // LEFT +1
    pmac(acc, rc.x, rc.y, own[-kWinRows]);              // RIGHT -1
    pmac(acc, rc.z, rc.w, own[kWinRows]);               // RIGHT +1
    prmac(acc, c0.z, own[-1 - kWinRows]);               // own (-1,-1)
    if (has_sm) {
      prmac(acc, c0.w, w[-1 - kWinRows]);               // smaller (-2,-2)
      prmac(acc, c1.x, w[0]);                           // smaller (-1,-1)
    }
    if (has_lg) {
      prmac(acc, c1.y, w[2 * kWinElems - 1 - kWinRows]);  // larger (0,0)
      prmac(acc, c1.z, w[2 * kWinElems]);                 // larger (1,1)
    }
    if (PLUS) {
      const float4 c2 = __ldg(ep + 2);
      prmac(acc, c1.w, own[1 + kWinRows]);                  // own (1,1)
      if (has_sm) prmac(acc, c2.x, w[1 + kWinRows]);        // smaller (0,0)
      if (has_lg) prmac(acc, c2.y, w[2 * kWinElems + 1 + kWinRows]);  // larger (2,2)
    }
    if (border.scale != 1.0) {
      acc.x *= scale;
      acc.y *= scale;
    }
    if (b0 + k == a && alpha != nullptr) {
      const double2 al = *alpha;
      const double v = border.coords ? sec.border_z : sec.border_x;
      acc.x += (float)(al.x * v);
      acc.y += (float)(al.y * v);
    }
    sink(e0 + (long long)k * n, acc);
  }
}

// The output entries (a, b0 .. b0 + ncol - 1) of one thread from the separable line planes:
// r holds row a's factors, colp the tile's column factors, wb points at the thread's entry
// (a, b0) in the own-sector-relative window frame of staged windows with WR rows and WE
// elements per slot.  Every merged coefficient is formed with a few FMAs in the order the
// entry plane was built, so the result is bitwise apply_tile_planes_to's.
template <bool PLUS, int WR, int WE, typename Sink>
__device__ __forceinline__ void sep_entries(const float* r, const float4* colp, const float2* wb, int lb, int ncol,
                                            int a, int b0, const DevSector& sec, const BorderArgs& border,
                                            const double2* alpha, const Sink& sink) {
  constexpr int NF4 = PLUS ? kSepF4Plus : kSepF4;
  const int n = sec.n;
  const long long e0 = sec.offset + a + (long long)b0 * n;
  const float scale = (float)border.scale;
  const bool has_sm = sec.src[0] >= 0, has_lg = sec.src[2] >= 0;  // block-uniform
#pragma unroll
  for (int k = 0; k < kColsPerThread; ++k) {
    if (k >= ncol) break;
    // the same column for the whole warp: broadcast shared reads at their point of use
    const float* c = reinterpret_cast<const float*>(colp + (lb + k) * NF4);
    // sandwich position p: alpha_0 beta_0 + alpha_1 beta_1 + alpha_2 beta_2
    auto sand = [&](int p) {
      const int o = 6 + 3 * p;
      return fmaf(r[o + 2], c[o + 2], fmaf(r[o + 1], c[o + 1], r[o] * c[o]));
    };
    const float cre = fmaf(r[8], c[8], fmaf(r[7], c[7], fmaf(r[6], c[6], r[0] + c[0])));
    const float cim = r[1] + c[1];
    const float2* w = wb + k * WR;
    const float2* own = w + WE;
    float2 acc = make_float2(0.f, 0.f);
    pmac(acc, cre, cim, own[0]);                          // centre
    pmac(acc, r[2], r[3], own[-1]);                       // LEFT -1
    pmac(acc, r[4], r[5], own[1]);                        // LEFT +1
    pmac(acc, c[2], c[3], own[-WR]);                      // RIGHT -1
    pmac(acc, c[4], c[5], own[WR]);                       // RIGHT +1
    prmac(acc, sand(1), own[-1 - WR]);                    // own (-1,-1)
    if (has_sm) {
      prmac(acc, sand(2), w[-1 - WR]);                    // smaller (-2,-2)
      prmac(acc, sand(3), w[0]);                          // smaller (-1,-1)
    }
    if (has_lg) {
      prmac(acc, sand(4), w[2 * WE - 1 - WR]);            // larger (0,0)
      prmac(acc, sand(5), w[2 * WE]);                     // larger (1,1)
    }
    if (PLUS) {
      prmac(acc, sand(6), own[1 + WR]);                          // own (1,1)
      if (has_sm) prmac(acc, sand(7), w[1 + WR]);                // smaller (0,0)
      if (has_lg) prmac(acc, sand(8), w[2 * WE + 1 + WR]);       // larger (2,2)
    }
    if (border.scale != 1.0) {
      acc.x *= scale;
      acc.y *= scale;
    }
    if (b0 + k == a && alpha != nullptr) {
      const double2 al = *alpha;
      const double v = border.coords ? sec.border_z : sec.border_x;
      acc.x += (float)(al.x * v);
      acc.y += (float)(al.y * v);
    }
    sink(e0 + (long long)k * n, acc);
  }
}

// The same tile from the separable line planes: each thread loads its row's factors once and
// each column's factors as broadcast loads, so y is bitwise the same as apply_tile_planes_to's
// while only 16 bytes per entry (x in, y out) come from memory.
template <bool PLUS, typename Sink>
__device__ __forceinline__ void apply_tile_sep_to(const DevSector* __restrict__ sectors, const DevTile tile,
                                                  const float2* __restrict__ x, const Sink& sink,
                                                  const BorderArgs& border, const double2* alpha,
                                                  const SplitPlanes& pl, float2* win) {
  constexpr int NF4 = PLUS ? kSepF4Plus : kSepF4;
  __shared__ __align__(16) float4 colp[kTileCols * NF4];  // the tile's column planes
  const DevSector& sec = sectors[tile.sector];
  const int la = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int n = sec.n;
  const int loff = __ldg(pl.line_off + tile.sector);
  // column planes of the tile's 32 columns land with the source windows (one cp.async wait)
  for (int i = threadIdx.x; i < kTileCols * NF4; i += blockDim.x) {
    const int b = tile.b0 + i / NF4;
    const bool ok = b < n;
    cp_async_zfill<16>(colp + i, ok ? pl.scol + (long long)(loff + b) * NF4 + i % NF4 : pl.scol, ok);
  }
  // this thread's row factors, in flight during the staging
  const int a = tile.a0 + la;
  const int ar = a < n ? a : 0;
  float4 rv[NF4];
#pragma unroll
  for (int k = 0; k < NF4; ++k) rv[k] = __ldg(pl.srow + (long long)(loff + ar) * NF4 + k);
  stage_windows<float>(sectors, sec, tile, x, win);
  const int lb = warp * kColsPerThread;
  const int b0 = tile.b0 + lb;
  if (a >= n || b0 >= n) return;
  float r[4 * NF4];
#pragma unroll
  for (int k = 0; k < NF4; ++k) {
    r[4 * k] = rv[k].x;
    r[4 * k + 1] = rv[k].y;
    r[4 * k + 2] = rv[k].z;
    r[4 * k + 3] = rv[k].w;
  }
  const float2* wb = win + (la + kHalo) + (lb + kHalo) * kWinRows;
  sep_entries<PLUS, kWinRows, kWinElems>(r, colp, wb, lb, min(kColsPerThread, n - b0), a, b0, sec, border, alpha,
                                         sink);
}

// ---------------------------------------------------------------------------------------
// Two-stage separable-plane tiles for persistent launches.  The canonical positions read
// only the shifts -1..+1 around (a + e, b + e), so each source window needs a halo of one
// (34 x 34) instead of the general stencil's two (36 x 36).  One stage holds the three
// windows and the tile's 32 row and 32 column factor lines; a block computes the tile of one
// stage while the next tile's stage is in flight.
// ---------------------------------------------------------------------------------------
constexpr int kSepRows = kTileRows + 2;
constexpr int kSepCols = kTileCols + 2;
constexpr int kSepElems = kSepRows * kSepCols;
constexpr int kSepLineBytes = kTileRows * kSepF4Plus * 16;                    // row or column factors
constexpr int kSepStageBytes = 3 * kSepElems * (int)sizeof(float2) + 2 * kSepLineBytes;
constexpr int kSepSmemBytes = 2 * kSepStageBytes;
static_assert(kSepStageBytes % 16 == 0, "stages must keep 16-byte cp.async destinations aligned");
static_assert(kTileRows == kTileCols, "row and column factor lines share one stage layout");

struct SepStage {
  float2* win;   // [3][kSepElems]: slot e + 1 starts at (a0 + e - 1, b0 + e - 1)
  float4* colp;  // [kTileCols][NF4]
  float4* rowp;  // [kTileRows][NF4]
};

__device__ __forceinline__ SepStage sep_stage(unsigned char* smem, int stage) {
  unsigned char* p = smem + stage * kSepStageBytes;
  constexpr int kWinBytes = 3 * kSepElems * (int)sizeof(float2);
  return SepStage{reinterpret_cast<float2*>(p), reinterpret_cast<float4*>(p + kWinBytes),
                  reinterpret_cast<float4*>(p + kWinBytes + kSepLineBytes)};
}

// Issues (and commits as one cp.async group) the stage of `tile`: the zero-padded windows
// x_src[a0 + e - 2 .. a0 + e + 31, b0 + e - 2 .. b0 + e + 31] of the source sectors that exist
// (lane = window row, plus rows 32..33 on lanes 0..1; warps stride over the 34 columns) and
// the factor lines of the tile's rows and columns (zeros past the block edge).
template <int NF4>
__device__ __forceinline__ void sep_issue(const DevSector* __restrict__ sectors, const DevTile tile,
                                          const float2* __restrict__ x, const SplitPlanes& pl, SepStage sg) {
  const DevSector& sec = sectors[tile.sector];
  const int n = sec.n;
  const int loff = __ldg(pl.line_off + tile.sector);
  for (int i = threadIdx.x; i < 2 * kTileCols * NF4; i += blockDim.x) {
    const bool col = i < kTileCols * NF4;
    const int ii = col ? i : i - kTileCols * NF4;
    const int q = (col ? tile.b0 : tile.a0) + ii / NF4;
    const float4* src = col ? pl.scol : pl.srow;
    const bool ok = q < n;
    cp_async_zfill<16>((col ? sg.colp : sg.rowp) + ii, ok ? src + (long long)(loff + q) * NF4 + ii % NF4 : src, ok);
  }
  const int la = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const bool extra = la < kSepRows - 32;
#pragma unroll 1
  for (int slot = 0; slot < 3; ++slot) {
    const int s2 = sec.src[slot];
    if (s2 < 0) continue;
    const int m = sectors[s2].n;
    const float2* xs = x + sectors[s2].offset;
    const int r0 = tile.a0 + slot - 2, c0 = tile.b0 + slot - 2;
    float2* w = sg.win + slot * kSepElems;
    const int R = r0 + la, R2 = r0 + 32 + la;
    const bool rv = (unsigned)R < (unsigned)m, rv2 = extra && (unsigned)R2 < (unsigned)m;
#pragma unroll
    for (int j = warp; j < kSepCols; j += kApplyWarps) {
      const int C = c0 + j;
      const bool cv = (unsigned)C < (unsigned)m;
      const bool v1 = rv && cv, v2 = rv2 && cv;
      cp_async_zfill<sizeof(float2)>(w + la + j * kSepRows, v1 ? xs + R + (long long)C * m : x, v1);
      if (extra) cp_async_zfill<sizeof(float2)>(w + 32 + la + j * kSepRows, v2 ? xs + R2 + (long long)C * m : x, v2);
    }
  }
  cp_async_commit();
}

// The tile of a landed stage (the caller has waited for its group and synchronised).
template <bool PLUS, typename Sink>
__device__ __forceinline__ void sep_compute(const DevSector* __restrict__ sectors, const DevTile tile, const Sink& sink,
                                            const BorderArgs& border, const double2* alpha, SepStage sg) {
  constexpr int NF4 = PLUS ? kSepF4Plus : kSepF4;
  const DevSector& sec = sectors[tile.sector];
  const int la = threadIdx.x & 31;
  const int lb = (threadIdx.x >> 5) * kColsPerThread;
  const int n = sec.n;
  const int a = tile.a0 + la;
  const int b0 = tile.b0 + lb;
  if (a >= n || b0 >= n) return;
  float r[4 * NF4];
  const float4* rp = sg.rowp + la * NF4;
#pragma unroll
  for (int k = 0; k < NF4; ++k) {
    const float4 v = rp[k];
    r[4 * k] = v.x;
    r[4 * k + 1] = v.y;
    r[4 * k + 2] = v.z;
    r[4 * k + 3] = v.w;
  }
  const float2* wb = sg.win + (la + 1) + (lb + 1) * kSepRows;
  sep_entries<PLUS, kSepRows, kSepElems>(r, sg.colp, wb, lb, min(kColsPerThread, n - b0), a, b0, sec, border, alpha,
                                         sink);
}

template <typename T>
__device__ __forceinline__ void apply_tile(const DevSector* __restrict__ sectors, const DevTerm* __restrict__ terms,
                                           const typename Vec2<T>::type* __restrict__ coef, const DevTile tile,
                                           const typename Vec2<T>::type* __restrict__ x,
                                           typename Vec2<T>::type* __restrict__ y, const BorderArgs& border,
                                           const double2* alpha, typename Vec2<T>::type* win, int4* st, int* ge) {
  apply_tile_to<T>(sectors, terms, coef, tile, x, StoreSink<typename Vec2<T>::type>{y}, border, alpha, win, st, ge);
}

}  // namespace picuda
