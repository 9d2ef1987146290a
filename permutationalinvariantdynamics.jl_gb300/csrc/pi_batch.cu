// Multi-instance Krylov engine (see pi_batch.hpp): device kernels over the engine's
// (instance, tile) and (instance, chunk) work lists, the engine's stage execution, the
// dynamics and steady-state job controllers, and the batched C entry points.
#include "pi_batch.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <random>
#include <tuple>
#include <unordered_set>
#include <utility>

#include "pi_apply_impl.cuh"
#include "pi_dense.hpp"

namespace picuda {
namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 conjd(double2 a) { return make_double2(a.x, -a.y); }

__device__ __forceinline__ double2 ld2(const double2* p) { return *p; }
__device__ __forceinline__ double2 ld2(const float2* p) {
  const float2 v = *p;
  return make_double2((double)v.x, (double)v.y);
}
__device__ __forceinline__ void st2(double2* p, double x, double y) { *p = make_double2(x, y); }
__device__ __forceinline__ void st2(float2* p, double x, double y) { *p = make_float2((float)x, (float)y); }

// Deterministic block sum of NV values (blockDim.x a multiple of 32); result in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[warp * NV + k] = v[k];
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = lane < nw ? smem[lane * NV + k] : 0.0;
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  }
}

// Double-float accumulator (FP32 pair): exact products by FMA, TwoSum accumulation.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ void df_add_prod(DF& acc, float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  const float s = acc.hi + p;
  const float bb = s - acc.hi;
  const float err = (acc.hi - (s - bb)) + (p - bb);
  acc.hi = s;
  acc.lo += err + e;
}

__device__ __forceinline__ void chunk_range(const DevInst& S, int c, long long& beg, long long& end) {
  beg = (long long)(c - S.chunk_begin) * S.chunk;
  end = min(beg + (long long)S.chunk, S.dim);
}

constexpr int kRT = kReduceThreads;  // threads of the chunk kernels

// ---------------------------------------------------------------------------------------
// Stage-1 kernels
// ---------------------------------------------------------------------------------------

// cout (+)= sum_k ccoef[k] V_k, FP64 accumulation.
template <typename T2>
__global__ void __launch_bounds__(kRT) k_s1_combine(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst) {
  __shared__ double2 cs[kBatchMaxKrylov + 2];
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  double2* out = S.cout;
  if (!out) return;
  const int nc = S.ccount;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) cs[i] = S.ccoef[i];
  __syncthreads();
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  const T2* V = (const T2*)S.V;
  const long long dim = S.ldv;
  const int acc = S.cacc;
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    double yx = 0, yy = 0;
    for (int k = 0; k < nc; ++k) {
      const double2 v = ld2(V + (long long)k * dim + e);
      yx = fma(v.x, cs[k].x, yx);
      yx = fma(-v.y, cs[k].y, yx);
      yy = fma(v.x, cs[k].y, yy);
      yy = fma(v.y, cs[k].x, yy);
    }
    if (acc) {
      const double2 o = out[e];
      yx += o.x;
      yy += o.y;
    }
    out[e] = make_double2(yx, yy);
  }
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

// Complex normal probe (unit variance): Box-Muller on a counter-based 64-bit hash
// (SplitMix64 finaliser) of (seed, element).
__global__ void __launch_bounds__(kRT) k_s1_probe(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst) {
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  double2* p = S.probe;
  if (!p) return;
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  const unsigned long long seed = mix64(S.seed);
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const unsigned long long h = mix64(seed ^ (unsigned long long)e);
    const double u1 = ((double)(h >> 32) + 1.0) * 2.3283064365386963e-10;  // (0, 1]
    const double u2 = (double)(h & 0xffffffffULL) * 2.3283064365386963e-10;  // [0, 1)
    const double r = sqrt(-2.0 * log(u1)) * 0.70710678118654752;
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    p[e] = make_double2(r * cs, r * sn);
  }
}

// aux_alpha = t^H ax for bordered stage-1 applies, and out[2..3] = t^H tr.
__global__ void __launch_bounds__(kRT) k_s1_trace(DevInst* __restrict__ st) {
  __shared__ double smem[32 * 4];
  DevInst& S = st[blockIdx.x];
  const double2* ax = (S.ax && S.aux_border) ? S.ax : nullptr;
  const double2* tr = S.tr;
  if (!ax && !tr) return;
  double acc[4] = {0, 0, 0, 0};
  for (int i = threadIdx.x; i < S.ndiag; i += blockDim.x) {
    const double w = S.sectors[S.diag_sector[i]].sqrt_f;
    const long long e = S.diag_index[i];
    if (ax) {
      acc[0] = fma(w, ax[e].x, acc[0]);
      acc[1] = fma(w, ax[e].y, acc[1]);
    }
    if (tr) {
      acc[2] = fma(w, tr[e].x, acc[2]);
      acc[3] = fma(w, tr[e].y, acc[3]);
    }
  }
  block_sum<4>(acc, smem);
  if (threadIdx.x == 0) {
    if (ax) S.aux_alpha = make_double2(acc[0], acc[1]);
    if (tr) {
      S.out[2] = acc[2];
      S.out[3] = acc[3];
    }
  }
}

// Applies over the (instance, tile) list.  AUX: ay = aux_scale L ax (+ border), FP64;
// otherwise the Arnoldi step w = scale L V_j (+ border) in the basis precision.
template <typename T, bool AUX>
__global__ void __launch_bounds__(kApplyThreads, sizeof(T) == 4 && !AUX ? 4 : 1)
    k_bapply(const DevInst* __restrict__ st, const int* __restrict__ tile_inst, const int* __restrict__ tile_local) {
  using T2 = typename Vec2<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* win = reinterpret_cast<T2*>(smem_raw);
  __shared__ int4 sterms[kMaxSectorTerms];
  __shared__ int ge[G_COUNT + 1];
  const DevInst& S = st[tile_inst[blockIdx.x]];
  if (AUX) {
    if (!S.ax) return;
    const DevTile tile = S.tiles[tile_local[blockIdx.x]];
    BorderArgs b{S.aux_scale, nullptr, 0};
    apply_tile<T>(S.sectors, S.terms, (const T2*)S.coef64, tile, (const T2*)S.ax, (T2*)S.ay, b,
                  S.aux_border ? &S.aux_alpha : nullptr, win, sterms, ge);
  } else {
    if (S.done) return;
    const DevTile tile = S.tiles[tile_local[blockIdx.x]];
    BorderArgs b{S.scale, nullptr, S.coords};
    const T2* xin = (const T2*)S.V + (long long)S.j * S.ldv;
    if constexpr (sizeof(T) == sizeof(float)) {
      if (S.planes.eplane != nullptr && S.coords == S.pwhich) {  // block-uniform
        const StoreSink<float2> sink{(float2*)S.w};
        if (S.planes.srow != nullptr) {  // separable line planes: x in, y out per entry
          if (S.planes.plus)
            apply_tile_sep_to<true>(S.sectors, tile, xin, sink, b, S.border ? &S.alpha : nullptr, S.planes, win);
          else
            apply_tile_sep_to<false>(S.sectors, tile, xin, sink, b, S.border ? &S.alpha : nullptr, S.planes, win);
        } else if (S.planes.plus) {
          apply_tile_planes_to<true>(S.sectors, tile, xin, sink, b, S.border ? &S.alpha : nullptr, S.planes, win);
        } else {
          apply_tile_planes_to<false>(S.sectors, tile, xin, sink, b, S.border ? &S.alpha : nullptr, S.planes, win);
        }
        return;
      }
    }
    apply_tile<T>(S.sectors, S.terms, (const T2*)S.coefb, tile, xin, (T2*)S.w, b, S.border ? &S.alpha : nullptr, win,
                  sterms, ge);
  }
}

// Persistent FP32 Arnoldi-step apply w = scale L V_j (+ border) over the (instance, tile)
// list: gridDim.x blocks (a multiple of the SM count, picked by the engine's autotuner)
// stride over the list.  Tiles of instances with separable line planes run two-stage: a
// block computes one tile while the stage of its next such tile is in flight; any other
// tile runs the general stencil synchronously.  Per-entry arithmetic is k_bapply<float,
// false>'s, so w is bitwise the same for every grid size and for the one-block-per-tile
// launch.
__global__ void __launch_bounds__(kApplyThreads, 3)
    k_bapply_persist(const DevInst* __restrict__ st, const int* __restrict__ tile_inst,
                     const int* __restrict__ tile_local, int ntotal) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // work kind of list item i, block-uniform: 0 skip (instance stopped this cycle), 1 / 2
  // separable planes without / with the +1 diagonal shifts, 3 general stencil
  auto kind = [&](int i) -> int {
    if (i >= ntotal) return -1;
    const DevInst& S = st[tile_inst[i]];
    if (S.done) return 0;
    if (S.planes.srow != nullptr && S.coords == S.pwhich) return S.planes.plus ? 2 : 1;
    return 3;
  };
  auto issue = [&](int i, int k, int stage) {
    const DevInst& S = st[tile_inst[i]];
    const DevTile tile = S.tiles[tile_local[i]];
    const float2* xin = (const float2*)S.V + (long long)S.j * S.ldv;
    if (k == 2)
      sep_issue<kSepF4Plus>(S.sectors, tile, xin, S.planes, sep_stage(smem_raw, stage));
    else
      sep_issue<kSepF4>(S.sectors, tile, xin, S.planes, sep_stage(smem_raw, stage));
  };
  int i = blockIdx.x;
  int stage = 0;
  bool staged = false;  // item i's stage was issued by the previous iteration
  while (i < ntotal) {
    const int ki = kind(i);
    if (ki == 0) {
      i += gridDim.x;
      continue;
    }
    const DevInst& S = st[tile_inst[i]];
    const DevTile tile = S.tiles[tile_local[i]];
    const BorderArgs b{S.scale, nullptr, S.coords};
    const double2* al = S.border ? &S.alpha : nullptr;
    if (ki == 3) {  // nothing is in flight here: only separable tiles are prefetched
      float2* win = reinterpret_cast<float2*>(smem_raw);
      int4* sterms = reinterpret_cast<int4*>(smem_raw + 3 * kWinElems * sizeof(float2));
      int* ge = reinterpret_cast<int*>(sterms + kMaxSectorTerms);
      apply_tile<float>(S.sectors, S.terms, (const float2*)S.coefb, tile, (const float2*)S.V + (long long)S.j * S.ldv,
                        (float2*)S.w, b, al, win, sterms, ge);
      __syncthreads();  // the windows are restaged by the next item
      i += gridDim.x;
      continue;
    }
    if (!staged) issue(i, ki, stage);
    int j = i + gridDim.x;
    int kj = kind(j);
    while (kj == 0) {
      j += gridDim.x;
      kj = kind(j);
    }
    const bool pre = kj == 1 || kj == 2;
    if (pre) {
      issue(j, kj, stage ^ 1);
      cp_async_wait<1>();  // item i's group has landed, item j's stays in flight
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const StoreSink<float2> sink{(float2*)S.w};
    if (ki == 2)
      sep_compute<true>(S.sectors, tile, sink, b, al, sep_stage(smem_raw, stage));
    else
      sep_compute<false>(S.sectors, tile, sink, b, al, sep_stage(smem_raw, stage));
    __syncthreads();  // this stage is refilled by the prefetch of the item after j
    staged = pre;
    if (pre) stage ^= 1;
    i = kj < 0 ? ntotal : j;
  }
}

__global__ void __launch_bounds__(kRT) k_s1_resid(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst) {
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  double2* r = S.rout;
  if (!r) return;
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const double2 b = S.rb[e], a = S.ay[e];
    r[e] = make_double2(b.x - a.x, b.y - a.y);
  }
}

__global__ void __launch_bounds__(kRT)
    k_s1_norm_partial(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst, double* __restrict__ part) {
  __shared__ double smem[32 * 2];
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  const double2* a = S.nrm0;
  const double2* b = S.nrm1;
  if (!a && !b) return;
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  double acc[2] = {0, 0};
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    if (a) {
      const double2 v = a[e];
      acc[0] = fma(v.x, v.x, acc[0]);
      acc[0] = fma(v.y, v.y, acc[0]);
    }
    if (b) {
      const double2 v = b[e];
      acc[1] = fma(v.x, v.x, acc[1]);
      acc[1] = fma(v.y, v.y, acc[1]);
    }
  }
  block_sum<2>(acc, smem);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = acc[0];
    part[2 * blockIdx.x + 1] = acc[1];
  }
}

__global__ void __launch_bounds__(kRT)
    k_s1_norm_final(const DevInst* __restrict__ st, const int* __restrict__ nchunks, const double* __restrict__ part) {
  __shared__ double smem[32 * 2];
  const DevInst& S = st[blockIdx.x];
  if (!S.nrm0 && !S.nrm1) return;
  double acc[2] = {0, 0};
  for (int c = threadIdx.x; c < nchunks[blockIdx.x]; c += blockDim.x) {
    acc[0] += part[2 * (S.chunk_begin + c)];
    acc[1] += part[2 * (S.chunk_begin + c) + 1];
  }
  block_sum<2>(acc, smem);
  if (threadIdx.x == 0) {
    S.out[0] = acc[0];
    S.out[1] = acc[1];
  }
}

// Observable dots conj(ob_o) . obx over one chunk (FP64 data).  Only the live observables
// are reduced: warp shuffles per observable, then one shared-memory pass.
__global__ void __launch_bounds__(kRT)
    k_s1_obs_partial(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst, double2* __restrict__ partv) {
  __shared__ double2 red[kBatchMaxObs][kRT / 32];
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  const int nob = S.nob;
  if (nob == 0) return;
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o0 = 0; o0 < nob; o0 += 4) {
    double acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = 0;
    for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
      const double2 x = S.obx[e];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (o0 + k < nob) {
          const double2 v = S.ob[(long long)(o0 + k) * S.dim + e];
          acc[2 * k] = fma(v.x, x.x, acc[2 * k]);
          acc[2 * k] = fma(v.y, x.y, acc[2 * k]);
          acc[2 * k + 1] = fma(v.x, x.y, acc[2 * k + 1]);
          acc[2 * k + 1] = fma(-v.y, x.x, acc[2 * k + 1]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (o0 + k < nob) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          acc[2 * k] += __shfl_down_sync(0xffffffffu, acc[2 * k], off);
          acc[2 * k + 1] += __shfl_down_sync(0xffffffffu, acc[2 * k + 1], off);
        }
        if (lane == 0) red[o0 + k][warp] = make_double2(acc[2 * k], acc[2 * k + 1]);
      }
    }
  }
  __syncthreads();
  for (int o = threadIdx.x; o < nob; o += blockDim.x) {
    double sx = 0, sy = 0;
#pragma unroll
    for (int wdx = 0; wdx < kRT / 32; ++wdx) {
      sx += red[o][wdx].x;
      sy += red[o][wdx].y;
    }
    partv[(long long)blockIdx.x * kMaxDots + o] = make_double2(sx, sy);
  }
}

// Per-instance sums of chunk partials: one warp per value, fixed order.
__device__ __forceinline__ double2 warp_chunk_sum(const double2* partv, int begin, int nc, int i) {
  const int lane = threadIdx.x & 31;
  double sx = 0, sy = 0;
  for (int c = lane; c < nc; c += 32) {
    const double2 p = partv[(long long)(begin + c) * kMaxDots + i];
    sx += p.x;
    sy += p.y;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    sx += __shfl_down_sync(0xffffffffu, sx, off);
    sy += __shfl_down_sync(0xffffffffu, sy, off);
  }
  return make_double2(sx, sy);
}

__global__ void __launch_bounds__(kRT)
    k_s1_obs_final(const DevInst* __restrict__ st, const int* __restrict__ nchunks, const double2* __restrict__ partv) {
  const DevInst& S = st[blockIdx.x];
  const int nob = S.nob;
  if (nob == 0) return;
  const int warp = threadIdx.x >> 5;
  for (int o = warp; o < nob; o += blockDim.x >> 5) {
    const double2 v = warp_chunk_sum(partv, S.chunk_begin, nchunks[blockIdx.x], o);
    if ((threadIdx.x & 31) == 0) {
      S.out[4 + 2 * o] = v.x;
      S.out[5 + 2 * o] = v.y;
    }
  }
}

// ---------------------------------------------------------------------------------------
// Arnoldi-step kernels
// ---------------------------------------------------------------------------------------

// V_0 = v0 / v0norm; the instance's first chunk also resets the GMRES right-hand side.
template <typename T2>
__global__ void __launch_bounds__(kRT) k_load_v0(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst) {
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  const double2* x = S.v0;
  if (!x) return;
  const double f = 1.0 / S.v0norm;
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  T2* V = (T2*)S.V;
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const double2 v = x[e];
    st2(V + e, f * v.x, f * v.y);
  }
  if ((int)blockIdx.x == S.chunk_begin)
    for (int r = threadIdx.x; r < S.ldh; r += blockDim.x) S.g[r] = make_double2(r == 0 ? S.v0norm : 0.0, 0.0);
}

// alpha = t^H V_j for bordered cycles.
template <typename T2>
__global__ void __launch_bounds__(kRT) k_step_trace(DevInst* __restrict__ st) {
  __shared__ double smem[32 * 2];
  DevInst& S = st[blockIdx.x];
  if (S.done || !S.border) return;
  const T2* x = (const T2*)S.V + (long long)S.j * S.ldv;
  double acc[2] = {0, 0};
  for (int i = threadIdx.x; i < S.ndiag; i += blockDim.x) {
    const double w = S.coords ? 1.0 : S.sectors[S.diag_sector[i]].sqrt_f;
    const double2 v = ld2(x + S.diag_index[i]);
    acc[0] = fma(w, v.x, acc[0]);
    acc[1] = fma(w, v.y, acc[1]);
  }
  block_sum<2>(acc, smem);
  if (threadIdx.x == 0) S.alpha = make_double2(acc[0], acc[1]);
}

// |w|^2 partials (image norm, skipped by GMRES cycles which do not use it).
template <typename T2>
__global__ void __launch_bounds__(kRT)
    k_step_image_partial(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst, double* __restrict__ part) {
  __shared__ double smem[32];
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  if (S.done || S.givens) return;
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  const T2* w = (const T2*)S.w;
  double acc[1] = {0};
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const double2 v = ld2(w + e);
    acc[0] = fma(v.x, v.x, acc[0]);
    acc[0] = fma(v.y, v.y, acc[0]);
  }
  block_sum<1>(acc, smem);
  if (threadIdx.x == 0) part[blockIdx.x] = acc[0];
}

// CGS2 projections: partv[c][i] = sum over chunk c of conj(V_i) w, i in [8 y, 8 y + 8).
template <typename T2, bool DFACC>
__global__ void __launch_bounds__(kRT)
    k_step_mdot_partial(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst, double2* __restrict__ partv) {
  __shared__ double smem[32 * 16];
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  if (S.done) return;
  const int nv = S.j + 1;
  const int g0 = blockIdx.y * 8;
  if (g0 >= nv) return;
  const int cnt = min(8, nv - g0);
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  const long long dim = S.ldv;
  const T2* V = (const T2*)S.V + (long long)g0 * dim;
  const T2* w = (const T2*)S.w;
  double acc[16];
  if (DFACC) {
    DF re[8], im[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) re[k] = im[k] = DF{0.f, 0.f};
    for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
      const float2 wv = reinterpret_cast<const float2*>(w)[e];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (k < cnt) {
          const float2 v = reinterpret_cast<const float2*>(V)[(long long)k * dim + e];
          df_add_prod(re[k], v.x, wv.x);
          df_add_prod(re[k], v.y, wv.y);
          df_add_prod(im[k], v.x, wv.y);
          df_add_prod(im[k], -v.y, wv.x);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      acc[2 * k] = (double)re[k].hi + (double)re[k].lo;
      acc[2 * k + 1] = (double)im[k].hi + (double)im[k].lo;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k] = 0;
    for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
      const double2 wv = ld2(w + e);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (k < cnt) {
          const double2 v = ld2(V + (long long)k * dim + e);
          acc[2 * k] = fma(v.x, wv.x, acc[2 * k]);
          acc[2 * k] = fma(v.y, wv.y, acc[2 * k]);
          acc[2 * k + 1] = fma(v.x, wv.y, acc[2 * k + 1]);
          acc[2 * k + 1] = fma(-v.y, wv.x, acc[2 * k + 1]);
        }
      }
    }
  }
  block_sum<16>(acc, smem);
  if (threadIdx.x == 0)
    for (int k = 0; k < cnt; ++k)
      partv[(long long)blockIdx.x * kMaxDots + g0 + k] = make_double2(acc[2 * k], acc[2 * k + 1]);
}

// which 0: hA, 1: hB.  Grid (instances, column groups): warp w of block (x, y) reduces
// column i = y * warps + w, so every column of every instance has its own warp (one warp
// walking several columns left a single SM reducing a long chunk list per column).
__global__ void __launch_bounds__(kRT)
    k_step_mdot_final(const DevInst* __restrict__ st, const int* __restrict__ nchunks, const double2* __restrict__ partv,
                      int which) {
  const DevInst& S = st[blockIdx.x];
  if (S.done) return;
  const int nv = S.j + 1;
  double2* h = which == 0 ? S.hA : S.hB;
  const int i = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= nv) return;  // warp-uniform
  const double2 v = warp_chunk_sum(partv, S.chunk_begin, nchunks[blockIdx.x], i);
  if ((threadIdx.x & 31) == 0) h[i] = v;
}

// The first-pass reductions of a step in one launch: blocks (x, y < gridDim.y - 1) reduce the
// projections into hA as k_step_mdot_final(which 0) does, blocks (x, gridDim.y - 1) the
// image norm |w|^2 into image2 (expv cycles): thread t sums the chunk partials t, t + 256,
// ... and a deterministic block sum combines the threads.
__global__ void __launch_bounds__(kRT)
    k_step_first_final(DevInst* __restrict__ st, const int* __restrict__ nchunks, const double2* __restrict__ partv,
                       const double* __restrict__ part, int all_images) {
  __shared__ double smem[32];
  DevInst& S = st[blockIdx.x];
  if (S.done) return;
  if (blockIdx.y == gridDim.y - 1) {  // image norm (block-uniform)
    if (S.givens && !all_images) return;
    double acc[1] = {0};
    for (int c = threadIdx.x; c < nchunks[blockIdx.x]; c += blockDim.x) acc[0] += part[S.chunk_begin + c];
    block_sum<1>(acc, smem);
    if (threadIdx.x == 0) S.image2 = acc[0];
    return;
  }
  const int nv = S.j + 1;
  const int i = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= nv) return;  // warp-uniform
  const double2 v = warp_chunk_sum(partv, S.chunk_begin, nchunks[blockIdx.x], i);
  if ((threadIdx.x & 31) == 0) S.hA[i] = v;
}

// |w|^2 of job S from its chunk partials (thread t sums partials t, t + 256, ..., then a
// deterministic block sum), broadcast to the whole block: every block of the job obtains
// the same value.
__device__ __forceinline__ double job_norm2(const DevInst& S, int nchunks, const double* __restrict__ part) {
  __shared__ double smem[32];
  __shared__ double total;
  double acc[1] = {0};
  for (int c = threadIdx.x; c < nchunks; c += blockDim.x) acc[0] += part[S.chunk_begin + c];
  block_sum<1>(acc, smem);
  if (threadIdx.x == 0) total = acc[0];
  __syncthreads();
  return total;
}

// w -= sum_i V_i h_i (which 0: hA, 1: hB); with part != nullptr also |w|^2 partials.
template <typename T2>
__global__ void __launch_bounds__(kRT)
    k_step_maxpy(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst, int which, double* __restrict__ part) {
  __shared__ double2 hs[kMaxDots];
  __shared__ double smem[32];
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  if (S.done) return;
  const int nv = S.j + 1;
  const double2* h = which == 0 ? S.hA : S.hB;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) hs[i] = h[i];
  __syncthreads();
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  const long long dim = S.ldv;
  const T2* V = (const T2*)S.V;
  T2* w = (T2*)S.w;
  constexpr bool F32 = sizeof(T2) == sizeof(float2);
  double acc[1] = {0};
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    double2 out;
    if (F32) {  // FP32 basis: FP32 update
      float2 wv = reinterpret_cast<const float2*>(w)[e];
      for (int i = 0; i < nv; ++i) {
        const float2 v = reinterpret_cast<const float2*>(V)[(long long)i * dim + e];
        const float cx = (float)hs[i].x, cy = (float)hs[i].y;
        wv.x = fmaf(-v.x, cx, wv.x);
        wv.x = fmaf(v.y, cy, wv.x);
        wv.y = fmaf(-v.x, cy, wv.y);
        wv.y = fmaf(-v.y, cx, wv.y);
      }
      reinterpret_cast<float2*>(w)[e] = wv;
      out = make_double2(wv.x, wv.y);
    } else {
      double2 wv = ld2(w + e);
      for (int i = 0; i < nv; ++i) {
        const double2 v = ld2(V + (long long)i * dim + e);
        wv.x = fma(-v.x, hs[i].x, wv.x);
        wv.x = fma(v.y, hs[i].y, wv.x);
        wv.y = fma(-v.x, hs[i].y, wv.y);
        wv.y = fma(-v.y, hs[i].x, wv.y);
      }
      st2(w + e, wv.x, wv.y);
      out = wv;
    }
    acc[0] = fma(out.x, out.x, acc[0]);
    acc[0] = fma(out.y, out.y, acc[0]);
  }
  if (part) {
    block_sum<1>(acc, smem);
    if (threadIdx.x == 0) part[blockIdx.x] = acc[0];
  }
}

// V_{j+1} = w / |w| (zero on an exact breakdown).  Every block reduces the job's |w|^2
// partials itself (the job's first block stores rem2 for the step finish), so no separate
// reduction launch sits between the second-pass update and the normalisation.
template <typename T2>
__global__ void __launch_bounds__(kRT) k_step_normalize(DevInst* __restrict__ st, const int* __restrict__ chunk_inst,
                                                        const int* __restrict__ nchunks, const double* __restrict__ part) {
  const int inst = chunk_inst[blockIdx.x];
  DevInst& S = st[inst];
  if (S.done) return;
  const double rem2 = job_norm2(S, nchunks[inst], part);
  if (blockIdx.x == S.chunk_begin && threadIdx.x == 0) S.rem2 = rem2;
  const double r = sqrt(rem2);
  const double f = r > 0 ? 1.0 / r : 0.0;
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  const T2* w = (const T2*)S.w;
  T2* out = (T2*)S.V + (long long)(S.j + 1) * S.ldv;
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const double2 v = ld2(w + e);
    st2(out + e, f * v.x, f * v.y);
  }
}

// ---- FP32-basis CGS2 kernels: pairs of complex elements per 16-byte load ---------------
// Basis columns and the image vector have an even, zero-padded stride, so element pairs
// never straddle a column; padding entries stay zero through every update.

__device__ __forceinline__ void pair_range(const DevInst& S, int c, long long& beg, long long& end) {
  beg = (long long)(c - S.chunk_begin) * (S.chunk / 2);
  end = min(beg + (long long)(S.chunk / 2), (S.dim + 1) / 2);
}

// a += t, the rounding error of the addition carried in a.lo (TwoSum).
__device__ __forceinline__ void df_add(DF& a, float t) {
  const float s = a.hi + t;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (t - bb);
  a.hi = s;
  a.lo += err;
}

// a + b for double-float values (TwoSum of the leading parts).
__device__ __forceinline__ DF df_sum(DF a, DF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b.hi - bb);
  return DF{s, (a.lo + b.lo) + err};
}

// Warp sum of double-float values in FP32 arithmetic (GB300's FP64 pipe is narrow: the
// per-column reductions stay off it); the result is valid in lane 0.
__device__ __forceinline__ DF warp_df_sum(DF v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const DF o{__shfl_down_sync(0xffffffffu, v.hi, off), __shfl_down_sync(0xffffffffu, v.lo, off)};
    v = df_sum(v, o);
  }
  return v;
}

// Block sum of one double-float value; the FP64 result is valid in thread 0.
__device__ __forceinline__ double block_df_sum(DF v, float2* smem) {
  v = warp_df_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) smem[warp] = make_float2(v.hi, v.lo);
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    DF t{0.f, 0.f};
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t = df_sum(t, DF{smem[i].x, smem[i].y});
    r = (double)t.hi + (double)t.lo;
  }
  return r;
}

// CGS2 projections for an FP32 basis: partv[c][i] = conj(V_i) . w over chunk c for every
// i <= j.  The block stages its chunk of w (CH elements) in shared memory and streams every
// basis column once: per column it forms each pair term (two complex products) in FP32 and
// accumulates the terms in double-float (no rounding error in the accumulation), then the
// warp sums its lanes in FP64 into shared memory.

__device__ __forceinline__ void pair_terms(const float4 a, const float4 b, DF& re, DF& im) {
  df_add(re, fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, a.w * b.w))));
  df_add(im, fmaf(a.x, b.y, fmaf(-a.y, b.x, fmaf(a.z, b.w, -(a.w * b.z)))));
}

// With ipart (first pass of a step) the block also writes the double-float |w|^2 partial of
// its chunk for the image norm |L V_j| (the expv error estimate and the reorthogonalisation
// test) -- the same pairs in the same order as a separate sweep over w would take -- while w
// is staged anyway.
//
// Second pass with npart1 (selective reorthogonalisation, Daniel-Gragg-Kaufman-Stewart): the
// block first sums its job's |w1|^2 partials of the first-pass update; when |w1|^2 >= |w0|^2
// / 2 (w0 = L V_j before any projection, image2) the first pass left w orthogonal to the
// basis to working precision, so the block writes zero projections instead of sweeping the
// basis again, and the job's first block records the choice in reorth for the update.
template <int CH>
__global__ void __launch_bounds__(kRT, 3)
    k_step_mdot_f32(DevInst* __restrict__ st, const int* __restrict__ chunk_inst, double2* __restrict__ partv,
                    double* __restrict__ ipart, const int* __restrict__ nchunks, const double* __restrict__ npart1) {
  constexpr int kPairs = CH / 2 / kRT;  // element pairs per thread and chunk
  __shared__ float4 wsm[CH / 2];
  // per warp: (re.hi, re.lo, im.hi, im.lo) of each basis column (at most kBatchMaxKrylov + 1);
  // sized to the engine's Krylov limit so the block stays inside 48 KB of static shared memory
  __shared__ float4 red[kBatchMaxKrylov + 2][kRT / 32];
  const int inst = chunk_inst[blockIdx.x];
  DevInst& S = st[inst];
  if (S.done) return;
  const int nv = S.j + 1;
  if (npart1 != nullptr) {
    const bool reorth = job_norm2(S, nchunks[inst], npart1) < 0.5 * S.image2;  // block-uniform
    if (blockIdx.x == S.chunk_begin && threadIdx.x == 0) S.reorth = reorth ? 1 : 0;
    if (!reorth) {
      for (int kk = threadIdx.x; kk < nv; kk += blockDim.x)
        partv[(long long)blockIdx.x * kMaxDots + kk] = make_double2(0.0, 0.0);
      return;
    }
  }
  long long beg, end;
  pair_range(S, blockIdx.x, beg, end);
  const int npair = (int)(end - beg);
  const float4* __restrict__ w4 = reinterpret_cast<const float4*>(S.w) + beg;
  const float4* __restrict__ V4 = reinterpret_cast<const float4*>(S.V) + beg;
  const long long ld4 = S.ldv / 2;
  DF nrm{0.f, 0.f};
#pragma unroll
  for (int q = 0; q < kPairs; ++q) {
    const int p = threadIdx.x + q * kRT;
    const float4 wv = p < npair ? w4[p] : make_float4(0.f, 0.f, 0.f, 0.f);
    wsm[p] = wv;
    if (p < npair) df_add(nrm, fmaf(wv.x, wv.x, fmaf(wv.y, wv.y, fmaf(wv.z, wv.z, wv.w * wv.w))));
  }
  if (ipart != nullptr) {  // block-uniform
    const double r = block_df_sum(nrm, reinterpret_cast<float2*>(&red[0][0]));
    if (threadIdx.x == 0) ipart[blockIdx.x] = r;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  int k = 0;
  // two columns per iteration: 2 * kPairs independent 16-byte loads in flight per thread
  for (; k + 1 < nv; k += 2) {
    const float4* __restrict__ c0 = V4 + (long long)k * ld4;
    const float4* __restrict__ c1 = c0 + ld4;
    float4 a[kPairs], b[kPairs];
#pragma unroll
    for (int q = 0; q < kPairs; ++q) {
      const int p = threadIdx.x + q * kRT;
      a[q] = p < npair ? c0[p] : zero;
      b[q] = p < npair ? c1[p] : zero;
    }
    DF r0{0.f, 0.f}, i0{0.f, 0.f}, r1{0.f, 0.f}, i1{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < kPairs; ++q) {
      const float4 wv = wsm[threadIdx.x + q * kRT];
      pair_terms(a[q], wv, r0, i0);
      pair_terms(b[q], wv, r1, i1);
    }
    r0 = warp_df_sum(r0);
    i0 = warp_df_sum(i0);
    r1 = warp_df_sum(r1);
    i1 = warp_df_sum(i1);
    if (lane == 0) {
      red[k][warp] = make_float4(r0.hi, r0.lo, i0.hi, i0.lo);
      red[k + 1][warp] = make_float4(r1.hi, r1.lo, i1.hi, i1.lo);
    }
  }
  if (k < nv) {
    const float4* __restrict__ c0 = V4 + (long long)k * ld4;
    DF r0{0.f, 0.f}, i0{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < kPairs; ++q) {
      const int p = threadIdx.x + q * kRT;
      pair_terms(p < npair ? c0[p] : zero, wsm[p], r0, i0);
    }
    r0 = warp_df_sum(r0);
    i0 = warp_df_sum(i0);
    if (lane == 0) red[k][warp] = make_float4(r0.hi, r0.lo, i0.hi, i0.lo);
  }
  __syncthreads();
  for (int kk = threadIdx.x; kk < nv; kk += blockDim.x) {
    DF sr{0.f, 0.f}, si{0.f, 0.f};
#pragma unroll
    for (int wdx = 0; wdx < kRT / 32; ++wdx) {
      const float4 r = red[kk][wdx];
      sr = df_sum(sr, DF{r.x, r.y});
      si = df_sum(si, DF{r.z, r.w});
    }
    partv[(long long)blockIdx.x * kMaxDots + kk] =
        make_double2((double)sr.hi + (double)sr.lo, (double)si.hi + (double)si.lo);
  }
}

// cout (+)= sum_k ccoef[k] V_k for an FP32 basis in double-float arithmetic: each FP64
// coefficient is split into hi + lo floats, hi * v is formed exactly (FMA residual), lo * v
// in FP32, and the sum is carried as a double-float per component, so the FP64 output
// matches an FP64 accumulation to ~1e-14 while the FP64 pipe stays idle.
__device__ __forceinline__ void df_axpy(DF& acc, float ch, float cl, float v) {
  const float p = ch * v;
  const float e = fmaf(ch, v, -p);
  const float s = acc.hi + p;
  const float bb = s - acc.hi;
  const float err = (acc.hi - (s - bb)) + (p - bb);
  acc.hi = s;
  acc.lo += err + fmaf(cl, v, e);
}

__global__ void __launch_bounds__(kRT)
    k_s1_combine_f32(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst) {
  __shared__ float4 cs[kBatchMaxKrylov + 2];  // (re.hi, re.lo, im.hi, im.lo)
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  double2* out = S.cout;
  if (!out) return;
  const int nc = S.ccount;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) {
    const double2 c = S.ccoef[i];
    const float rh = (float)c.x, ih = (float)c.y;
    cs[i] = make_float4(rh, (float)(c.x - (double)rh), ih, (float)(c.y - (double)ih));
  }
  __syncthreads();
  long long beg, end;
  chunk_range(S, blockIdx.x, beg, end);
  const float2* __restrict__ V = reinterpret_cast<const float2*>(S.V);
  const long long ld = S.ldv;
  const int acc = S.cacc;
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    DF yr{0.f, 0.f}, yi{0.f, 0.f};
#pragma unroll 4
    for (int k = 0; k < nc; ++k) {
      const float2 v = V[(long long)k * ld + e];
      const float4 c = cs[k];
      df_axpy(yr, c.x, c.y, v.x);
      df_axpy(yr, -c.z, -c.w, v.y);
      df_axpy(yi, c.x, c.y, v.y);
      df_axpy(yi, c.z, c.w, v.x);
    }
    double ox = (double)yr.hi + (double)yr.lo, oy = (double)yi.hi + (double)yi.lo;
    if (acc) {
      const double2 o = out[e];
      ox += o.x;
      oy += o.y;
    }
    out[e] = make_double2(ox, oy);
  }
}

// w -= sum_i V_i h_i for an FP32 basis (which 0: hA, 1: hB), FP32 update; with part also
// the double-float |w|^2 partial of the result.
// With npart1 (second pass under selective reorthogonalisation) a job that skipped the second
// projection keeps w and forwards its first-pass |w1|^2 partials as this pass's partials.
__global__ void __launch_bounds__(kRT)
    k_step_maxpy_f32(const DevInst* __restrict__ st, const int* __restrict__ chunk_inst, int which,
                     double* __restrict__ part, const double* __restrict__ npart1) {
  __shared__ float2 hs[kMaxDots];
  __shared__ float2 smem[32];
  const DevInst& S = st[chunk_inst[blockIdx.x]];
  if (S.done) return;
  if (npart1 != nullptr && !S.reorth) {
    if (threadIdx.x == 0) part[blockIdx.x] = npart1[blockIdx.x];
    return;
  }
  const int nv = S.j + 1;
  const double2* h = which == 0 ? S.hA : S.hB;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) hs[i] = make_float2((float)h[i].x, (float)h[i].y);
  __syncthreads();
  long long beg, end;
  pair_range(S, blockIdx.x, beg, end);
  float4* __restrict__ w4 = reinterpret_cast<float4*>(S.w);
  const float4* __restrict__ V4 = reinterpret_cast<const float4*>(S.V);
  const long long ld4 = S.ldv / 2;
  DF nrm{0.f, 0.f};
  for (long long p = beg + threadIdx.x; p < end; p += blockDim.x) {
    float4 wv = w4[p];
#pragma unroll 4
    for (int i = 0; i < nv; ++i) {
      const float4 v = V4[(long long)i * ld4 + p];
      const float2 c = hs[i];
      wv.x = fmaf(-v.x, c.x, wv.x);
      wv.x = fmaf(v.y, c.y, wv.x);
      wv.y = fmaf(-v.x, c.y, wv.y);
      wv.y = fmaf(-v.y, c.x, wv.y);
      wv.z = fmaf(-v.z, c.x, wv.z);
      wv.z = fmaf(v.w, c.y, wv.z);
      wv.w = fmaf(-v.z, c.y, wv.w);
      wv.w = fmaf(-v.w, c.x, wv.w);
    }
    w4[p] = wv;
    df_add(nrm, fmaf(wv.x, wv.x, fmaf(wv.y, wv.y, fmaf(wv.z, wv.z, wv.w * wv.w))));
  }
  if (part) {
    const double r = block_df_sum(nrm, smem);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
  }
}

// V_{j+1} = w / |w| (zero on an exact breakdown), FP32 basis; |w|^2 as in k_step_normalize.
__global__ void __launch_bounds__(kRT)
    k_step_normalize_f32(DevInst* __restrict__ st, const int* __restrict__ chunk_inst, const int* __restrict__ nchunks,
                         const double* __restrict__ part) {
  const int inst = chunk_inst[blockIdx.x];
  DevInst& S = st[inst];
  if (S.done) return;
  const double rem2 = job_norm2(S, nchunks[inst], part);
  if (blockIdx.x == S.chunk_begin && threadIdx.x == 0) S.rem2 = rem2;
  const double r = sqrt(rem2);
  const float f = r > 0 ? (float)(1.0 / r) : 0.f;
  long long beg, end;
  pair_range(S, blockIdx.x, beg, end);
  const float4* __restrict__ w4 = reinterpret_cast<const float4*>(S.w);
  float4* __restrict__ out = reinterpret_cast<float4*>(S.V) + (long long)(S.j + 1) * (S.ldv / 2);
  for (long long p = beg + threadIdx.x; p < end; p += blockDim.x) {
    const float4 v = w4[p];
    out[p] = make_float4(f * v.x, f * v.y, f * v.z, f * v.w);
  }
}

// Per instance (one warp): records Hessenberg column j, applies the GMRES rotations and stop
// test (krylov.jl:759-777), advances j.  The warp gathers the column (hA + hB), the zero
// fill and the stored rotations into shared memory in parallel; lane 0 then runs the
// sequential rotation arithmetic on shared memory (the same operations in the same order
// as a single-thread pass over global memory, whose dependent loads dominated the step) and
// the warp writes the column back.
__global__ void __launch_bounds__(32) k_step_finish(DevInst* __restrict__ st, int n) {
  __shared__ double2 colv[kBatchMaxKrylov + 2];
  __shared__ double csv[kBatchMaxKrylov + 2];
  __shared__ double2 snv[kBatchMaxKrylov + 2];
  const int i = blockIdx.x;
  if (i >= n) return;
  DevInst& S = st[i];
  if (S.done) return;
  const int lane = threadIdx.x;
  const int j = S.j;
  const int ld = S.ldh;
  double2* col = S.H + (long long)j * ld;
  double2* cs = S.csn;
  double2* sn = S.csn + ld;
  for (int r = lane; r < ld; r += 32)
    colv[r] = r <= j ? make_double2(S.hA[r].x + S.hB[r].x, S.hA[r].y + S.hB[r].y) : make_double2(0.0, 0.0);
  if (S.givens)
    for (int r = lane; r < j; r += 32) {
      csv[r] = cs[r].x;
      snv[r] = sn[r];
    }
  __syncwarp();
  if (lane == 0) {
    const double rem = sqrt(S.rem2);
    colv[j + 1] = make_double2(rem, 0.0);
    S.image[j] = sqrt(S.image2);
    S.kdone = j + 1;
    bool stop = (j + 1 >= S.m) || rem == 0.0 || (long long)(j + 1) == S.dim;
    if (S.givens) {
      for (int r = 0; r < j; ++r) {
        const double2 h1 = colv[r], h2 = colv[r + 1];
        const double c = csv[r];
        const double2 s = snv[r];
        const double2 sh2 = cmul(s, h2);
        const double2 csh1 = cmul(conjd(s), h1);
        colv[r] = make_double2(c * h1.x + sh2.x, c * h1.y + sh2.y);
        colv[r + 1] = make_double2(-csh1.x + c * h2.x, -csh1.y + c * h2.y);
      }
      // complex Givens rotation (krylov.jl:710-716)
      const double2 a = colv[j], b = colv[j + 1];
      double c;
      double2 s;
      if (b.x == 0.0 && b.y == 0.0) {
        c = 1.0;
        s = make_double2(0.0, 0.0);
      } else if (a.x == 0.0 && a.y == 0.0) {
        c = 0.0;
        s = make_double2(1.0, 0.0);
      } else {
        const double aa = hypot(a.x, a.y), bb = hypot(b.x, b.y);
        const double sc = aa + bb;
        const double ax = a.x / sc, ay = a.y / sc, bx = b.x / sc, by = b.y / sc;
        const double normab = sc * sqrt((ax * ax + ay * ay) + (bx * bx + by * by));
        const double2 al = make_double2(a.x / aa, a.y / aa);
        c = aa / normab;
        const double2 t = cmul(al, conjd(b));
        s = make_double2(t.x / normab, t.y / normab);
      }
      cs[j] = make_double2(c, 0.0);
      sn[j] = s;
      const double2 sb = cmul(s, b);
      colv[j] = make_double2(c * a.x + sb.x, c * a.y + sb.y);
      colv[j + 1] = make_double2(0.0, 0.0);
      const double2 g1 = S.g[j], g2 = S.g[j + 1];
      const double2 sg2 = cmul(s, g2);
      const double2 csg1 = cmul(conjd(s), g1);
      S.g[j] = make_double2(c * g1.x + sg2.x, c * g1.y + sg2.y);
      S.g[j + 1] = make_double2(-csg1.x + c * g2.x, -csg1.y + c * g2.y);
      if (hypot(S.g[j + 1].x, S.g[j + 1].y) <= S.tol) stop = true;
    }
    if (stop)
      S.done = 1;
    else
      S.j = j + 1;
  }
  __syncwarp();
  for (int r = lane; r < ld; r += 32) col[r] = colv[r];
}

// Dense normalized trace vector v = t / (t^H t) in reference coordinates.
__global__ void k_fill_border_vec(const DevSector* __restrict__ sectors, const int* __restrict__ diag_sector,
                                  const long long* __restrict__ diag_index, int ndiag, double2* __restrict__ v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndiag; i += gridDim.x * blockDim.x)
    v[diag_index[i]] = make_double2(sectors[diag_sector[i]].border_x, 0.0);
}

template <typename K>
void set_smem(K kernel, size_t bytes, cudaError_t& err) {
  const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess && err == cudaSuccess) err = e;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// Job base
// ---------------------------------------------------------------------------------------

Job::~Job() {
  for (void* p : allocs_) cudaFreeAsync(p, s_);
}

void* Job::alloc(size_t b, cudaError_t* err) {
  void* p = nullptr;
  const cudaError_t e = cudaMallocAsync(&p, b ? b : 16, s_);
  if (e != cudaSuccess) {
    *err = e;
    return nullptr;
  }
  allocs_.push_back(p);
  bytes += b;
  return p;
}

void Job::fail_job(int code, const std::string& m) {
  if (rc == PI_OK) {
    rc = code;
    msg = m;
  }
  finished = true;
}

// ---------------------------------------------------------------------------------------
// Dynamics job
// ---------------------------------------------------------------------------------------

DynamicsJob::DynamicsJob(pi_plan* p, double* state, std::vector<double> times, int nobs, const double* obs,
                         double* values, const pi_expv_opts_t& o, bool single_interval)
    : state_(state), times_(std::move(times)), nobs_(nobs), obs_(obs), values_(values), o_(o), single_(single_interval) {
  plan = p;
  dim = p->host.dim;
}

bool DynamicsJob::setup(cudaStream_t s, int m, bool f32) {
  s_ = s;
  m_engine = m;
  ldh = m + 2;
  mixed_ = f32;
  cudaError_t e = cudaSuccess;
  const size_t es = f32 ? sizeof(float2) : sizeof(double2);
  ldv = basis_stride(dim);
  V = alloc(es * (size_t)ldv * (m + 2), &e);
  w = alloc(es * (size_t)ldv, &e);
  if (e == cudaSuccess) e = cudaMemsetAsync(V, 0, es * (size_t)ldv * (m + 2), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w, 0, es * (size_t)ldv, s);
  cur_ = (double2*)alloc(sizeof(double2) * dim, &e);
  trial_ = (double2*)alloc(sizeof(double2) * dim, &e);
  if (nobs_ > 0 && mixed_) obsz_ = (double2*)alloc(sizeof(double2) * dim * nobs_, &e);
  if (e != cudaSuccess) return false;
  const DevicePlan& dp = plan->dev;
  if (mixed_) {
    // population coordinates: z = sqrt(f) x; observables dot(O, x) = dot(O / sqrt(f), z)
    e = x_to_z_f64(dp, (const double2*)state_, cur_, 1.0, s);
    for (int o = 0; o < nobs_ && e == cudaSuccess; ++o)
      e = z_to_x_f64(dp, (const double2*)obs_ + (size_t)o * dim, obsz_ + (size_t)o * dim, 1.0, 0, s);
  } else {
    e = cudaMemcpyAsync(cur_, state_, sizeof(double2) * dim, cudaMemcpyDeviceToDevice, s);
  }
  if (e != cudaSuccess) return false;
  obs_pending_ = nobs_ > 0 ? 0 : -1;
  need_norm_ = true;
  return true;
}

unsigned DynamicsJob::stage1(DevInst& d, double2* coef) {
  unsigned f = 0;
  if (obs_pending_ >= 0) {
    d.nob = nobs_;
    d.ob = mixed_ ? obsz_ : (const double2*)obs_;
    d.obx = cur_;
    f |= S1_OBS;
  }
  if (pending_trial_) {
    d.cout = trial_;
    d.ccount = (int)coef_.size();
    d.cacc = 0;
    for (size_t k = 0; k < coef_.size(); ++k) coef[k] = make_double2(coef_[k].real(), coef_[k].imag());
    d.nrm0 = trial_;
    f |= S1_COMBINE | S1_NORM;
  } else if (need_norm_) {
    d.nrm0 = cur_;
    f |= S1_NORM;
  }
  return f;
}

void DynamicsJob::begin_interval() {
  // Zero-length intervals keep the state; their saved values equal the previous ones.
  while (interval_ < (int)times_.size() && times_[interval_] == times_[interval_ - 1]) {
    if (nobs_ > 0) {
      if (obs_pending_ >= 0)
        zero_copies_.push_back(interval_);
      else
        std::memcpy(values_ + (size_t)interval_ * nobs_ * 2, values_ + (size_t)(interval_ - 1) * nobs_ * 2,
                    sizeof(double) * 2 * nobs_);
    }
    ++interval_;
  }
  if (interval_ >= (int)times_.size()) {
    if (obs_pending_ < 0) finished = true;
    return;
  }
  const double dt = times_[interval_] - times_[interval_ - 1];
  total_ = std::abs(dt);
  direction_ = dt < 0 ? -1.0 : 1.0;
  hmax_ = o_.maximum_step > 0 ? o_.maximum_step : total_;
  hmin_ = o_.minimum_step > 0 ? o_.minimum_step : 0.0;
  const double h0 = o_.initial_step > 0 ? o_.initial_step : hmax_;
  hmax_ = std::min(hmax_, total_);
  h_ = std::min(h0, hmax_);
  if (hmin_ > hmax_) return fail_job(PI_ERR_INVALID_ARGUMENT, "minimum_step must not exceed the effective maximum step");
  if (h0 < hmin_) return fail_job(PI_ERR_INVALID_ARGUMENT, "initial_step must not be smaller than minimum_step");
  reached_ = 0.0;
  attempts_ = 0;
  have_ = false;
  attempt();
}

// One trial of krylov_expv!'s loop: factorize if needed, else project again.
void DynamicsJob::attempt() {
  if (attempts_ >= o_.max_steps) {
    char m[200];
    std::snprintf(m, sizeof(m), "adaptive Krylov exponential action reached time %.17g of %.17g after %d attempts",
                  direction_ * reached_, direction_ * total_, attempts_);
    converged_ = false;
    return fail_job(PI_ERR_NOT_CONVERGED, m);
  }
  ++attempts_;
  ++trials_;
  h_ = std::min(h_, total_ - reached_);
  if (!have_)
    want_factor_ = true;
  else
    project();
}

bool DynamicsJob::cycle(DevInst& d) {
  if (!want_factor_ || finished) return false;
  want_factor_ = false;
  ++factorizations_;
  have_ = true;
  beta_ = cur_norm_;
  enlarged_ = false;
  next_rem_ = 0.0;
  if (!std::isfinite(beta_)) {
    fail_job(PI_ERR_INVALID_ARGUMENT, "exponential-action state is not finite");
    return false;
  }
  if (beta_ == 0.0) {
    zero_ = true;
    completed_ = true;
    k_ = q_ = 0;
    project();
    return false;
  }
  zero_ = false;
  d.v0 = cur_;
  d.v0norm = beta_;
  d.m = (int)std::min<long long>(m_engine, dim);
  d.coords = mixed_ ? 1 : 0;
  d.coefb = mixed_ ? (const void*)plan->dev.coef32z : (const void*)plan->dev.coef64;
  d.border = 0;
  d.givens = 0;
  d.scale = 1.0;
  d.tol = 0.0;
  d.j = 0;
  d.done = 0;
  return true;
}

bool DynamicsJob::after_cycle(const DevInst& r, const double2* rec, DevInst& d) {
  const int k = r.kdone;
  const double* image = (const double*)(rec + (size_t)(m_engine + 4) * ldh);
  applications_ += k;
  const double breakfactor = std::sqrt(std::numeric_limits<double>::epsilon());
  const double rem_last = rec[(size_t)(k - 1) * ldh + k].x;
  const bool exact = rem_last == 0.0 || (long long)k == dim;
  bool near = false;
  for (int jj = 0; jj < k; ++jj) {
    const double rem = rec[(size_t)jj * ldh + jj + 1].x;
    if (!std::isfinite(rem)) {
      fail_job(PI_ERR_INVALID_ARGUMENT, "exponential-action Arnoldi remainder is not finite");
      return false;
    }
    if (!std::isfinite(image[jj])) {
      fail_job(PI_ERR_INVALID_ARGUMENT, "exponential-action Arnoldi image is not finite");
      return false;
    }
    if (jj < k - 1 || !exact) near |= rem <= breakfactor * std::max(image[jj], std::numeric_limits<double>::min());
  }
  k_ = k;
  q_ = k + (exact ? 0 : 1);
  S_.assign((size_t)q_ * q_, std::complex<double>(0, 0));
  for (int l = 0; l < k; ++l)
    for (int i = 0; i < k; ++i)
      S_[(size_t)l * q_ + i] = std::complex<double>(rec[(size_t)l * ldh + i].x, rec[(size_t)l * ldh + i].y);
  if (!exact) S_[(size_t)(k - 1) * q_ + k] = std::complex<double>(rem_last, 0.0);
  completed_ = exact;
  if (!exact && near) {
    d.coords = mixed_ ? 1 : 0;
    d.coefb = mixed_ ? (const void*)plan->dev.coef32z : (const void*)plan->dev.coef64;
    d.scale = 1.0;
    d.m = k + 1;
    d.j = k;
    d.done = 0;
    return true;
  }
  project();
  return false;
}

void DynamicsJob::after_enlarge(const DevInst& r, const double2* rec) {
  (void)r;
  const int col = q_ - 1;
  const double* image = (const double*)(rec + (size_t)(m_engine + 4) * ldh);
  for (int i = 0; i < q_; ++i)
    S_[(size_t)col * q_ + i] += std::complex<double>(rec[(size_t)col * ldh + i].x, rec[(size_t)col * ldh + i].y);
  next_rem_ = rec[(size_t)col * ldh + q_].x;
  applications_ += 1;
  if (!std::isfinite(next_rem_))
    return fail_job(PI_ERR_INVALID_ARGUMENT, "exponential-action enlarged Arnoldi remainder is not finite");
  if (!std::isfinite(image[col]))
    return fail_job(PI_ERR_INVALID_ARGUMENT, "exponential-action enlarged Arnoldi image is not finite");
  enlarged_ = true;
  completed_ = ((long long)q_ == dim) || next_rem_ == 0.0;
  project();
}

// _expv_project_factorization! (krylov_extensions.jl:1403-1426).
void DynamicsJob::project() {
  pending_trial_ = true;
  coef_.clear();
  if (zero_) {
    err_ = 0.0;
    return;
  }
  const double h = direction_ * h_;
  CMat A(q_);
  for (int i = 0; i < q_; ++i)
    for (int l = 0; l < q_; ++l) A(i, l) = h * S_[(size_t)l * q_ + i];
  const CMat E = expm(A);
  const int cc = enlarged_ ? q_ : k_;
  coef_.resize(cc);
  for (int i = 0; i < cc; ++i) coef_[i] = beta_ * E(i, 0);
  if (completed_)
    err_ = 0.0;
  else if (enlarged_)
    err_ = beta_ * std::abs(h) * next_rem_ * std::abs(E(q_ - 1, 0));
  else
    err_ = beta_ * std::abs(E(k_, 0));
}

void DynamicsJob::interval_done() {
  if (nobs_ > 0) obs_pending_ = interval_;
  reached_time_ = times_[interval_];
  ++interval_;
  begin_interval();
}

void DynamicsJob::after_stage1(const double* out) {
  if (obs_pending_ >= 0) {
    const int i = obs_pending_;
    for (int o = 0; o < nobs_; ++o) {
      values_[((size_t)i * nobs_ + o) * 2] = out[4 + 2 * o];
      values_[((size_t)i * nobs_ + o) * 2 + 1] = out[5 + 2 * o];
    }
    obs_pending_ = -1;
    // saved times after zero-length intervals repeat these values
    for (int z : zero_copies_)
      std::memcpy(values_ + (size_t)z * nobs_ * 2, values_ + (size_t)i * nobs_ * 2, sizeof(double) * 2 * nobs_);
    zero_copies_.clear();
    if (interval_ >= (int)times_.size() && !pending_trial_ && !want_factor_ && !need_norm_) finished = true;
  }
  if (need_norm_) {
    need_norm_ = false;
    cur_norm_ = std::sqrt(out[0]);
    begin_interval();
    return;
  }
  if (!pending_trial_) return;
  pending_trial_ = false;
  const double error = err_;
  double trial_norm = std::sqrt(out[0]);
  const bool finite = std::isfinite(trial_norm) && std::isfinite(error);
  if (!finite) {
    trial_norm = cur_norm_;
    if (!std::isfinite(trial_norm)) return fail_job(PI_ERR_INVALID_ARGUMENT, "exponential-action state is not finite");
  }
  const double localtol = (h_ / total_) * (o_.atol + o_.rtol * trial_norm);
  if (!std::isfinite(localtol))
    return fail_job(PI_ERR_INVALID_ARGUMENT,
                    "exponential-action local tolerance overflowed; rescale the state or use wider precision");
  const bool accept = finite && (completed_ || error <= localtol);
  if (accept) {
    std::swap(cur_, trial_);
    cur_norm_ = trial_norm;
    const double remaining = total_ - reached_;
    const double next = (h_ == remaining) ? total_ : reached_ + h_;
    if (!(next > reached_))
      return fail_job(PI_ERR_INVALID_ARGUMENT,
                      "exponential-action time step no longer advances; use fewer steps or wider precision");
    reached_ = next;
    ++accepted_;
    error_sum_ += error;
    have_ = false;
  } else {
    ++rejected_;
  }
  double factor;
  if (!finite)
    factor = 0.2;
  else if (completed_)
    factor = 5.0;
  else if (error == 0.0)
    factor = 2.0;
  else {
    factor = o_.safety * std::pow(localtol / error, 1.0 / (double)std::max(k_, 1));
    factor = std::min(std::max(factor, 0.2), 5.0);
  }
  if (!accept) factor = std::min(factor, 0.5);
  const double hnew = std::min(hmax_, h_ * factor);
  if (!accept && (hnew < hmin_ || hnew == 0.0 || (reached_ > 0.0 && reached_ + hnew == reached_))) {
    char m[200];
    std::snprintf(m, sizeof(m), "adaptive Krylov exponential action reached time %.17g of %.17g after %d attempts",
                  direction_ * reached_, direction_ * total_, attempts_);
    converged_ = false;
    return fail_job(PI_ERR_NOT_CONVERGED, m);
  }
  h_ = std::max(hnew, hmin_);
  if (reached_ < total_)
    attempt();
  else
    interval_done();
}

void DynamicsJob::finish(cudaStream_t s) {
  if (mixed_)
    z_to_x_f64(plan->dev, cur_, (double2*)state_, 1.0, 0, s);
  else
    cudaMemcpyAsync(state_, cur_, sizeof(double2) * dim, cudaMemcpyDeviceToDevice, s);
}

pi_expv_info_t DynamicsJob::info() const {
  pi_expv_info_t I;
  std::memset(&I, 0, sizeof(I));
  I.converged = rc == PI_OK && converged_;
  I.reached_time = single_ ? direction_ * reached_ : reached_time_;
  I.accepted_steps = accepted_;
  I.rejected_steps = rejected_;
  I.operator_applications = applications_;
  I.arnoldi_factorizations = factorizations_;
  I.trial_evaluations = trials_;
  I.estimated_error = error_sum_;
  return I;
}

// ---------------------------------------------------------------------------------------
// Steady-state job
// ---------------------------------------------------------------------------------------

SteadyJob::SteadyJob(pi_plan* p, double* x, const pi_gmres_opts_t& o, unsigned long long seed, bool host_probes)
    : x_((double2*)x), o_(o), seed_(seed), host_probes_(host_probes) {
  plan = p;
  dim = p->host.dim;
  bordered = true;
}

bool SteadyJob::setup(cudaStream_t s, int m, bool f32) {
  s_ = s;
  m_engine = m;
  ldh = m + 2;
  mixed_ = f32;
  m_ = (int)std::min<long long>(std::min(o_.krylovdim, m), dim);
  cudaError_t e = cudaSuccess;
  const size_t es = f32 ? sizeof(float2) : sizeof(double2);
  ldv = basis_stride(dim);
  V = alloc(es * (size_t)ldv * (m + 2), &e);
  w = alloc(es * (size_t)ldv, &e);
  if (e == cudaSuccess) e = cudaMemsetAsync(V, 0, es * (size_t)ldv * (m + 2), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w, 0, es * (size_t)ldv, s);
  b_ = (double2*)alloc(sizeof(double2) * dim, &e);
  r_ = (double2*)alloc(sizeof(double2) * dim, &e);
  ay_ = (double2*)alloc(sizeof(double2) * dim, &e);
  if (e != cudaSuccess) return false;
  const DevicePlan& dp = plan->dev;
  e = cudaMemsetAsync(b_, 0, sizeof(double2) * dim, s);
  if (e == cudaSuccess) {
    const int grid = std::max(1, std::min(608, (dp.ndiag + 255) / 256));
    k_fill_border_vec<<<grid, 256, 0, s>>>(dp.sectors, dp.diag_sector, dp.diag_index, dp.ndiag, b_);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && !o_.use_initial) e = cudaMemcpyAsync(x_, b_, sizeof(double2) * dim, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return false;
  if (host_probes_ && o_.operator_scale <= 0) {
    // krylov.jl:156-169 draws three complex normal probes from a seeded generator
    probes_ = (double2*)alloc(sizeof(double2) * dim * 3, &e);
    if (e != cudaSuccess) return false;
    std::vector<double2> h((size_t)dim * 3);
    std::mt19937_64 rng(seed_);
    std::normal_distribution<double> nd(0.0, 1.0);
    // same expression as the host-driven solver (argument evaluation order included)
    for (size_t i = 0; i < h.size(); ++i) h[i] = make_double2(nd(rng) * M_SQRT1_2, nd(rng) * M_SQRT1_2);
    e = cudaMemcpyAsync(probes_, h.data(), sizeof(double2) * h.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // h is released on return
    if (e != cudaSuccess) return false;
  }
  state_ = INIT;
  return true;
}

unsigned SteadyJob::stage1(DevInst& d, double2* coef) {
  switch (state_) {
    case INIT:
      d.nrm0 = b_;
      return S1_NORM;
    case SCALE:
      if (probes_) {
        const double2* pr = probes_ + (size_t)probe_ * dim;
        d.ax = pr;
        d.nrm0 = pr;
      } else {
        d.probe = r_;
        d.seed = seed_ * 4 + (unsigned long long)probe_;
        d.ax = r_;
        d.nrm0 = r_;
      }
      d.ay = ay_;
      d.aux_scale = 1.0;
      d.aux_border = 0;
      d.nrm1 = ay_;
      return (probes_ ? 0u : S1_PROBE) | S1_AUX | S1_NORM;
    case RESID: {
      unsigned f = 0;
      if (pending_update_) {
        d.cout = x_;
        d.ccount = (int)y_.size();
        d.cacc = 1;
        for (size_t k = 0; k < y_.size(); ++k) coef[k] = make_double2(y_[k].real(), y_[k].imag());
        f |= S1_COMBINE;
        pending_update_ = false;
      }
      d.ax = x_;
      d.ay = ay_;
      d.aux_scale = 1.0 / s_op_;
      d.aux_border = 1;
      d.rb = b_;
      d.rout = r_;
      d.nrm0 = r_;
      return f | S1_AUX | S1_RESID | S1_NORM;
    }
    case FINAL:
      d.ax = x_;
      d.ay = ay_;
      d.aux_scale = 1.0;
      d.aux_border = 0;
      d.nrm0 = ay_;
      d.nrm1 = x_;
      d.tr = x_;
      return S1_AUX | S1_NORM | S1_TRACE;
    default:
      return 0;
  }
}

void SteadyJob::after_stage1(const double* out) {
  switch (state_) {
    case INIT:
      tol_ = o_.atol + o_.rtol * std::sqrt(out[0]);
      if (o_.operator_scale > 0) {
        s_op_ = o_.operator_scale;
        state_ = RESID;
      } else {
        state_ = SCALE;
        probe_ = 0;
        scale_ = 0.0;
      }
      break;
    case SCALE:
      // krylov.jl:156-169: max |L r| / |r| over three complex normal probes
      ++applications_;
      scale_ = std::max(scale_, std::sqrt(out[1]) / std::sqrt(out[0]));
      if (++probe_ == 3) {
        s_op_ = scale_;
        if (!(std::isfinite(s_op_) && s_op_ > 0))
          return fail_job(PI_ERR_INVALID_ARGUMENT,
                          "operator_scale must be finite and positive; a numerically zero Liouvillian does not define "
                          "a unique trace-fixed Krylov solve");
        state_ = RESID;
      }
      break;
    case RESID:
      ++applications_;
      beta_ = std::sqrt(out[0]);
      linear_residual_ = beta_;
      if (beta_ <= tol_) {
        gm_converged_ = true;
        state_ = FINAL;
      } else if (iterations_ >= o_.maxiter || (mixed_ && refinements_ >= std::max(1, o_.max_refinements))) {
        state_ = FINAL;
      } else {
        if (mixed_) ++refinements_;
        want_cycle_ = true;
      }
      break;
    case FINAL: {
      ++applications_;
      const double residual = std::sqrt(out[0]);
      const double normalized = residual / s_op_;
      const double xn = std::sqrt(out[1]);
      const double terr = std::abs(std::complex<double>(out[2], out[3]) - std::complex<double>(1, 0));
      const double tol = o_.atol + o_.rtol * std::max(xn, 1.0);
      std::memset(&info_, 0, sizeof(info_));
      info_.converged = gm_converged_ && normalized <= tol && terr <= o_.atol + o_.rtol;
      info_.iterations = iterations_;
      info_.restarts = restarts_;
      info_.refinements = refinements_;
      info_.operator_applications = applications_;
      info_.residual = residual;
      info_.normalized_residual = normalized;
      info_.trace_error = terr;
      info_.operator_scale = s_op_;
      info_.linear_residual = linear_residual_;
      state_ = DONE;
      finished = true;
      if (!info_.converged) {
        char m[256];
        std::snprintf(m, sizeof(m),
                      "matrix-free Krylov steady-state solve did not converge in %d iterations; "
                      "normalized_residual=%.3e, trace_error=%.3e",
                      iterations_, normalized, terr);
        rc = PI_ERR_NOT_CONVERGED;
        msg = m;
      }
      break;
    }
    default:
      break;
  }
}

bool SteadyJob::cycle(DevInst& d) {
  if (!want_cycle_ || finished) return false;
  want_cycle_ = false;
  d.v0 = r_;
  d.v0norm = beta_;
  d.m = std::min(m_, o_.maxiter - iterations_);
  d.border = 1;
  d.givens = 1;
  d.scale = 1.0 / s_op_;
  d.coords = 0;
  d.coefb = mixed_ ? (const void*)plan->dev.coef32x : (const void*)plan->dev.coef64;
  // FP32 inner solves stop at a relative reduction they can resolve; the FP64 outer
  // residual restores the rest.
  d.tol = mixed_ ? std::max(tol_ * 0.5, 1e-5 * beta_) : tol_;
  d.j = 0;
  d.done = 0;
  return true;
}

bool SteadyJob::after_cycle(const DevInst& r, const double2* rec, DevInst&) {
  const int k = r.kdone;
  iterations_ += k;
  applications_ += k;
  if (k == 0) {
    state_ = FINAL;
    return false;
  }
  const double2* g = rec + (size_t)(m_engine + 1) * ldh;
  y_.assign(k, std::complex<double>(0, 0));
  for (int i = k - 1; i >= 0; --i) {
    std::complex<double> s(g[i].x, g[i].y);
    for (int jj = i + 1; jj < k; ++jj) {
      const double2 h = rec[(size_t)jj * ldh + i];
      s -= std::complex<double>(h.x, h.y) * y_[jj];
    }
    const double2 hd = rec[(size_t)i * ldh + i];
    if (hd.x == 0.0 && hd.y == 0.0) {
      fail_job(PI_ERR_NOT_CONVERGED, "singular GMRES triangular factor");
      return false;
    }
    y_[i] = s / std::complex<double>(hd.x, hd.y);
  }
  ++restarts_;
  pending_update_ = true;
  state_ = RESID;
  return false;
}

// ---------------------------------------------------------------------------------------
// Engine
// ---------------------------------------------------------------------------------------

Engine::Engine(int device, int krylovdim, bool f32, bool use_graphs)
    : device_(device), m_(krylovdim), f32_(f32), graphs_(use_graphs) {
  chk(cudaSetDevice(device));
  chk(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
  // Job workspaces come from the device's default memory pool; keep freed memory in the
  // pool so that admitting the next requests does not go back to the driver.
  cudaMemPool_t pool = nullptr;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess && pool) {
    unsigned long long keep = ~0ULL;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  const size_t smem64 = 3 * kWinElems * sizeof(double2);
  const size_t smem32 = 3 * kWinElems * sizeof(float2);
  set_smem(k_bapply<double, true>, smem64, err);
  set_smem(k_bapply<double, false>, smem64, err);
  set_smem(k_bapply<float, false>, smem32, err);
  set_smem(k_bapply_persist, kSepSmemBytes, err);
  chk(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&persist_max_, k_bapply_persist, kApplyThreads,
                                                    kSepSmemBytes) != cudaSuccess) {
    persist_max_ = 0;
    (void)cudaGetLastError();  // no persistent schedule; the error is not the engine's
  }
  rec_stride_ = (size_t)(m_ + 5) * (m_ + 2);
}

Engine::~Engine() {
  if (graph_) cudaGraphExecDestroy(graph_);
  if (s_) cudaStreamSynchronize(s_);
  for (void* p : {st_, tile_inst_, tile_local_, chunk_inst_, nchunks_, part1_, partv_, hab_, rec_, out_, coefs_})
    if (p) cudaFree(p);
  for (void* p : {st_h_, st_dl_, rec_h_, out_h_, coefs_h_})
    if (p) cudaFreeHost(p);
  if (s_) cudaStreamDestroy(s_);
}

void Engine::reserve(void** p, size_t* cap, size_t bytes, bool pinned) {
  if (bytes <= *cap && *p) return;
  chk(cudaStreamSynchronize(s_));
  if (*p) {
    if (pinned)
      cudaFreeHost(*p);
    else
      cudaFree(*p);
    *p = nullptr;
  }
  const size_t nb = std::max(bytes + bytes / 2, (size_t)256);
  chk(pinned ? cudaMallocHost(p, nb) : cudaMalloc(p, nb));
  *cap = *p ? nb : 0;
}

void Engine::add(Job* j) {
  jobs_.push_back(j);
  dirty_ = true;
}

std::vector<Job*> Engine::retire() {
  std::vector<Job*> done, keep;
  for (Job* j : jobs_) (j->finished ? done : keep).push_back(j);
  if (!done.empty()) {
    jobs_.swap(keep);
    dirty_ = true;
  }
  return done;
}

void Engine::rebuild() {
  const int n = (int)jobs_.size();
  const size_t nn = std::max(n, 1);
  // Chunk size: large chunks amortise the per-block reductions; when the active jobs hold
  // fewer elements than about eight large chunks per SM, small chunks keep the GPU full.
  long long total_elems = 0;
  for (int i = 0; i < n; ++i) total_elems += jobs_[i]->dim;
  chunk_ = total_elems >= 8LL * 152 * kBatchChunk ? kBatchChunk : kBatchChunkSmall;
  // the trace of each step's input column is only needed by bordered (steady-state) cycles
  any_border_ = false;
  for (int i = 0; i < n; ++i) any_border_ = any_border_ || jobs_[i]->bordered;
  std::vector<int> ti, tl, ci, nc(n);
  for (int i = 0; i < n; ++i) {
    const int ntiles = jobs_[i]->plan->dev.ntiles;
    for (int t = 0; t < ntiles; ++t) {
      ti.push_back(i);
      tl.push_back(t);
    }
    nc[i] = (int)((jobs_[i]->dim + chunk_ - 1) / chunk_);
  }
  reserve(&hab_, &hab_cap_, sizeof(double2) * 2 * kMaxDots * nn, false);
  reserve(&rec_, &rec_cap_, sizeof(double2) * rec_stride_ * nn, false);
  reserve(&out_, &out_cap_, sizeof(double) * kOutSlots * nn, false);
  reserve(&coefs_, &coefs_cap_, sizeof(double2) * (m_ + 2) * nn, false);
  base_.assign(n, DevInst());
  for (int i = 0; i < n; ++i) {
    Job* J = jobs_[i];
    const DevicePlan& dp = J->plan->dev;
    DevInst& d = base_[i];
    std::memset(&d, 0, sizeof(d));
    d.sectors = dp.sectors;
    d.terms = dp.terms;
    d.tiles = dp.tiles;
    d.coef64 = dp.coef64;
    d.coefb = f32_ ? (const void*)dp.coef32x : (const void*)dp.coef64;
    d.diag_sector = dp.diag_sector;
    d.diag_index = dp.diag_index;
    d.dim = J->dim;
    d.ldv = J->ldv;
    d.ndiag = dp.ndiag;
    d.chunk_begin = (int)ci.size();
    d.chunk = chunk_;
    // FP32 Arnoldi applies of canonical plans read merged coefficients: dynamics cycles run in
    // population coordinates, steady-state cycles in reference coordinates
    d.planes = SplitPlanes{nullptr, nullptr, nullptr, nullptr, 0};
    d.pwhich = J->bordered ? 0 : 1;
    if (f32_ && dp.canon && em_split_planes(J->plan, d.pwhich, &d.planes) != PI_OK)
      d.planes = SplitPlanes{nullptr, nullptr, nullptr, nullptr, 0};
    for (int c = 0; c < nc[i]; ++c) ci.push_back(i);
    d.V = J->V;
    d.w = J->w;
    d.hA = (double2*)hab_ + (size_t)i * 2 * kMaxDots;
    d.hB = d.hA + kMaxDots;
    double2* rec = (double2*)rec_ + (size_t)i * rec_stride_;
    d.H = rec;
    d.g = rec + (size_t)(m_ + 1) * (m_ + 2);
    d.csn = rec + (size_t)(m_ + 2) * (m_ + 2);
    d.image = (double*)(rec + (size_t)(m_ + 4) * (m_ + 2));
    d.ldh = m_ + 2;
    d.ccoef = (const double2*)coefs_ + (size_t)i * (m_ + 2);
    d.out = (double*)out_ + (size_t)i * kOutSlots;
    d.scale = 1.0;
    d.aux_scale = 1.0;
    d.done = 1;
  }
  total_tiles_ = (int)ti.size();
  total_chunks_ = (int)ci.size();
  reserve(&st_, &st_cap_, sizeof(DevInst) * nn, false);
  reserve(&tile_inst_, &tile_inst_cap_, sizeof(int) * std::max<size_t>(ti.size(), 1), false);
  reserve(&tile_local_, &tile_local_cap_, sizeof(int) * std::max<size_t>(tl.size(), 1), false);
  reserve(&chunk_inst_, &chunk_inst_cap_, sizeof(int) * std::max<size_t>(ci.size(), 1), false);
  reserve(&nchunks_, &nchunks_cap_, sizeof(int) * nn, false);
  reserve(&part1_, &part1_cap_, sizeof(double) * 2 * std::max(total_chunks_, 1), false);
  reserve(&partv_, &partv_cap_, sizeof(double2) * kMaxDots * std::max(total_chunks_, 1), false);
  reserve(&st_h_, &st_h_cap_, sizeof(DevInst) * nn, true);
  reserve(&st_dl_, &st_dl_cap_, sizeof(DevInst) * nn, true);
  reserve(&rec_h_, &rec_h_cap_, sizeof(double2) * rec_stride_ * nn, true);
  reserve(&out_h_, &out_h_cap_, sizeof(double) * kOutSlots * nn, true);
  reserve(&coefs_h_, &coefs_h_cap_, sizeof(double2) * (m_ + 2) * nn, true);
  if (!ti.empty()) chk(cudaMemcpyAsync(tile_inst_, ti.data(), sizeof(int) * ti.size(), cudaMemcpyHostToDevice, s_));
  if (!tl.empty()) chk(cudaMemcpyAsync(tile_local_, tl.data(), sizeof(int) * tl.size(), cudaMemcpyHostToDevice, s_));
  if (!ci.empty()) chk(cudaMemcpyAsync(chunk_inst_, ci.data(), sizeof(int) * ci.size(), cudaMemcpyHostToDevice, s_));
  if (n) chk(cudaMemcpyAsync(nchunks_, nc.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s_));
  chk(cudaStreamSynchronize(s_));  // the host vectors above go out of scope
  if (graph_) {
    cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
  }
  schedule_chosen_ = false;
  dirty_ = false;
}

namespace {

// Process-wide schedule setting, choice cache and the record of the last choice.
std::atomic<int> g_apply_schedule{PI_SCHEDULE_AUTO};
std::mutex g_schedule_mu;
std::map<long long, int> g_schedule_cache;  // (device, job-set shape) -> schedule
pi_schedule_info_t g_schedule_info{};

}  // namespace

void Engine::launch_step_apply(int schedule) {
  DevInst* st = (DevInst*)st_;
  const int* ti = (const int*)tile_inst_;
  const int* tl = (const int*)tile_local_;
  if (schedule > 0) {
    const int grid = std::max(1, std::min(total_tiles_, schedule * sm_count_));
    launch(k_bapply_persist, grid, kApplyThreads, kSepSmemBytes, (const DevInst*)st, ti, tl, total_tiles_);
  } else {
    launch(k_bapply<float, false>, total_tiles_, kApplyThreads, 3 * kWinElems * sizeof(float2), (const DevInst*)st,
           ti, tl);
  }
}

// Picks the FP32 step-apply schedule of the current job set.  Runs on the engine stream
// after the cycle's control blocks and first basis columns are on the device and before the
// cycle's steps are launched or captured: the timed applies write only each running job's
// step column w, which the first step overwrites.
void Engine::choose_apply_schedule() {
  schedule_chosen_ = true;
  apply_schedule_ = PI_SCHEDULE_PER_TILE;
  if (!f32_ || total_tiles_ == 0 || persist_max_ < 1 || sm_count_ < 1) return;
  const int setting = g_apply_schedule.load();
  bool general = false;
  for (const DevInst& d : base_) general = general || d.planes.srow == nullptr;
  int size_class = 0;
  while ((2LL << size_class) <= total_tiles_) ++size_class;
  const long long key = ((long long)device_ << 16) | (size_class << 1) | (general ? 1 : 0);
  pi_schedule_info_t rec{};
  rec.items = total_tiles_;
  rec.resident_max = persist_max_;
  if (setting != PI_SCHEDULE_AUTO) {
    apply_schedule_ = setting > 0 ? std::min(setting, persist_max_) : PI_SCHEDULE_PER_TILE;
  } else {
    bool cached = false;
    {
      std::lock_guard<std::mutex> lk(g_schedule_mu);
      auto it = g_schedule_cache.find(key);
      if (it != g_schedule_cache.end()) {
        apply_schedule_ = std::min(it->second, persist_max_);
        cached = true;
      }
    }
    if (!cached) {
      std::vector<int> cand{PI_SCHEDULE_PER_TILE};
      for (int b = 1; b <= std::min(persist_max_, 7); ++b) cand.push_back(b);
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      chk(cudaEventCreate(&e0));
      chk(cudaEventCreate(&e1));
      constexpr int kReps = 3;
      double best = 0;
      for (size_t c = 0; c < cand.size() && err == cudaSuccess; ++c) {
        launch_step_apply(cand[c]);  // warm-up
        float t[kReps];
        for (int r = 0; r < kReps; ++r) {
          chk(cudaEventRecord(e0, s_));
          launch_step_apply(cand[c]);
          chk(cudaEventRecord(e1, s_));
          chk(cudaEventSynchronize(e1));
          t[r] = 0.f;
          chk(cudaEventElapsedTime(&t[r], e0, e1));
        }
        std::sort(t, t + kReps);
        const double us = 1e3 * t[kReps / 2];
        rec.cand[rec.ncand] = cand[c];
        rec.cand_us[rec.ncand] = us;
        ++rec.ncand;
        if (c == 0 || us < best) {
          best = us;
          apply_schedule_ = cand[c];
        }
      }
      chk(cudaGetLastError());
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      if (err == cudaSuccess) {
        std::lock_guard<std::mutex> lk(g_schedule_mu);
        g_schedule_cache[key] = apply_schedule_;
        ++g_schedule_info.tunings;
      }
    }
  }
  std::lock_guard<std::mutex> lk(g_schedule_mu);
  rec.choices = g_schedule_info.choices + 1;
  rec.tunings = g_schedule_info.tunings;
  rec.schedule = apply_schedule_;
  g_schedule_info = rec;
}

// Launches a kernel on the engine stream, or appends it as the next node of the graph under
// construction (explicit kernel nodes, no stream capture: a capture would forbid
// device-wide synchronisation by other host threads, e.g. a serving client).
template <typename... KArgs, typename... Args>
void Engine::launch(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, Args... args) {
  if (!build_) {
    k<<<grid, block, smem, s_>>>(args...);
    return;
  }
  std::tuple<KArgs...> vals(args...);
  void* ptrs[sizeof...(KArgs)];
  fill_ptrs(vals, ptrs, std::index_sequence_for<KArgs...>{});
  cudaKernelNodeParams p{};
  p.func = reinterpret_cast<void*>(k);
  p.gridDim = grid;
  p.blockDim = block;
  p.sharedMemBytes = (unsigned)smem;
  p.kernelParams = ptrs;
  p.extra = nullptr;
  cudaGraphNode_t node = nullptr;
  chk(cudaGraphAddKernelNode(&node, build_, last_ ? &last_ : nullptr, last_ ? 1 : 0, &p));
  if (node) last_ = node;
}

void Engine::arnoldi_step() {
  DevInst* st = (DevInst*)st_;
  const int* ci = (const int*)chunk_inst_;
  const int* nc = (const int*)nchunks_;
  const int* ti = (const int*)tile_inst_;
  const int* tl = (const int*)tile_local_;
  double* part = (double*)part1_;
  double2* partv = (double2*)partv_;
  double* none = nullptr;
  const int n = (int)jobs_.size();
  const dim3 gmd(total_chunks_, (m_ + 1 + 7) / 8);
  const dim3 gfin(n, (m_ + 1 + kRT / 32 - 1) / (kRT / 32));
  const dim3 gfirst(n, gfin.y + 1);  // projections into hA plus one row of image-norm blocks
  const int C = total_chunks_;
  if (f32_) {
    if (any_border_) launch(k_step_trace<float2>, n, kRT, 0, st);
    launch_step_apply(apply_schedule_);
    // CGS with selective reorthogonalisation: the first pass also takes the image norm
    // |w0|^2 (every job) and the first update the |w1|^2 partials (second half of part);
    // the second pass runs only for jobs whose first projection removed more than half of
    // |w0|^2 (k_step_mdot_f32)
    double* npart1 = part + C;
    const int* ncn = nullptr;
    const double* npn = nullptr;
    if (chunk_ == kBatchChunk)
      launch(k_step_mdot_f32<kBatchChunk>, C, kRT, 0, st, ci, partv, part, ncn, npn);
    else
      launch(k_step_mdot_f32<kBatchChunkSmall>, C, kRT, 0, st, ci, partv, part, ncn, npn);
    launch(k_step_first_final, gfirst, kRT, 0, st, nc, (const double2*)partv, (const double*)part, 1);
    launch(k_step_maxpy_f32, C, kRT, 0, (const DevInst*)st, ci, 0, npart1, npn);
    double* noi = nullptr;
    if (chunk_ == kBatchChunk)
      launch(k_step_mdot_f32<kBatchChunk>, C, kRT, 0, st, ci, partv, noi, nc, (const double*)npart1);
    else
      launch(k_step_mdot_f32<kBatchChunkSmall>, C, kRT, 0, st, ci, partv, noi, nc, (const double*)npart1);
    launch(k_step_mdot_final, gfin, kRT, 0, (const DevInst*)st, nc, (const double2*)partv, 1);
    launch(k_step_maxpy_f32, C, kRT, 0, (const DevInst*)st, ci, 1, part, (const double*)npart1);
    launch(k_step_normalize_f32, C, kRT, 0, st, ci, nc, (const double*)part);
  } else {
    if (any_border_) launch(k_step_trace<double2>, n, kRT, 0, st);
    launch(k_bapply<double, false>, total_tiles_, kApplyThreads, 3 * kWinElems * sizeof(double2), (const DevInst*)st, ti, tl);
    launch(k_step_image_partial<double2>, C, kRT, 0, (const DevInst*)st, ci, part);
    launch(k_step_mdot_partial<double2, false>, gmd, kRT, 0, (const DevInst*)st, ci, partv);
    launch(k_step_first_final, gfirst, kRT, 0, st, nc, (const double2*)partv, (const double*)part, 0);
    launch(k_step_maxpy<double2>, C, kRT, 0, (const DevInst*)st, ci, 0, none);
    launch(k_step_mdot_partial<double2, false>, gmd, kRT, 0, (const DevInst*)st, ci, partv);
    launch(k_step_mdot_final, gfin, kRT, 0, (const DevInst*)st, nc, (const double2*)partv, 1);
    launch(k_step_maxpy<double2>, C, kRT, 0, (const DevInst*)st, ci, 1, part);
    launch(k_step_normalize<double2>, C, kRT, 0, st, ci, nc, (const double*)part);
  }
  launch(k_step_finish, n, 32, 0, st, n);
  if (!build_) chk(cudaGetLastError());
}

void Engine::run_cycle_steps() {
  if (!schedule_chosen_) choose_apply_schedule();
  if (err != cudaSuccess) return;
  if (!graphs_) {
    for (int j = 0; j < m_; ++j) arnoldi_step();
    return;
  }
  if (!graph_) {
    chk(cudaGraphCreate(&build_, 0));
    last_ = nullptr;
    if (build_) {
      for (int j = 0; j < m_; ++j) arnoldi_step();
      if (err == cudaSuccess) chk(cudaGraphInstantiate(&graph_, build_, 0));
      cudaGraphDestroy(build_);
    }
    build_ = nullptr;
    last_ = nullptr;
    if (err != cudaSuccess) return;
  }
  chk(cudaGraphLaunch(graph_, s_));
}

bool Engine::tick() {
  if (err != cudaSuccess) return false;
  if (dirty_) rebuild();
  if (err != cudaSuccess) return false;
  const int n = (int)jobs_.size();
  if (n == 0) return true;
  ++ticks;
  DevInst* sth = (DevInst*)st_h_;
  double2* coefh = (double2*)coefs_h_;
  const double* outh = (const double*)out_h_;
  DevInst* st = (DevInst*)st_;
  const int* ci = (const int*)chunk_inst_;
  const int* ti = (const int*)tile_inst_;
  const int* tl = (const int*)tile_local_;
  const int C = total_chunks_;
  // ---- stage 1: vector work and one read
  unsigned flags = 0;
  for (int i = 0; i < n; ++i) {
    sth[i] = base_[i];
    if (!jobs_[i]->finished) flags |= jobs_[i]->stage1(sth[i], coefh + (size_t)i * (m_ + 2));
  }
  if (flags) {
    chk(cudaMemcpyAsync(st_, st_h_, sizeof(DevInst) * n, cudaMemcpyHostToDevice, s_));
    if (flags & S1_COMBINE) {
      chk(cudaMemcpyAsync(coefs_, coefs_h_, sizeof(double2) * (m_ + 2) * n, cudaMemcpyHostToDevice, s_));
      if (f32_)
        k_s1_combine_f32<<<C, kRT, 0, s_>>>(st, ci);
      else
        k_s1_combine<double2><<<C, kRT, 0, s_>>>(st, ci);
    }
    if (flags & S1_PROBE) k_s1_probe<<<C, kRT, 0, s_>>>(st, ci);
    if (flags & (S1_AUX | S1_TRACE)) k_s1_trace<<<n, kRT, 0, s_>>>(st);
    if (flags & S1_AUX)
      k_bapply<double, true><<<total_tiles_, kApplyThreads, 3 * kWinElems * sizeof(double2), s_>>>(st, ti, tl);
    if (flags & S1_RESID) k_s1_resid<<<C, kRT, 0, s_>>>(st, ci);
    if (flags & S1_NORM) {
      k_s1_norm_partial<<<C, kRT, 0, s_>>>(st, ci, (double*)part1_);
      k_s1_norm_final<<<n, kRT, 0, s_>>>(st, (const int*)nchunks_, (const double*)part1_);
    }
    if (flags & S1_OBS) {
      k_s1_obs_partial<<<C, kRT, 0, s_>>>(st, ci, (double2*)partv_);
      k_s1_obs_final<<<n, kRT, 0, s_>>>(st, (const int*)nchunks_, (const double2*)partv_);
    }
    chk(cudaGetLastError());
    chk(cudaMemcpyAsync(out_h_, out_, sizeof(double) * kOutSlots * n, cudaMemcpyDeviceToHost, s_));
    chk(cudaStreamSynchronize(s_));
    if (err != cudaSuccess) return false;
    for (int i = 0; i < n; ++i)
      if (!jobs_[i]->finished) jobs_[i]->after_stage1(outh + (size_t)i * kOutSlots);
  }
  // ---- stage 3: one Arnoldi cycle for the jobs that need a factorization
  std::vector<char> in_cycle(n, 0);
  bool any = false;
  for (int i = 0; i < n; ++i) {
    sth[i] = base_[i];
    if (!jobs_[i]->finished && jobs_[i]->cycle(sth[i])) {
      in_cycle[i] = 1;
      any = true;
    }
  }
  if (!any) return err == cudaSuccess;
  ++cycles;
  chk(cudaMemcpyAsync(st_, st_h_, sizeof(DevInst) * n, cudaMemcpyHostToDevice, s_));
  if (f32_)
    k_load_v0<float2><<<C, kRT, 0, s_>>>(st, ci);
  else
    k_load_v0<double2><<<C, kRT, 0, s_>>>(st, ci);
  chk(cudaGetLastError());
  run_cycle_steps();
  steps += m_;
  const DevInst* dl = (const DevInst*)st_dl_;
  const double2* rech = (const double2*)rec_h_;
  chk(cudaMemcpyAsync(st_dl_, st_, sizeof(DevInst) * n, cudaMemcpyDeviceToHost, s_));
  chk(cudaMemcpyAsync(rec_h_, rec_, sizeof(double2) * rec_stride_ * n, cudaMemcpyDeviceToHost, s_));
  chk(cudaStreamSynchronize(s_));
  if (err != cudaSuccess) return false;
  bool enl = false;
  std::vector<char> in_enl(n, 0);
  for (int i = 0; i < n; ++i) {
    sth[i] = base_[i];
    if (in_cycle[i] && jobs_[i]->after_cycle(dl[i], rech + (size_t)i * rec_stride_, sth[i])) {
      in_enl[i] = 1;
      enl = true;
    }
  }
  if (!enl) return err == cudaSuccess;
  // near-breakdown enlargement: one more step for the jobs that asked
  chk(cudaMemcpyAsync(st_, st_h_, sizeof(DevInst) * n, cudaMemcpyHostToDevice, s_));
  arnoldi_step();
  ++steps;
  chk(cudaMemcpyAsync(st_dl_, st_, sizeof(DevInst) * n, cudaMemcpyDeviceToHost, s_));
  chk(cudaMemcpyAsync(rec_h_, rec_, sizeof(double2) * rec_stride_ * n, cudaMemcpyDeviceToHost, s_));
  chk(cudaStreamSynchronize(s_));
  if (err != cudaSuccess) return false;
  for (int i = 0; i < n; ++i)
    if (in_enl[i]) jobs_[i]->after_enlarge(dl[i], rech + (size_t)i * rec_stride_);
  return err == cudaSuccess;
}

int run_single_job(pi_plan* plan, Job* job, int m, bool f32, const char* what) {
  if (plan->engine && (plan->engine_m != m || plan->engine_f32 != f32 || plan->engine->err != cudaSuccess)) {
    delete plan->engine;
    plan->engine = nullptr;
  }
  if (!plan->engine) {
    plan->engine = new Engine(plan->device, m, f32, true);
    plan->engine_m = m;
    plan->engine_f32 = f32;
    if (plan->engine->err != cudaSuccess) {
      const cudaError_t e = plan->engine->err;
      delete plan->engine;
      plan->engine = nullptr;
      return cuda_fail(e, what);
    }
  }
  Engine& E = *plan->engine;
  if (!job->setup(E.stream(), E.m(), E.f32())) return cuda_fail(cudaErrorMemoryAllocation, what);
  E.add(job);
  while (E.njobs() > 0) {
    if (!E.tick()) {
      const cudaError_t e = E.err;
      E.retire();
      delete plan->engine;
      plan->engine = nullptr;
      return cuda_fail(e, what);
    }
    for (Job* j : E.retire()) j->finish(E.stream());
  }
  const cudaError_t e = cudaStreamSynchronize(E.stream());
  if (e != cudaSuccess) return cuda_fail(e, what);
  return PI_OK;
}

void release_plan_engine(pi_plan* plan) {
  delete plan->engine;
  plan->engine = nullptr;
}

namespace {

int check_expv_opts(const pi_expv_opts_t* o) {
  if (!o) return fail(PI_ERR_INVALID_ARGUMENT, "null options");
  if (o->krylovdim < 1 || o->krylovdim > kBatchMaxKrylov)
    return fail(PI_ERR_INVALID_ARGUMENT, "krylovdim must lie in 1:120 for batched solves");
  if (!(o->atol >= 0) || !(o->rtol >= 0) || !std::isfinite(o->atol) || !std::isfinite(o->rtol))
    return fail(PI_ERR_INVALID_ARGUMENT, "atol and rtol must be finite nonnegative real numbers");
  if (!(o->safety > 0 && o->safety < 1))
    return fail(PI_ERR_INVALID_ARGUMENT, "safety must lie strictly between zero and one");
  if (o->max_steps < 1) return fail(PI_ERR_INVALID_ARGUMENT, "max_steps must be positive");
  if (o->precision != PI_FP64 && o->precision != PI_FP32)
    return fail(PI_ERR_INVALID_ARGUMENT, "precision must be PI_FP64 or PI_FP32");
  return PI_OK;
}

int check_gmres_opts(const pi_gmres_opts_t* o) {
  if (!o) return fail(PI_ERR_INVALID_ARGUMENT, "null options");
  if (o->krylovdim < 1 || o->krylovdim > kBatchMaxKrylov)
    return fail(PI_ERR_INVALID_ARGUMENT, "krylovdim must lie in 1:120 for batched solves");
  if (o->maxiter < 1) return fail(PI_ERR_INVALID_ARGUMENT, "maxiter must be positive");
  if (!(o->atol >= 0) || !(o->rtol >= 0)) return fail(PI_ERR_INVALID_ARGUMENT, "tolerances must be nonnegative");
  if (o->precision != PI_FP64 && o->precision != PI_FP32)
    return fail(PI_ERR_INVALID_ARGUMENT, "precision must be PI_FP64 or PI_FP32");
  if (o->preconditioner != nullptr || o->drive_preconditioner != nullptr || o->coords != PI_COORDS_REFERENCE)
    return fail(PI_ERR_UNSUPPORTED,
                "batched steady states run unpreconditioned in reference coordinates; solve preconditioned or "
                "population-coordinate steady states with pi_steady_state");
  return PI_OK;
}

int check_plans(int n, pi_plan* const* plans, double* const* states, int* device) {
  if (n < 1 || !plans || !states) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  std::unordered_set<const void*> seen;
  for (int i = 0; i < n; ++i) {
    if (!plans[i] || !states[i]) return fail(PI_ERR_INVALID_ARGUMENT, "null plan or state in the batch");
    if (plans[i]->device != plans[0]->device)
      return fail(PI_ERR_INVALID_ARGUMENT, "all plans of a batch must live on one device");
    if (!seen.insert(states[i]).second)
      return fail(PI_ERR_INVALID_ARGUMENT, "two batch instances share one state buffer");
  }
  *device = plans[0]->device;
  return PI_OK;
}

// Runs the engine until every job finished; returns the first job error (or a CUDA error).
int run_jobs(Engine& E, std::vector<Job*>& jobs, const char* what) {
  for (Job* j : jobs) {
    if (!j->setup(E.stream(), E.m(), E.f32())) return cuda_fail(cudaErrorMemoryAllocation, what);
    E.add(j);
  }
  while (E.njobs() > 0) {
    if (!E.tick()) return cuda_fail(E.err, what);
    for (Job* j : E.retire()) j->finish(E.stream());
  }
  const cudaError_t e = cudaStreamSynchronize(E.stream());
  if (e != cudaSuccess) return cuda_fail(e, what);
  for (size_t i = 0; i < jobs.size(); ++i)
    if (jobs[i]->rc != PI_OK) {
      char m[64];
      std::snprintf(m, sizeof(m), "batch instance %zu: ", i);
      return fail(jobs[i]->rc, std::string(m) + jobs[i]->msg);
    }
  return PI_OK;
}

}  // namespace
}  // namespace picuda

using namespace picuda;

extern "C" {

int pi_expv_batch(int ninst, pi_plan* const* plans, double* const* x_devs, const double* t,
                  const pi_expv_opts_t* opts, pi_expv_info_t* infos) {
  int device = 0;
  int rc = check_plans(ninst, plans, x_devs, &device);
  if (rc) return rc;
  rc = check_expv_opts(opts);
  if (rc) return rc;
  if (!t) return fail(PI_ERR_INVALID_ARGUMENT, "null times");
  for (int i = 0; i < ninst; ++i)
    if (!std::isfinite(t[i])) return fail(PI_ERR_INVALID_ARGUMENT, "time must be finite");
  std::vector<DynamicsJob*> jobs;
  std::vector<Job*> base;
  for (int i = 0; i < ninst; ++i) {
    jobs.push_back(new DynamicsJob(plans[i], x_devs[i], {0.0, t[i]}, 0, nullptr, nullptr, *opts, true));
    base.push_back(jobs.back());
  }
  {
    Engine E(plans[0]->device, opts->krylovdim, opts->precision == PI_FP32, true);
    if (E.err != cudaSuccess) rc = cuda_fail(E.err, "batched expv engine");
    if (!rc) rc = run_jobs(E, base, "batched expv");
    if (infos)
      for (int i = 0; i < ninst; ++i) infos[i] = jobs[i]->info();
    for (Job* j : base) delete j;
  }
  (void)device;
  return rc;
}

int pi_dynamics_batch(int njobs, const pi_dynamics_job_t* specs, const pi_expv_opts_t* opts, pi_expv_info_t* infos) {
  if (njobs < 1 || !specs) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<pi_plan*> plans(njobs);
  std::vector<double*> states(njobs);
  for (int i = 0; i < njobs; ++i) {
    plans[i] = specs[i].plan;
    states[i] = specs[i].state_dev;
  }
  int device = 0;
  int rc = check_plans(njobs, plans.data(), states.data(), &device);
  if (rc) return rc;
  rc = check_expv_opts(opts);
  if (rc) return rc;
  for (int i = 0; i < njobs; ++i) {
    const pi_dynamics_job_t& s = specs[i];
    if (s.nt < 1 || !s.times) return fail(PI_ERR_INVALID_ARGUMENT, "every job needs at least one saved time");
    if (s.nobs < 0 || s.nobs > kBatchMaxObs || (s.nobs > 0 && (!s.obs_dev || !s.values_host)))
      return fail(PI_ERR_INVALID_ARGUMENT, "observables must number 0..16 with device data and a host output");
    for (int k = 0; k < s.nt; ++k) {
      if (!std::isfinite(s.times[k])) return fail(PI_ERR_INVALID_ARGUMENT, "saved times must be finite");
      if (k > 0 && !(s.times[k] >= s.times[k - 1]))
        return fail(PI_ERR_INVALID_ARGUMENT, "Krylov exponential output times must be nondecreasing");
    }
  }
  std::vector<DynamicsJob*> jobs;
  std::vector<Job*> base;
  for (int i = 0; i < njobs; ++i) {
    const pi_dynamics_job_t& s = specs[i];
    jobs.push_back(new DynamicsJob(s.plan, s.state_dev, std::vector<double>(s.times, s.times + s.nt), s.nobs,
                                   s.obs_dev, s.values_host, *opts, false));
    base.push_back(jobs.back());
  }
  {
    Engine E(device, opts->krylovdim, opts->precision == PI_FP32, true);
    if (E.err != cudaSuccess) rc = cuda_fail(E.err, "batched dynamics engine");
    if (!rc) rc = run_jobs(E, base, "batched dynamics");
    if (infos)
      for (int i = 0; i < njobs; ++i) infos[i] = jobs[i]->info();
    for (Job* j : base) delete j;
  }
  return rc;
}

int pi_engine_set_apply_schedule(int schedule) {
  if (schedule < PI_SCHEDULE_PER_TILE || schedule > 64)
    return fail(PI_ERR_INVALID_ARGUMENT, "schedule must be PI_SCHEDULE_AUTO, PI_SCHEDULE_PER_TILE or 1..64 blocks per SM");
  g_apply_schedule.store(schedule);
  return PI_OK;
}

int pi_engine_schedule_info(pi_schedule_info_t* out) {
  if (!out) return fail(PI_ERR_INVALID_ARGUMENT, "null output");
  std::lock_guard<std::mutex> lk(g_schedule_mu);
  *out = g_schedule_info;
  return PI_OK;
}

int pi_steady_state_batch(int ninst, pi_plan* const* plans, double* const* x_devs, const pi_gmres_opts_t* opts,
                          pi_gmres_info_t* infos) {
  int device = 0;
  int rc = check_plans(ninst, plans, x_devs, &device);
  if (rc) return rc;
  rc = check_gmres_opts(opts);
  if (rc) return rc;
  std::vector<SteadyJob*> jobs;
  std::vector<Job*> base;
  for (int i = 0; i < ninst; ++i) {
    jobs.push_back(new SteadyJob(plans[i], x_devs[i], *opts, 0x51ca1eULL));
    base.push_back(jobs.back());
  }
  {
    Engine E(device, opts->krylovdim, opts->precision == PI_FP32, true);
    if (E.err != cudaSuccess) rc = cuda_fail(E.err, "batched steady-state engine");
    if (!rc) rc = run_jobs(E, base, "batched steady state");
    if (infos)
      for (int i = 0; i < ninst; ++i) infos[i] = jobs[i]->info();
    for (Job* j : base) delete j;
  }
  return rc;
}

}  // extern "C"
