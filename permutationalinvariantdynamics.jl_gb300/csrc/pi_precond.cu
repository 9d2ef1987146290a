// Level-sweep preconditioner for the trace-fixed steady-state GMRES.
//
// The reference preconditions krylov_steady_state with the LU factors of the diagonal Schur
// blocks of L/s + v t^H (schur_sector_preconditioner, krylov.jl:183-700, applied on the left
// in _gmres!, krylov.jl:732-787).  That is one dense n^2 x n^2 factorisation per sector:
// O(n^6) work and a 40k x 40k matrix per sector at N = 200.  This file keeps the reference's
// left-preconditioned GMRES and replaces the factors by the exact inverse of a different
// part of L, one that a GPU can invert in O(dim) work.
//
// Write an entry of sector s as (a, b) with a = j - M and b = j - M' (GT order).  Every term
// of a qubit Liouvillian reads x_src[a + e + p, b + e + q].  The terms with p == q keep the
// charge d = b - a = M - M' (they commute with the U(1) rotation generated by Jz): the
// dissipators of Jz-covariant jump operators (sigma-, sigma+, sigma_z, J-, ...), the
// diagonal of the Hamiltonian, and the loss anticommutators.  The terms with p != q -- the
// drive, Jx and Jy -- change d by one.  L0, the charge-keeping part, is block diagonal in
// d.  Inside one charge block, with the level index lambda = 2M = n_s - 1 - 2a:
//   - p = q = 0 terms couple an entry to the same (M, M') in the sectors s-1, s, s+1:
//     a tridiagonal system over the sectors present at that level;
//   - p = q = -1 terms (decay-type gains) read the level lambda + 2, and p = q = +1 terms
//     (pump-type gains) read lambda - 2.
// When the gains all point one way, the block is block lower-triangular in lambda with
// tridiagonal diagonal blocks, so L0 z = r is solved exactly by sweeping the levels in that
// order with one Thomas solve per level.  The Thomas factors are computed once here.
//
// The bordered operator M = L0/s + v t^H is then inverted exactly, in one of two ways:
//   - L0 singular, its null vector on one "free" entry: the zero pivot of the last level of
//     the d = 0 chain (the all-down population for decay models).  Write z = y + c e_f with
//     beta = t^H z; then L0 y = s (r - beta v).  The sweep of s r with the free equation
//     dropped gives y_r and that equation's residual rho_r; the same for s v, precomputed,
//     gives y_v and rho_v.  The free equation fixes beta = rho_r / rho_v, so
//     y = y_r - beta y_v, and c = (beta - t^H y) / t_f.  (For a trace-preserving L0 this is
//     beta = t^H r.)
//   - L0 nonsingular (or regularised): Sherman-Morrison with the precomputed w0 = s L0^-1 v.
// v and t live on the block diagonals, which are exactly the d = 0 chain, and sweeps keep the
// charge, so y_v, w0 and both corrections stay inside the thread block that sweeps that
// chain.
//
// Device layout: one thread block per charge chain (2 n_max - 1 chains, the longest first),
// four warps each.  A ring of four shared-memory level slots keeps the sweep fed: warps 1-3
// copy the factors of level l+3 and gather r at the elements of level l+2 with cp.async
// (each thread gathers the entries whose indices it copied), while warp 0 solves level l.
// Warp 0 subtracts the gains from the previous level's solution and runs both Thomas
// recurrences as warp-wide scans of affine maps (each lane composes a chunk of at most five
// entries, five shuffle steps combine the lanes), so a level costs a few dozen dependent
// steps however many sectors it spans.  Population coordinates run in FP32 (the
// preconditioner is an approximation of L^-1 either way, and every entry is a bounded
// population); reference coordinates run in FP64, since their entries span many decades at
// large N.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/picuda.h"
#include "pi_handle.hpp"
#include "pi_internal.hpp"
#include "pi_precond.hpp"
#include "pi_drive.hpp"

namespace picuda {

namespace {

constexpr int kSweepThreads = 128;
constexpr int kNoGain = 1023;

template <typename T>
struct V2;
template <>
struct V2<double> {
  using type = double2;
  static __host__ __device__ double2 make(double x, double y) { return make_double2(x, y); }
};
template <>
struct V2<float> {
  using type = float2;
  static __host__ __device__ float2 make(float x, float y) { return make_float2(x, y); }
};

template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// c + a * b
template <typename T2>
__device__ __forceinline__ T2 cfma(T2 a, T2 b, T2 c) {
  T2 r;
  r.x = fma(a.x, b.x, fma(-a.y, b.y, c.x));
  r.y = fma(a.x, b.y, fma(a.y, b.x, c.y));
  return r;
}
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

template <typename TI>
__device__ __forceinline__ double2 load_d2(const TI* p) {
  const TI v = *p;
  return make_double2((double)v.x, (double)v.y);
}

template <typename TO, typename T2>
__device__ __forceinline__ void store_as(TO* p, T2 v);
template <>
__device__ __forceinline__ void store_as<double2, double2>(double2* p, double2 v) { *p = v; }
template <>
__device__ __forceinline__ void store_as<double2, float2>(double2* p, float2 v) {
  *p = make_double2((double)v.x, (double)v.y);
}
template <>
__device__ __forceinline__ void store_as<float2, float2>(float2* p, float2 v) { *p = v; }
template <>
__device__ __forceinline__ void store_as<float2, double2>(float2* p, double2 v) {
  *p = make_float2((float)v.x, (float)v.y);
}

// Block-wide sum of two doubles per thread (fixed order).
__device__ __forceinline__ double2 block_sum2(double2 v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, off);
    v.y += __shfl_down_sync(0xffffffffu, v.y, off);
  }
  __syncthreads();
  if (lane == 0) {
    red[2 * warp] = v.x;
    red[2 * warp + 1] = v.y;
  }
  __syncthreads();
  double2 out = make_double2(0.0, 0.0);
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    out.x += red[2 * w];
    out.y += red[2 * w + 1];
  }
  __syncthreads();
  return out;
}

constexpr int kStagers = kSweepThreads - 32;  // warps 1.. stage levels ahead of warp 0
static_assert(kPrecondMaxLevel <= 5 * 32, "warp 0 solves levels of at most five entries per lane");
// Depth of the level ring: the factors of level k + DF and the gather of r at level k + DG are
// issued while level k is solved, so copies have DF - DG and gathers DG - 1 levels of time to
// land.  FP32 sweeps keep six slots (about 70 KB of shared memory, three blocks per SM);
// FP64 sweeps keep four to stay at two blocks per SM.
template <typename T>
struct Ring;
template <>
struct Ring<float> {
  static constexpr int DF = 5, DG = 3;
};
template <>
struct Ring<double> {
  static constexpr int DF = 3, DG = 2;
};
constexpr int kMaxChainLevels = 2 * kPrecondMaxLevel + 4;

__device__ __forceinline__ float2 shfl_up_c(float2 v, int d) {
  return make_float2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}
__device__ __forceinline__ double2 shfl_up_c(double2 v, int d) {
  return make_double2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}
__device__ __forceinline__ float2 shfl_down_c(float2 v, int d) {
  return make_float2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}
__device__ __forceinline__ double2 shfl_down_c(double2 v, int d) {
  return make_double2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}

__device__ __forceinline__ void cpa(void* smem, const void* gmem, int bytes) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
  if (bytes == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(gmem) : "memory");
  else if (bytes == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(a), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// One staged level: r at the level's elements (as stored) and the level's factors and gain
// tables.
// Slot position of entry i of a level with K = ceil(cnt / 32) entries per lane: lane l's q-th
// entry (i = l K + q) sits at q * 32 + l, so warp 0's accesses of one q are bank-conflict free.
__device__ __forceinline__ int slot_pos(int i, int K) { return (i % K) * 32 + i / K; }

template <typename T, typename TI>
struct Slot {
  using T2 = typename V2<T>::type;
  TI rv[kPrecondMaxLevel];    // r at the level's elements
  T2 w[kPrecondMaxLevel];     // 1 / pivot
  T2 a[kPrecondMaxLevel];     // forward multiplier
  T2 c[kPrecondMaxLevel];     // backward multiplier
  T2 g[3][kPrecondMaxLevel];  // gain coefficients
  int gp[kPrecondMaxLevel];   // packed gain positions in the previous level
  int el[kPrecondMaxLevel];   // element index
};

template <typename T, typename TI>
struct SweepSmem {
  using T2 = typename V2<T>::type;
  static constexpr int kSlots = Ring<T>::DF + 1;
  Slot<T, TI> slot[kSlots];
  T2 u[2][kPrecondMaxLevel];     // solution of the previous / current level
  T2 b[kPrecondMaxLevel];        // W_i (s r_i - gains), slot order
  int lev_ent[kMaxChainLevels];  // the chain's level bounds
  double red[2 * (kSweepThreads / 32)];
};

// Stager thread t copies the factors of entries t, t + kStagers, ... of chain level k into
// its slot with cp.async (one commit group per call, empty past the chain's end).
template <typename T, typename TI>
__device__ __forceinline__ void issue_factors(const PrecondDev& P, SweepSmem<T, TI>& S, int k, int nlev, int t) {
  using T2 = typename V2<T>::type;
  if (k >= 0 && k < nlev) {
    Slot<T, TI>& L = S.slot[k % SweepSmem<T, TI>::kSlots];
    const T2* W = reinterpret_cast<const T2*>(P.W);
    const T2* A = reinterpret_cast<const T2*>(P.A);
    const T2* C = reinterpret_cast<const T2*>(P.C);
    const T2* G = reinterpret_cast<const T2*>(P.G);
    const int e0 = S.lev_ent[k], cnt = S.lev_ent[k + 1] - e0;
    const int K = (cnt + 31) >> 5;
    for (int i = t; i < cnt; i += kStagers) {
      const int e = e0 + i;
      const int p = slot_pos(i, K);
      cpa(&L.el[p], P.elem + e, 4);
      cpa(&L.gp[p], P.gsrc + e, 4);
      cpa(&L.w[p], W + e, sizeof(T2));
      cpa(&L.a[p], A + e, sizeof(T2));
      cpa(&L.c[p], C + e, sizeof(T2));
#pragma unroll
      for (int q = 0; q < 3; ++q) cpa(&L.g[q][p], G + 3LL * e + q, sizeof(T2));
    }
  }
  cpa_commit();
}

// The same stager thread gathers r at the elements whose indices it copied, with cp.async.
template <typename T, typename TI>
__device__ __forceinline__ void issue_gather(const TI* __restrict__ r, SweepSmem<T, TI>& S, int k, int nlev, int t) {
  if (k >= 0 && k < nlev) {
    Slot<T, TI>& L = S.slot[k % SweepSmem<T, TI>::kSlots];
    const int cnt = S.lev_ent[k + 1] - S.lev_ent[k];
    const int K = (cnt + 31) >> 5;
    for (int i = t; i < cnt; i += kStagers) {
      const int p = slot_pos(i, K);
      cpa(&L.rv[p], r + L.el[p], sizeof(TI));
    }
  }
  cpa_commit();
}

// Right-hand sides of one level, all warps: b_i = W_i (s r_i - sum of the gains from the
// previous level's solution), at slot positions.  Absent gains read slot 0 with a zero
// coefficient; the thread that meets the free entry keeps its unscaled residual.
template <typename T, typename TI>
__device__ __forceinline__ void level_rhs(const PrecondDev& Pd, const Slot<T, TI>& L,
                                          const typename V2<T>::type* __restrict__ uprev,
                                          typename V2<T>::type* __restrict__ b, int e0, int cnt, T sT, int tid,
                                          double2& rho_r, bool& has_rho) {
  using T2 = typename V2<T>::type;
  const int K = (cnt + 31) >> 5;
  for (int p = tid; p < 32 * K; p += kSweepThreads) {
    const int i = (p & 31) * K + (p >> 5);  // entry of slot p
    if (i >= cnt) continue;
    const TI x = L.rv[p];
    T2 rv = V2<T>::make(sT * (T)x.x, sT * (T)x.y);
    const int packed = L.gp[p];
#pragma unroll
    for (int g3 = 0; g3 < 3; ++g3) {
      int pos = (packed >> (10 * g3)) & 1023;  // slot position in the previous level
      pos = pos == kNoGain ? 0 : pos;          // an absent gain has a zero coefficient
      const T2 g = L.g[g3][p];
      T2 m;
      m.x = -g.x;
      m.y = -g.y;
      rv = cfma(m, uprev[pos], rv);
    }
    const bool hit = e0 + i == Pd.free_ent;
    rho_r.x = hit ? (double)rv.x : rho_r.x;
    rho_r.y = hit ? (double)rv.y : rho_r.y;
    has_rho = has_rho || hit;
    b[p] = cmul(L.w[p], rv);
  }
}

// Warp 0's solve of one level of cnt entries, K = ceil(cnt / 32) of them per lane.  Lane l
// owns the K consecutive entries l K .. l K + K - 1 (slots q 32 + l).  Both Thomas
// recurrences, y_i = A_i y_{i-1} + b_i and u_i = C_i u_{i+1} + y_i, are affine maps composed
// over each lane's chunk, combined across lanes by a five-step shuffle scan, then replayed
// inside the chunk.  Specialised on K so that short levels issue short code.
template <typename T, typename TI, typename TO, int K>
__device__ __forceinline__ void solve_level(const PrecondDev& Pd, const Slot<T, TI>& L,
                                            const typename V2<T>::type* __restrict__ b,
                                            typename V2<T>::type* __restrict__ ucur, TO* __restrict__ z, int e0,
                                            int cnt, bool sum_t, int lane, double2& tsum) {
  using T2 = typename V2<T>::type;
  const int i0 = lane * K;
  T2 Bv[K], Av[K], Cv[K];
  bool ok[K];
  const T2 one = V2<T>::make((T)1, (T)0), zero = V2<T>::make((T)0, (T)0);
#pragma unroll
  for (int q = 0; q < K; ++q) {
    ok[q] = i0 + q < cnt;
    const int p = q * 32 + lane;
    const T2 bb = b[p], a = L.a[p], c = L.c[p];
    Bv[q] = ok[q] ? bb : zero;
    Av[q] = ok[q] ? a : zero;
    Cv[q] = ok[q] ? c : zero;
  }
  // the lane's forward map y_out = P y_in + Q
  T2 P = one, Q = zero;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    const T2 Pq = cmul(Av[q], P), Qq = cfma(Av[q], Q, Bv[q]);
    P = ok[q] ? Pq : P;
    Q = ok[q] ? Qq : Q;
  }
  // inclusive scan in lane order: (P, Q) <- (P, Q) o (P_prev, Q_prev)
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T2 Pn = shfl_up_c(P, d), Qn = shfl_up_c(Q, d);
    if (lane >= d) {
      Q = cfma(P, Qn, Q);
      P = cmul(P, Pn);
    }
  }
  T2 y = shfl_up_c(Q, 1);
  if (lane == 0) y = zero;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    y = cfma(Av[q], y, Bv[q]);  // Av = Bv = 0 past the level: harmless zeros
    Bv[q] = y;                  // Bv now holds y_i
  }
  // the lane's backward map u_in = P2 u_next + Q2 over its entries of the level
  T2 P2 = one, Q2 = zero;
#pragma unroll
  for (int q = K - 1; q >= 0; --q) {
    const T2 Pq = cmul(Cv[q], P2), Qq = cfma(Cv[q], Q2, Bv[q]);
    P2 = ok[q] ? Pq : P2;
    Q2 = ok[q] ? Qq : Q2;
  }
  // suffix scan in reverse lane order
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T2 Pn = shfl_down_c(P2, d), Qn = shfl_down_c(Q2, d);
    if (lane + d < 32) {
      Q2 = cfma(P2, Qn, Q2);
      P2 = cmul(P2, Pn);
    }
  }
  T2 uv = shfl_down_c(Q2, 1);
  if (lane == 31) uv = zero;
  T2 U[K];
#pragma unroll
  for (int q = K - 1; q >= 0; --q) {
    uv = cfma(Cv[q], uv, Bv[q]);
    U[q] = uv;
  }
#pragma unroll
  for (int q = 0; q < K; ++q) {
    if (ok[q]) {
      ucur[q * 32 + lane] = U[q];
      store_as<TO, T2>(z + L.el[q * 32 + lane], U[q]);
    }
  }
  if (sum_t) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      if (ok[q]) {
        const double t = Pd.t0[e0 + i0 + q - Pd.chain0_ent];
        tsum.x = fma(t, (double)U[q].x, tsum.x);
        tsum.y = fma(t, (double)U[q].y, tsum.y);
      }
    }
  }
}

template <typename T, typename TI, typename TO>
__global__ void __launch_bounds__(kSweepThreads)
    k_level_sweep(const PrecondDev Pd, const TI* __restrict__ r, TO* __restrict__ z, double s) {
  using T2 = typename V2<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SweepSmem<T, TI>& S = *reinterpret_cast<SweepSmem<T, TI>*>(smem_raw);
  const int chain = Pd.chain_order[blockIdx.x];
  const int lev0 = Pd.chain_lev[chain], lev1 = Pd.chain_lev[chain + 1];
  const int nlev = lev1 - lev0;
  const bool chain0 = chain == Pd.chain0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int st = tid - 32;  // stager index
  for (int k = tid; k <= nlev; k += blockDim.x) S.lev_ent[k] = Pd.lev_ent[lev0 + k];
  for (int i = tid; i < 2 * kPrecondMaxLevel; i += blockDim.x)  // absent gains read finite zeros
    S.u[i / kPrecondMaxLevel][i % kPrecondMaxLevel] = V2<T>::make((T)0, (T)0);
  __syncthreads();
  // Level j's step issues the factors of j + DF, waits until this thread's factors of j + DG
  // and gather of j + 1 have landed (after the gather of j + 1 it has committed 2 DG - 3
  // groups, after the factors of j + DG 2 (DF - DG)), and issues the gather of j + DG; steps
  // j < 0 fill the ring before warp 0 starts (empty groups keep the commit counts uniform).
  constexpr int DF = Ring<T>::DF, DG = Ring<T>::DG;
  double2 tsum = make_double2(0.0, 0.0);
  double2 rho_r = make_double2(0.0, 0.0);  // residual of the dropped free equation (lane-held)
  bool has_rho = false;
  int prev = 0, cur = 1;
  const T sT = (T)s;
  for (int k = -DF; k < nlev; ++k) {
    const Slot<T, TI>& L = S.slot[(k + SweepSmem<T, TI>::kSlots) % SweepSmem<T, TI>::kSlots];
    const int e0 = k >= 0 ? S.lev_ent[k] : 0;
    const int cnt = k >= 0 ? S.lev_ent[k + 1] - e0 : 0;
    if (k >= 0) {
      level_rhs<T, TI>(Pd, L, S.u[prev], S.b, e0, cnt, sT, tid, rho_r, has_rho);
      __syncthreads();
    }
    if (warp > 0) {
      issue_factors<T, TI>(Pd, S, k + DF, nlev, st);
      cpa_wait<(2 * DG - 3 < 2 * (DF - DG) ? 2 * DG - 3 : 2 * (DF - DG))>();
      issue_gather<T, TI>(r, S, k + DG, nlev, st);
    } else if (k >= 0) {
      const bool sum_t = chain0 && Pd.mode == 1;
      switch ((cnt + 31) >> 5) {
        case 1: solve_level<T, TI, TO, 1>(Pd, L, S.b, S.u[cur], z, e0, cnt, sum_t, lane, tsum); break;
        case 2: solve_level<T, TI, TO, 2>(Pd, L, S.b, S.u[cur], z, e0, cnt, sum_t, lane, tsum); break;
        case 3: solve_level<T, TI, TO, 3>(Pd, L, S.b, S.u[cur], z, e0, cnt, sum_t, lane, tsum); break;
        case 4: solve_level<T, TI, TO, 4>(Pd, L, S.b, S.u[cur], z, e0, cnt, sum_t, lane, tsum); break;
        default: solve_level<T, TI, TO, 5>(Pd, L, S.b, S.u[cur], z, e0, cnt, sum_t, lane, tsum); break;
      }
    }
    __syncthreads();
    if (k >= 0) {
      prev ^= 1;
      cur ^= 1;
    }
  }
  if (!chain0) return;
  const int c0 = Pd.chain0_ent, c1 = Pd.lev_ent[lev1];
  if (Pd.mode == 0) {
    // beta = rho_r / rho_v; y = y_r - beta y_v; z_f = (beta - t^H y) / t_f
    double* rr = S.red;  // the lane that met the free entry hands rho_r over
    __syncthreads();
    if (has_rho) {
      rr[0] = rho_r.x;
      rr[1] = rho_r.y;
    }
    __syncthreads();
    const double2 rrv = make_double2(rr[0], rr[1]);
    __syncthreads();
    const double2 rv = Pd.sm_coef;  // rho_v
    const double den = rv.x * rv.x + rv.y * rv.y;
    const double2 beta =
        make_double2((rrv.x * rv.x + rrv.y * rv.y) / den, (rrv.y * rv.x - rrv.x * rv.y) / den);
    for (int e = c0 + tid; e < c1; e += blockDim.x) {
      const int el = Pd.elem[e];
      const double2 yv = Pd.w0[e - c0];
      double2 zv = load_d2(z + el);
      zv.x -= beta.x * yv.x - beta.y * yv.y;
      zv.y -= beta.x * yv.y + beta.y * yv.x;
      store_as<TO, double2>(z + el, zv);
      const double t = Pd.t0[e - c0];
      tsum.x = fma(t, zv.x, tsum.x);
      tsum.y = fma(t, zv.y, tsum.y);
    }
    const double2 tz = block_sum2(tsum, S.red);
    if (tid == 0 && Pd.free_ent >= 0) {
      const double t = Pd.t0[Pd.free_ent - c0];
      store_as<TO, double2>(z + Pd.elem[Pd.free_ent], make_double2((beta.x - tz.x) / t, (beta.y - tz.y) / t));
    }
  } else {
    // Sherman-Morrison: z -= w0 (t^H y) / (1 + t^H w0)
    const double2 tz = block_sum2(tsum, S.red);
    const double2 kk =
        make_double2(tz.x * Pd.sm_coef.x - tz.y * Pd.sm_coef.y, tz.x * Pd.sm_coef.y + tz.y * Pd.sm_coef.x);
    for (int e = c0 + tid; e < c1; e += blockDim.x) {
      const int el = Pd.elem[e];
      const double2 w0 = Pd.w0[e - c0];
      double2 zv = load_d2(z + el);
      zv.x -= w0.x * kk.x - w0.y * kk.y;
      zv.y -= w0.x * kk.y + w0.y * kk.x;
      store_as<TO, double2>(z + el, zv);
    }
  }
}

template <typename T, typename TI, typename TO>
cudaError_t launch_sweep(const PrecondDev& D, int blocks, const void* r, void* z, double scale, cudaStream_t stream) {
  const size_t smem = sizeof(SweepSmem<T, TI>);
  // the shared-memory opt-in is a per-function, per-device attribute: set once per device
  static std::atomic<unsigned long long> configured{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ULL << (dev & 63);
  if (!(configured.load() & bit)) {
    e = cudaFuncSetAttribute(k_level_sweep<T, TI, TO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured.fetch_or(bit);
  }
  k_level_sweep<T, TI, TO><<<blocks, kSweepThreads, smem, stream>>>(D, (const TI*)r, (TO*)z, scale);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Host construction
// ---------------------------------------------------------------------------------------

using cdv = std::complex<double>;

cdv term_coef(const StencilTerm& t, int a, int b) {
  switch (t.kind) {
    case ST_ADD: return t.alpha[a] + t.beta[b];
    case ST_LEFT: return t.alpha[a];
    case ST_RIGHT: return t.beta[b];
    default: return t.alpha[a] * t.beta[b];
  }
}

}  // namespace

int build_level_precond(const QubitPlan& hp, int coords, double regularization, double scale, LevelPrecondHost* out,
                        std::string* err) {
  LevelPrecondHost& H = *out;
  H = LevelPrecondHost{};
  const int S = (int)hp.sectors.size();
  if (S < 1) {
    *err = "empty basis";
    return PI_ERR_INVALID_ARGUMENT;
  }
  if (S > kPrecondMaxLevel) {
    *err = "the level-sweep preconditioner supports at most 160 sectors (N <= 318)";
    return PI_ERR_UNSUPPORTED;
  }
  if (hp.dim > 0x7fffffffLL) {
    *err = "basis too large for 32-bit element indices";
    return PI_ERR_UNSUPPORTED;
  }
  H.coords = coords;
  H.scale = scale;
  H.regularization = regularization;
  // classify the terms of every sector
  struct Lists {
    std::vector<const StencilTerm*> diag, side, gain;
  };
  std::vector<Lists> L(S);
  int dir = 0;  // -1: gains read level lambda + 2 (sweep lambda downward); +1 the reverse
  for (int s = 0; s < S; ++s) {
    for (const StencilTerm& t : hp.sectors[s].terms) {
      if (t.p != t.q) continue;  // changes the charge d: the drive, left out of L0
      if (t.p == 0) {
        if (t.src == s && t.e == 0) {
          L[s].diag.push_back(&t);
        } else if (t.src == s - 1 || t.src == s + 1) {
          L[s].side.push_back(&t);
        } else {
          *err = "a charge-keeping term couples non-adjacent sectors";
          return PI_ERR_UNSUPPORTED;
        }
      } else if (t.p == -1 || t.p == 1) {
        if (t.src < s - 1 || t.src > s + 1) {
          *err = "a charge-keeping gain couples non-adjacent sectors";
          return PI_ERR_UNSUPPORTED;
        }
        const int d = t.p < 0 ? -1 : 1;
        if (dir != 0 && dir != d) {
          *err = "the level-sweep preconditioner needs all charge-keeping gains to raise, or all to lower, the "
                 "magnetic number (decay-type or pump-type channels, not both)";
          return PI_ERR_UNSUPPORTED;
        }
        dir = d;
        L[s].gain.push_back(&t);
      } else {
        *err = "a charge-keeping term reaches more than one level";
        return PI_ERR_UNSUPPORTED;
      }
    }
  }
  if (dir == 0) dir = -1;
  H.direction = dir;
  std::vector<int> n(S);
  std::vector<double> sqf(S), f(S);
  for (int s = 0; s < S; ++s) {
    n[s] = hp.sectors[s].n;
    sqf[s] = hp.sectors[s].sqrt_f;
    f[s] = hp.sectors[s].f;
  }
  auto ratio = [&](int s, int src) { return coords == PI_COORDS_POPULATION ? sqf[s] / sqf[src] : 1.0; };
  const int nmax = n[0];
  // levels lambda = n - 1 - 2a, all of the parity of nmax - 1
  std::vector<int> lams;
  for (int lam = nmax - 1; lam >= -(nmax - 1); lam -= 2) lams.push_back(lam);
  if (dir > 0) std::reverse(lams.begin(), lams.end());
  // chains d = -(nmax-1) .. nmax-1
  double maxdiag = 0.0;
  std::vector<int> chain_len;
  H.chain_lev.push_back(0);
  H.lev_ent.push_back(0);
  for (int d = -(nmax - 1); d <= nmax - 1; ++d) {
    if (d == 0) H.chain0 = (int)H.chain_lev.size() - 1;
    const int chain_first_entry = (int)H.elem.size();
    for (int lam : lams) {
      const int need = std::max(std::abs(lam), std::abs(lam - 2 * d));
      int cnt = 0;
      while (cnt < S && n[cnt] - 1 >= need) ++cnt;
      if (cnt == 0) continue;
      if (d == 0 && H.chain0_ent < 0) H.chain0_ent = (int)H.elem.size();
      // tridiagonal coefficients over the sectors 0..cnt-1 at this (d, lambda)
      std::vector<cdv> D(cnt), lo(cnt), up(cnt);
      std::vector<double> mag(cnt, 0.0);
      for (int s = 0; s < cnt; ++s) {
        const int a = (n[s] - 1 - lam) / 2, b = a + d;
        H.elem.push_back((int)(hp.sectors[s].offset + a + (long long)b * n[s]));
        cdv dv = 0.0;
        for (const StencilTerm* t : L[s].diag) {
          const cdv c = term_coef(*t, a, b);
          dv += c;
          mag[s] += std::abs(c);
        }
        if (regularization > 0) dv += regularization * scale;
        D[s] = dv;
        for (const StencilTerm* t : L[s].side) {
          const int src = t->src;
          const int as = a + t->e, bs = b + t->e;
          if (as < 0 || bs < 0 || as >= n[src] || bs >= n[src] || src >= cnt) continue;
          const cdv c = term_coef(*t, a, b) * ratio(s, src);
          if (src == s - 1)
            lo[s] += c;
          else
            up[s] += c;
        }
        // gains from the previous level
        cdv g[3] = {0.0, 0.0, 0.0};
        bool has[3] = {false, false, false};
        for (const StencilTerm* t : L[s].gain) {
          const int src = t->src;
          const int as = a + t->e + t->p, bs = b + t->e + t->q;
          if (as < 0 || bs < 0 || as >= n[src] || bs >= n[src]) continue;
          const int slot = src - s + 1;
          g[slot] += term_coef(*t, a, b) * ratio(s, src);
          has[slot] = true;
        }
        int packed = 0;
        for (int k = 0; k < 3; ++k) {
          const int pos = has[k] ? s + k - 1 : kNoGain;
          packed |= pos << (10 * k);
          H.G.push_back(has[k] ? g[k] : cdv(0.0));
        }
        H.gsrc.push_back(packed);
        maxdiag = std::max(maxdiag, std::abs(dv));
      }
      // Thomas factors
      cdv cprev = 0.0;
      for (int s = 0; s < cnt; ++s) {
        const cdv lc = s > 0 ? lo[s] * cprev : cdv(0.0);
        const cdv piv = D[s] - lc;
        const double tol = 1e-11 * (mag[s] + std::abs(lc) + std::abs(D[s]));
        const long long e = (long long)H.elem.size() - cnt + s;
        if (std::abs(piv) <= tol || piv == cdv(0.0)) {
          H.zero_pivots.push_back(e);
          H.W.push_back(0.0);
          H.A.push_back(0.0);
          H.C.push_back(0.0);
          cprev = 0.0;
          continue;
        }
        const cdv w = 1.0 / piv;
        H.W.push_back(w);
        H.A.push_back(s > 0 ? -lo[s] * w : cdv(0.0));
        cprev = up[s] * w;
        H.C.push_back(-cprev);
      }
      H.lev_ent.push_back((int)H.elem.size());
      H.max_level = std::max(H.max_level, cnt);
    }
    H.chain_lev.push_back((int)H.lev_ent.size() - 1);
    chain_len.push_back((int)H.elem.size() - chain_first_entry);
  }
  H.maxdiag = maxdiag;
  for (size_t c = 0; c + 1 < H.chain_lev.size(); ++c)
    if (H.chain_lev[c + 1] - H.chain_lev[c] > 2 * kPrecondMaxLevel + 2) {
      *err = "a charge chain has more levels than the sweep kernel stages";
      return PI_ERR_UNSUPPORTED;
    }
  if ((long long)H.elem.size() != hp.dim) {
    *err = "level decomposition does not cover the basis";
    return PI_ERR_UNSUPPORTED;
  }
  // chain 0 data: trace weights t and border v (in the solve's coordinates)
  const int c0 = H.chain0;
  const int e0 = H.chain0_ent, e1 = H.lev_ent[H.chain_lev[c0 + 1]];
  for (int e = e0; e < e1; ++e) {
    const long long el = H.elem[e];
    int s = S - 1;
    while (s > 0 && hp.sectors[s].offset > el) --s;
    const double t = coords == PI_COORDS_POPULATION ? 1.0 : sqf[s];
    const double v = coords == PI_COORDS_POPULATION ? f[s] / hp.trace_norm2 : sqf[s] / hp.trace_norm2;
    H.t0.push_back(t);
    H.v0.push_back(v);
  }
  // the free entry: one zero pivot, alone in the last level of the d = 0 chain
  const int last_lev = H.chain_lev[c0 + 1] - 1;
  const bool last_single = H.lev_ent[last_lev + 1] - H.lev_ent[last_lev] == 1;
  if (H.zero_pivots.size() == 1 && H.zero_pivots[0] == e1 - 1 && last_single) {
    H.mode = 0;
    H.free_ent = (int)H.zero_pivots[0];
  } else if (!H.zero_pivots.empty()) {
    *err = "a level block of the preconditioner is singular; pass a small regularization";
    return PI_ERR_INVALID_ARGUMENT;
  } else {
    H.mode = 1;
  }
  // Host sweep of s v over the d = 0 chain in FP64 (the free equation dropped): y_v, and
  // rho_v, the dropped equation's residual (mode 0), or w0 = s L0^-1 v (mode 1).
  {
    const int nl0 = H.chain_lev[c0], nl1 = H.chain_lev[c0 + 1];
    std::vector<cdv> yv(e1 - e0, 0.0);
    std::vector<cdv> prevu, curu;
    cdv rho_v = 0.0;
    for (int lev = nl0; lev < nl1; ++lev) {
      const int b0 = H.lev_ent[lev], cnt = H.lev_ent[lev + 1] - b0;
      std::vector<cdv> y(cnt);
      for (int i = 0; i < cnt; ++i) {
        const int e = b0 + i;
        cdv rv = scale * H.v0[e - e0];
        for (int k = 0; k < 3; ++k) {
          const int pos = (H.gsrc[e] >> (10 * k)) & 1023;
          if (pos != kNoGain) rv -= H.G[3LL * e + k] * prevu[pos];
        }
        if (e == H.free_ent) rho_v = rv;
        y[i] = H.W[e] * rv;
        if (i > 0) y[i] += H.A[e] * y[i - 1];
      }
      curu.assign(cnt, 0.0);
      for (int i = cnt - 1; i >= 0; --i) curu[i] = y[i] + (i + 1 < cnt ? H.C[b0 + i] * curu[i + 1] : cdv(0.0));
      for (int i = 0; i < cnt; ++i) yv[b0 + i - e0] = curu[i];
      prevu = curu;
    }
    H.w0 = yv;
    if (H.mode == 0) {
      if (std::abs(rho_v) == 0.0) {
        *err = "the trace border does not fix the free entry of the preconditioner; pass a small regularization";
        return PI_ERR_INVALID_ARGUMENT;
      }
      H.sm_coef = rho_v;
    } else {
      cdv tw = 0.0;
      for (int e = e0; e < e1; ++e) tw += H.t0[e - e0] * yv[e - e0];
      H.sm_coef = 1.0 / (1.0 + tw);
    }
  }
  // schedule: longest chains first
  H.chain_order.resize(chain_len.size());
  for (size_t i = 0; i < chain_len.size(); ++i) H.chain_order[i] = (int)i;
  std::stable_sort(H.chain_order.begin(), H.chain_order.end(),
                   [&](int x, int y) { return chain_len[x] > chain_len[y]; });
  return PI_OK;
}

}  // namespace picuda

struct pi_precond {
  pi_plan* plan = nullptr;
  int kind = PI_PRECOND_LEVEL;
  picuda::LevelPrecondHost host;  // kind LEVEL: the tables; both kinds: coords and scale
  picuda::PrecondDev dev{};
  picuda::DriveState* drive = nullptr;  // kind DRIVE
  int fp64 = 0;
  size_t bytes = 0;
  double setup_seconds = 0.0;
  std::vector<void*> allocs;
};

namespace picuda {
namespace {

template <typename X>
int upload_vec(pi_precond* P, const std::vector<X>& v, const X** out) {
  void* p = nullptr;
  const size_t bytes = std::max<size_t>(sizeof(X) * v.size(), 16);
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return cuda_fail(e, "preconditioner tables");
  P->allocs.push_back(p);
  P->bytes += bytes;
  if (!v.empty()) {
    e = cudaMemcpy(p, v.data(), sizeof(X) * v.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "preconditioner upload");
  }
  *out = (const X*)p;
  return PI_OK;
}

template <typename T>
int upload_factors(pi_precond* P) {
  using T2 = typename V2<T>::type;
  const LevelPrecondHost& H = P->host;
  auto conv = [](const std::vector<cdv>& v) {
    std::vector<T2> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) o[i] = V2<T>::make((T)v[i].real(), (T)v[i].imag());
    return o;
  };
  int rc;
  const T2* p = nullptr;
  if ((rc = upload_vec(P, conv(H.W), &p))) return rc;
  P->dev.W = p;
  if ((rc = upload_vec(P, conv(H.A), &p))) return rc;
  P->dev.A = p;
  if ((rc = upload_vec(P, conv(H.C), &p))) return rc;
  P->dev.C = p;
  if ((rc = upload_vec(P, conv(H.G), &p))) return rc;
  P->dev.G = p;
  return PI_OK;
}

void free_precond(pi_precond* P) {
  if (!P) return;
  for (void* p : P->allocs) cudaFree(p);
  drive_free(P->drive);
  delete P;
}

}  // namespace

cudaError_t precond_apply(const pi_precond* P, const void* r, int r_f32, void* z, int z_f32, double scale,
                          cudaStream_t stream) {
  // the drive state's scratch is written: applications on one plan are serialised by its lock
  if (P->kind == PI_PRECOND_DRIVE) return drive_apply(P->drive, r, r_f32, z, z_f32, stream);
  const PrecondDev& D = P->dev;
  const int blocks = (int)P->host.chain_order.size();
  if (r_f32 != z_f32) return cudaErrorInvalidValue;
  if (P->fp64)
    return r_f32 ? launch_sweep<double, float2, float2>(D, blocks, r, z, scale, stream)
                 : launch_sweep<double, double2, double2>(D, blocks, r, z, scale, stream);
  return r_f32 ? launch_sweep<float, float2, float2>(D, blocks, r, z, scale, stream)
               : launch_sweep<float, double2, double2>(D, blocks, r, z, scale, stream);
}

int precond_coords(const pi_precond* P) { return P->host.coords; }
int precond_kind(const pi_precond* P) { return P->kind; }
double precond_scale(const pi_precond* P) { return P->host.scale; }
const pi_plan* precond_plan(const pi_precond* P) { return P->plan; }

}  // namespace picuda

using namespace picuda;

namespace picuda {
// operator-scale estimate of the plan in the given coordinates (pi_solvers.cu)
int estimate_operator_scale(pi_plan* plan, int coords, double* out);
}  // namespace picuda

extern "C" {

int pi_precond_create(pi_plan* plan, int coords, double regularization, double operator_scale, pi_precond** out) {
  if (!plan || !out) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (coords != PI_COORDS_REFERENCE && coords != PI_COORDS_POPULATION)
    return fail(PI_ERR_INVALID_ARGUMENT, "coords must be PI_COORDS_REFERENCE or PI_COORDS_POPULATION");
  if (!(std::isfinite(regularization) && regularization >= 0))
    return fail(PI_ERR_INVALID_ARGUMENT, "regularization must be finite and nonnegative");
  if (operator_scale != 0 && !(std::isfinite(operator_scale) && operator_scale > 0))
    return fail(PI_ERR_INVALID_ARGUMENT, "operator_scale must be finite and positive");
  const auto t0 = std::chrono::steady_clock::now();
  double s = operator_scale;
  if (s == 0) {
    const int rc = estimate_operator_scale(plan, coords, &s);
    if (rc) return rc;
  }
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  pi_precond* P = new pi_precond();
  P->plan = plan;
  P->fp64 = coords == PI_COORDS_REFERENCE ? 1 : 0;
  std::string err;
  int rc = build_level_precond(plan->host, coords, regularization, s, &P->host, &err);
  if (rc) {
    delete P;
    return fail(rc, err);
  }
  const LevelPrecondHost& H = P->host;
  const int* ip = nullptr;
  if ((rc = upload_vec(P, H.chain_order, &ip))) return free_precond(P), rc;
  P->dev.chain_order = ip;
  if ((rc = upload_vec(P, H.chain_lev, &ip))) return free_precond(P), rc;
  P->dev.chain_lev = ip;
  if ((rc = upload_vec(P, H.lev_ent, &ip))) return free_precond(P), rc;
  P->dev.lev_ent = ip;
  if ((rc = upload_vec(P, H.elem, &ip))) return free_precond(P), rc;
  P->dev.elem = ip;
  {
    // the kernel keeps each level in slot order (entry i of a level with K = ceil(cnt / 32)
    // entries per lane at (i mod K) 32 + i / K): store the gain positions as slots of the
    // previous level
    std::vector<int> gslot(H.gsrc.size());
    for (size_t c = 0; c + 1 < H.chain_lev.size(); ++c) {
      for (int lev = H.chain_lev[c]; lev < H.chain_lev[c + 1]; ++lev) {
        const int Kp = lev > H.chain_lev[c] ? (H.lev_ent[lev] - H.lev_ent[lev - 1] + 31) / 32 : 1;
        for (int e = H.lev_ent[lev]; e < H.lev_ent[lev + 1]; ++e) {
          int packed = 0;
          for (int q = 0; q < 3; ++q) {
            int pos = (H.gsrc[e] >> (10 * q)) & 1023;
            if (pos != 1023) pos = (pos % Kp) * 32 + pos / Kp;
            packed |= pos << (10 * q);
          }
          gslot[e] = packed;
        }
      }
    }
    if ((rc = upload_vec(P, gslot, &ip))) return free_precond(P), rc;
  }
  P->dev.gsrc = ip;
  rc = P->fp64 ? upload_factors<double>(P) : upload_factors<float>(P);
  if (rc) return free_precond(P), rc;
  const double* dp = nullptr;
  if ((rc = upload_vec(P, H.t0, &dp))) return free_precond(P), rc;
  P->dev.t0 = dp;
  if ((rc = upload_vec(P, H.v0, &dp))) return free_precond(P), rc;
  P->dev.v0 = dp;
  std::vector<double2> w0(H.w0.size());
  for (size_t i = 0; i < w0.size(); ++i) w0[i] = make_double2(H.w0[i].real(), H.w0[i].imag());
  const double2* wp = nullptr;
  if ((rc = upload_vec(P, w0, &wp))) return free_precond(P), rc;
  P->dev.w0 = wp;
  P->dev.chain0 = H.chain0;
  P->dev.chain0_ent = H.chain0_ent;
  P->dev.free_ent = H.free_ent;
  P->dev.mode = H.mode;
  P->dev.sm_coef = make_double2(H.sm_coef.real(), H.sm_coef.imag());
  P->setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *out = P;
  return PI_OK;
}

int pi_precond_create_drive(pi_plan* plan, int coords, double operator_scale, pi_precond** out) {
  if (!plan || !out) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (coords != PI_COORDS_REFERENCE && coords != PI_COORDS_POPULATION)
    return fail(PI_ERR_INVALID_ARGUMENT, "coords must be PI_COORDS_REFERENCE or PI_COORDS_POPULATION");
  if (operator_scale != 0 && !(std::isfinite(operator_scale) && operator_scale > 0))
    return fail(PI_ERR_INVALID_ARGUMENT, "operator_scale must be finite and positive");
  double s = operator_scale;
  if (s == 0) {
    const int rc = estimate_operator_scale(plan, coords, &s);
    if (rc) return rc;
  }
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  pi_precond* P = new pi_precond();
  P->plan = plan;
  P->kind = PI_PRECOND_DRIVE;
  P->fp64 = 0;
  P->host.coords = coords;
  P->host.scale = s;
  std::string err;
  const int rc = drive_create(plan, coords, s, &P->drive, &err);
  if (rc) {
    delete P;
    return fail(rc, err);
  }
  P->bytes = drive_bytes(P->drive);
  P->setup_seconds = drive_setup_seconds(P->drive);
  *out = P;
  return PI_OK;
}

int pi_precond_destroy(pi_precond* P) {
  free_precond(P);
  return PI_OK;
}

int pi_precond_info(const pi_precond* P, pi_precond_info_t* out) {
  if (!P || !out) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  const LevelPrecondHost& H = P->host;
  out->coords = H.coords;
  out->fp64 = P->fp64;
  out->operator_scale = H.scale;
  out->regularization = H.regularization;
  out->chains = (int)H.chain_order.size();
  out->levels = (int)H.lev_ent.size() - 1;
  out->entries = (long long)H.elem.size();
  out->max_level = H.max_level;
  out->direction = H.direction;
  out->singular = H.mode == 0 ? 1 : 0;
  out->device_bytes = P->bytes;
  out->setup_seconds = P->setup_seconds;
  out->kind = P->kind;
  out->max_asymmetry = 0.0;
  out->max_nonhermitian = 0.0;
  if (P->kind == PI_PRECOND_DRIVE) {
    const DriveHost& D = drive_host(P->drive);
    out->chains = out->levels = out->max_level = out->direction = out->singular = 0;
    out->entries = P->plan->host.dim;
    out->max_asymmetry = D.max_asymmetry;
    out->max_nonhermitian = D.max_nonhermitian;
  }
  return PI_OK;
}

int pi_precond_apply(const pi_precond* P, double* z_dev, const double* r_dev, void* stream) {
  if (!P || !z_dev || !r_dev) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (z_dev == r_dev) return fail(PI_ERR_INVALID_ARGUMENT, "source and destination must not share storage");
  cudaError_t e = precond_apply(P, r_dev, 0, z_dev, 0, P->host.scale, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "preconditioner apply");
  return PI_OK;
}

}  // extern "C"
