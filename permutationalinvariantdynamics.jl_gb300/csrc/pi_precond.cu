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
// two warps each.  Warp 1 stages the next level's right-hand sides and factors into shared
// memory while warp 0 runs the current level: all lanes form the right-hand sides from the
// previous level's solution, then lane 0 runs the forward and backward Thomas recurrences
// and all lanes write the level's entries out.  Population coordinates run in FP32 (the
// preconditioner is an approximation of L^-1 either way, and every entry is a bounded
// population); reference coordinates run in FP64, since their entries span many decades at
// large N.
#include <cuda_runtime.h>

#include <algorithm>
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

namespace picuda {

namespace {

constexpr int kSweepThreads = 64;
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

// Block-wide sum of two doubles per thread over a 64-thread block (fixed order).
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

template <typename T>
struct Stage {
  using T2 = typename V2<T>::type;
  T2 rhs[2][kPrecondMaxLevel];   // s r of each entry
  T2 w[2][kPrecondMaxLevel];     // 1 / pivot
  T2 a[2][kPrecondMaxLevel];     // forward multiplier
  T2 c[2][kPrecondMaxLevel];     // backward multiplier
  T2 g[2][kPrecondMaxLevel][3];  // gain coefficients
  int gp[2][kPrecondMaxLevel];   // packed gain positions in the previous level
  int el[2][kPrecondMaxLevel];   // element index
  T2 y[kPrecondMaxLevel];        // forward values
  T2 u[2][kPrecondMaxLevel];     // solution of the previous / current level
  double red[2 * (kSweepThreads / 32)];
};

template <typename T, typename TI>
__device__ __forceinline__ void stage_level(const PrecondDev& P, const TI* __restrict__ r, Stage<T>& S, int slot,
                                            int lev, int lane, double s) {
  using T2 = typename V2<T>::type;
  const T2* W = reinterpret_cast<const T2*>(P.W);
  const T2* A = reinterpret_cast<const T2*>(P.A);
  const T2* C = reinterpret_cast<const T2*>(P.C);
  const T2* G = reinterpret_cast<const T2*>(P.G);
  const int e0 = P.lev_ent[lev], cnt = P.lev_ent[lev + 1] - e0;
  for (int i = lane; i < cnt; i += 32) {
    const int e = e0 + i;
    const int el = P.elem[e];
    const double2 rv = load_d2(r + el);
    S.rhs[slot][i] = V2<T>::make((T)(s * rv.x), (T)(s * rv.y));
    S.w[slot][i] = W[e];
    S.a[slot][i] = A[e];
    S.c[slot][i] = C[e];
    S.gp[slot][i] = P.gsrc[e];
#pragma unroll
    for (int k = 0; k < 3; ++k) S.g[slot][i][k] = G[3LL * e + k];
    S.el[slot][i] = el;
  }
}

template <typename T, typename TI, typename TO>
__global__ void __launch_bounds__(kSweepThreads)
    k_level_sweep(const PrecondDev P, const TI* __restrict__ r, TO* __restrict__ z, double s) {
  using T2 = typename V2<T>::type;
  __shared__ Stage<T> S;
  __shared__ double2 rho_r;  // residual of the dropped free equation (d = 0 chain, mode 0)
  const int chain = P.chain_order[blockIdx.x];
  const int lev0 = P.chain_lev[chain], lev1 = P.chain_lev[chain + 1];
  const bool chain0 = chain == P.chain0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) rho_r = make_double2(0.0, 0.0);
  if (warp == 1) stage_level<T, TI>(P, r, S, 0, lev0, lane, s);
  __syncthreads();
  double2 tsum = make_double2(0.0, 0.0);
  int prev = 0, cur = 1;
  for (int lev = lev0; lev < lev1; ++lev) {
    const int slot = (lev - lev0) & 1;
    if (warp == 1) {
      if (lev + 1 < lev1) stage_level<T, TI>(P, r, S, slot ^ 1, lev + 1, lane, s);
    } else {
      const int e0 = P.lev_ent[lev];
      const int cnt = P.lev_ent[lev + 1] - e0;
      for (int i = lane; i < cnt; i += 32) {
        T2 rv = S.rhs[slot][i];
        const int packed = S.gp[slot][i];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int pos = (packed >> (10 * k)) & 1023;
          if (pos != kNoGain) {
            const T2 g = S.g[slot][i][k];
            const T2 un = S.u[prev][pos];
            T2 m;
            m.x = -g.x;
            m.y = -g.y;
            rv = cfma(m, un, rv);
          }
        }
        if (e0 + i == P.free_ent) rho_r = make_double2((double)rv.x, (double)rv.y);
        S.y[i] = cmul(S.w[slot][i], rv);
      }
      __syncwarp();
      if (lane == 0) {
        // forward: y_i += A_i y_{i-1}; backward: u_i = y_i + C_i u_{i+1}
        T2 yp = S.y[0];
        for (int i = 1; i < cnt; ++i) {
          yp = cfma(S.a[slot][i], yp, S.y[i]);
          S.y[i] = yp;
        }
        T2 un = S.y[cnt - 1];
        S.u[cur][cnt - 1] = un;
        for (int i = cnt - 2; i >= 0; --i) {
          un = cfma(S.c[slot][i], un, S.y[i]);
          S.u[cur][i] = un;
        }
      }
      __syncwarp();
      for (int i = lane; i < cnt; i += 32) {
        const T2 uv = S.u[cur][i];
        store_as<TO, T2>(z + S.el[slot][i], uv);
        if (chain0 && P.mode == 1) {
          const double t = P.t0[e0 + i - P.chain0_ent];
          tsum.x = fma(t, (double)uv.x, tsum.x);
          tsum.y = fma(t, (double)uv.y, tsum.y);
        }
      }
    }
    __syncthreads();
    prev ^= 1;
    cur ^= 1;
  }
  if (!chain0) return;
  const int c0 = P.chain0_ent, c1 = P.lev_ent[lev1];
  if (P.mode == 0) {
    // beta = rho_r / rho_v; y = y_r - beta y_v; z_f = (beta - t^H y) / t_f
    const double2 rv = P.sm_coef;  // rho_v
    const double den = rv.x * rv.x + rv.y * rv.y;
    const double2 beta = make_double2((rho_r.x * rv.x + rho_r.y * rv.y) / den, (rho_r.y * rv.x - rho_r.x * rv.y) / den);
    for (int e = c0 + tid; e < c1; e += blockDim.x) {
      const int el = P.elem[e];
      const double2 yv = P.w0[e - c0];
      double2 zv = load_d2(z + el);
      zv.x -= beta.x * yv.x - beta.y * yv.y;
      zv.y -= beta.x * yv.y + beta.y * yv.x;
      store_as<TO, double2>(z + el, zv);
      const double t = P.t0[e - c0];
      tsum.x = fma(t, zv.x, tsum.x);
      tsum.y = fma(t, zv.y, tsum.y);
    }
    const double2 tz = block_sum2(tsum, S.red);
    if (tid == 0 && P.free_ent >= 0) {
      const double t = P.t0[P.free_ent - c0];
      store_as<TO, double2>(z + P.elem[P.free_ent], make_double2((beta.x - tz.x) / t, (beta.y - tz.y) / t));
    }
  } else {
    // Sherman-Morrison: z -= w0 (t^H y) / (1 + t^H w0)
    const double2 tz = block_sum2(tsum, S.red);
    const double2 k = make_double2(tz.x * P.sm_coef.x - tz.y * P.sm_coef.y, tz.x * P.sm_coef.y + tz.y * P.sm_coef.x);
    for (int e = c0 + tid; e < c1; e += blockDim.x) {
      const int el = P.elem[e];
      const double2 w0 = P.w0[e - c0];
      double2 zv = load_d2(z + el);
      zv.x -= w0.x * k.x - w0.y * k.y;
      zv.y -= w0.x * k.y + w0.y * k.x;
      store_as<TO, double2>(z + el, zv);
    }
  }
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
  picuda::LevelPrecondHost host;
  picuda::PrecondDev dev{};
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
  delete P;
}

}  // namespace

cudaError_t precond_apply(const pi_precond* P, const void* r, int r_f32, void* z, int z_f32, double scale,
                          cudaStream_t stream) {
  const PrecondDev& D = P->dev;
  const int blocks = (int)P->host.chain_order.size();
  if (P->fp64) {
    if (!r_f32 && !z_f32)
      k_level_sweep<double, double2, double2><<<blocks, kSweepThreads, 0, stream>>>(D, (const double2*)r,
                                                                                   (double2*)z, scale);
    else if (r_f32 && z_f32)
      k_level_sweep<double, float2, float2><<<blocks, kSweepThreads, 0, stream>>>(D, (const float2*)r,
                                                                                 (float2*)z, scale);
    else
      return cudaErrorInvalidValue;
  } else {
    if (!r_f32 && !z_f32)
      k_level_sweep<float, double2, double2><<<blocks, kSweepThreads, 0, stream>>>(D, (const double2*)r,
                                                                                  (double2*)z, scale);
    else if (r_f32 && z_f32)
      k_level_sweep<float, float2, float2><<<blocks, kSweepThreads, 0, stream>>>(D, (const float2*)r,
                                                                                (float2*)z, scale);
    else
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

int precond_coords(const pi_precond* P) { return P->host.coords; }
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
  if ((rc = upload_vec(P, H.gsrc, &ip))) return free_precond(P), rc;
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
