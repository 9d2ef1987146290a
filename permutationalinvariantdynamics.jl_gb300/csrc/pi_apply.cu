// Fused Schur-block Liouvillian action y = L x on sm_103a.
//
// Replaces the reference's fused static kernel apply (src/liouvillian.jl:3070-3105), which
// copies every sector into dense scratch (:2952-2958) and runs sparse x dense products for
// the Hamiltonian commutator, the loss anticommutator and the collective gains plus the
// support-path sandwich loops of the one-body gains (:2486-2561).  Here every output entry
// (j, m, m') is produced once by one thread as a gather over the separable stencil terms
// of its sector: no scratch copies, one read stream of x (neighbouring sectors j +- 1 come
// from L2) and one write of y.  The same kernel serves the plain FP64 path (reference
// coordinates) and the FP32 path (population coordinates z = sqrt(f) x).
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

template <typename T, typename T2>
__device__ __forceinline__ void accumulate_term(const DevTerm& tm, const T2* __restrict__ coef, int a,
                                                int b, T2 xv, T& accr, T& acci) {
  switch (tm.kind) {
    case 0: {  // ADD: (alpha[a] + beta[b]) x[a, b]
      T2 al = __ldg(coef + tm.alpha_off + a);
      T2 be = __ldg(coef + tm.beta_off + b);
      T cr = al.x + be.x, ci = al.y + be.y;
      accr = fma(cr, xv.x, accr);
      accr = fma(-ci, xv.y, accr);
      acci = fma(cr, xv.y, acci);
      acci = fma(ci, xv.x, acci);
      break;
    }
    case 1: {  // LEFT: alpha[a] x[a + dr, b]
      T2 al = __ldg(coef + tm.alpha_off + a);
      if (tm.cls == 1) {
        accr = fma(-al.y, xv.y, accr);
        acci = fma(al.y, xv.x, acci);
      } else if (tm.cls == 0) {
        accr = fma(al.x, xv.x, accr);
        acci = fma(al.x, xv.y, acci);
      } else {
        accr = fma(al.x, xv.x, accr);
        accr = fma(-al.y, xv.y, accr);
        acci = fma(al.x, xv.y, acci);
        acci = fma(al.y, xv.x, acci);
      }
      break;
    }
    case 2: {  // RIGHT: beta[b] x[a, b + dc]
      T2 be = __ldg(coef + tm.beta_off + b);
      if (tm.cls == 1) {
        accr = fma(-be.y, xv.y, accr);
        acci = fma(be.y, xv.x, acci);
      } else if (tm.cls == 0) {
        accr = fma(be.x, xv.x, accr);
        acci = fma(be.x, xv.y, acci);
      } else {
        accr = fma(be.x, xv.x, accr);
        accr = fma(-be.y, xv.y, accr);
        acci = fma(be.x, xv.y, acci);
        acci = fma(be.y, xv.x, acci);
      }
      break;
    }
    default: {  // SAND: alpha[a] beta[b] x[a + dr, b + dc]
      T2 al = __ldg(coef + tm.alpha_off + a);
      T2 be = __ldg(coef + tm.beta_off + b);
      if (tm.cls == 0) {
        T c = al.x * be.x;
        accr = fma(c, xv.x, accr);
        acci = fma(c, xv.y, acci);
      } else {
        T cr = al.x * be.x - al.y * be.y;
        T ci = al.x * be.y + al.y * be.x;
        accr = fma(cr, xv.x, accr);
        accr = fma(-ci, xv.y, accr);
        acci = fma(cr, xv.y, acci);
        acci = fma(ci, xv.x, acci);
      }
      break;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kApplyThreads)
    k_apply(const DevSector* __restrict__ sectors, const DevTerm* __restrict__ terms,
            const typename Vec2<T>::type* __restrict__ coef, const DevTile* __restrict__ tiles,
            const typename Vec2<T>::type* __restrict__ x, typename Vec2<T>::type* __restrict__ y,
            long long ld, BorderArgs border) {
  using T2 = typename Vec2<T>::type;
  const DevTile tile = tiles[blockIdx.x];
  const long long col = blockIdx.y;
  x += col * ld;
  y += col * ld;
  const DevSector sec = sectors[tile.sector];
  const int a = tile.a0 + (threadIdx.x & (kTileRows - 1));
  const int b = tile.b0 + (threadIdx.x / kTileRows);
  if (a >= sec.n || b >= sec.n) return;
  T accr = 0, acci = 0;
  const int tend = sec.term_begin + sec.term_count;
  for (int t = sec.term_begin; t < tend; ++t) {
    const DevTerm tm = terms[t];
    const int r = a + tm.dr, c = b + tm.dc;
    if (r < 0 || r >= tm.src_n || c < 0 || c >= tm.src_n) continue;
    const T2 xv = __ldg(x + tm.src_off + r + (long long)c * tm.src_n);
    accumulate_term<T, T2>(tm, coef, a, b, xv, accr, acci);
  }
  T2 out;
  out.x = (T)border.scale * accr;
  out.y = (T)border.scale * acci;
  if (border.alpha != nullptr && a == b) {
    const double2 al = border.alpha[col];
    const double v = border.coords ? sec.border_z : sec.border_x;
    out.x += (T)(al.x * v);
    out.y += (T)(al.y * v);
  }
  y[sec.offset + a + (long long)b * sec.n] = out;
}

template <typename T>
cudaError_t launch_apply_t(const DevicePlan& dp, const void* coef, const void* x, void* y, int ncols,
                           long long ld, const BorderArgs& border, cudaStream_t stream) {
  using T2 = typename Vec2<T>::type;
  if (dp.ntiles == 0 || ncols == 0) return cudaSuccess;
  dim3 grid((unsigned)dp.ntiles, (unsigned)ncols);
  k_apply<T><<<grid, kApplyThreads, 0, stream>>>(dp.sectors, dp.terms, (const T2*)coef, dp.tiles,
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
