// Krylov vector kernels: CGS2 multi-dots and multi-axpys, norms, combinations and the
// trace functional, all with deterministic two-stage reductions (fixed element-to-block
// partition, fixed tree order), so a solve is bitwise reproducible run to run.
//
// Replaces the orthogonalisation loops of the reference (MGS x2: src/krylov.jl:762-766,
// src/krylov_extensions.jl:1358-1363), the basis combinations (krylov.jl:779,
// krylov_extensions.jl:1415-1416) and the trace functional dot (krylov.jl:855-860).
#include <algorithm>

#include "pi_internal.hpp"

namespace picuda {

namespace {

__device__ __forceinline__ void chunk_bounds(long long n, long long& beg, long long& end) {
  beg = (long long)blockIdx.x * n / gridDim.x;
  end = (long long)(blockIdx.x + 1) * n / gridDim.x;
}

// Block-wide sum of NV values per thread (deterministic); result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[warp * NV + k] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = lane < nw ? smem[lane * NV + k] : 0.0;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
    }
  }
  __syncthreads();
}

template <typename T2>
__device__ __forceinline__ double2 load_c(const T2* p) {
  T2 v = __ldg(p);
  return make_double2((double)v.x, (double)v.y);
}

// Stage 1 of a multi-dot: block (bx, by) reduces vectors by*8 .. by*8+7 over element chunk
// bx and writes partial[bx][i].  One block-wide sum per block.
constexpr int kDotGroup = 8;

template <typename T2>
__global__ void __launch_bounds__(kReduceThreads)
    k_mdot_partial(const T2* __restrict__ V, long long ldv, int nv, const T2* __restrict__ w, long long n,
                   double2* __restrict__ partial) {
  __shared__ double smem[32 * 2 * kDotGroup];
  long long beg, end;
  chunk_bounds(n, beg, end);
  const int g = blockIdx.y * kDotGroup;
  const int cnt = min(kDotGroup, nv - g);
  double acc[2 * kDotGroup];
#pragma unroll
  for (int k = 0; k < 2 * kDotGroup; ++k) acc[k] = 0.0;
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const double2 wv = load_c(w + e);
#pragma unroll
    for (int k = 0; k < kDotGroup; ++k) {
      if (k < cnt) {
        const double2 v = load_c(V + (long long)(g + k) * ldv + e);
        acc[2 * k] = fma(v.x, wv.x, acc[2 * k]);
        acc[2 * k] = fma(v.y, wv.y, acc[2 * k]);
        acc[2 * k + 1] = fma(v.x, wv.y, acc[2 * k + 1]);
        acc[2 * k + 1] = fma(-v.y, wv.x, acc[2 * k + 1]);
      }
    }
  }
  block_sum<2 * kDotGroup>(acc, smem);
  if (threadIdx.x == 0) {
    for (int k = 0; k < cnt; ++k)
      partial[(long long)blockIdx.x * kMaxDots + g + k] = make_double2(acc[2 * k], acc[2 * k + 1]);
  }
}

// Double-float accumulator: the pair (hi, lo) carries a ~48-bit significand on the FP32
// pipes.  Products of two FP32 numbers are split exactly with an FMA (a*b = p + e) and
// added with Knuth's TwoSum, so a dot of FP32 vectors is accumulated to FP64-class accuracy
// without the GB300 FP64 pipe (1/64 of the FP32 rate).
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

// Stage 1 of a multi-dot for FP32 vectors with double-float accumulation (grid as above).
__global__ void __launch_bounds__(kReduceThreads)
    k_mdot_partial_df(const float2* __restrict__ V, long long ldv, int nv, const float2* __restrict__ w, long long n,
                      double2* __restrict__ partial) {
  __shared__ double smem[32 * 2 * kDotGroup];
  long long beg, end;
  chunk_bounds(n, beg, end);
  const int g = blockIdx.y * kDotGroup;
  const int cnt = min(kDotGroup, nv - g);
  DF re[kDotGroup], im[kDotGroup];
#pragma unroll
  for (int k = 0; k < kDotGroup; ++k) re[k] = im[k] = DF{0.f, 0.f};
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const float2 wv = __ldg(w + e);
#pragma unroll
    for (int k = 0; k < kDotGroup; ++k) {
      if (k < cnt) {
        const float2 v = __ldg(V + (long long)(g + k) * ldv + e);
        df_add_prod(re[k], v.x, wv.x);
        df_add_prod(re[k], v.y, wv.y);
        df_add_prod(im[k], v.x, wv.y);
        df_add_prod(im[k], -v.y, wv.x);
      }
    }
  }
  double acc[2 * kDotGroup];
#pragma unroll
  for (int k = 0; k < kDotGroup; ++k) {
    acc[2 * k] = (double)re[k].hi + (double)re[k].lo;
    acc[2 * k + 1] = (double)im[k].hi + (double)im[k].lo;
  }
  block_sum<2 * kDotGroup>(acc, smem);
  if (threadIdx.x == 0) {
    for (int k = 0; k < cnt; ++k)
      partial[(long long)blockIdx.x * kMaxDots + g + k] = make_double2(acc[2 * k], acc[2 * k + 1]);
  }
}

// w -= sum_i V_i h_i in FP32 (h rounded once), optional |w|^2 partials in double-float.
__global__ void __launch_bounds__(kReduceThreads)
    k_maxpy_f32(const float2* __restrict__ V, long long ldv, int nv, const double2* __restrict__ h,
                float2* __restrict__ w, long long n, double* __restrict__ rpartial) {
  __shared__ float2 hs[kMaxDots];
  __shared__ double smem[32];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) hs[i] = make_float2((float)h[i].x, (float)h[i].y);
  __syncthreads();
  long long beg, end;
  chunk_bounds(n, beg, end);
  DF nrm{0.f, 0.f};
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    float2 wv = w[e];
    for (int i = 0; i < nv; ++i) {
      const float2 v = __ldg(V + (long long)i * ldv + e);
      const float2 c = hs[i];
      wv.x = fmaf(-v.x, c.x, wv.x);
      wv.x = fmaf(v.y, c.y, wv.x);
      wv.y = fmaf(-v.x, c.y, wv.y);
      wv.y = fmaf(-v.y, c.x, wv.y);
    }
    w[e] = wv;
    df_add_prod(nrm, wv.x, wv.x);
    df_add_prod(nrm, wv.y, wv.y);
  }
  if (rpartial != nullptr) {
    double acc[1] = {(double)nrm.hi + (double)nrm.lo};
    block_sum<1>(acc, smem);
    if (threadIdx.x == 0) rpartial[blockIdx.x] = acc[0];
  }
}

__global__ void __launch_bounds__(kReduceThreads)
    k_norm2_df(const float2* __restrict__ w, long long n, double* __restrict__ rpartial) {
  __shared__ double smem[32];
  long long beg, end;
  chunk_bounds(n, beg, end);
  DF nrm{0.f, 0.f};
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const float2 v = __ldg(w + e);
    df_add_prod(nrm, v.x, v.x);
    df_add_prod(nrm, v.y, v.y);
  }
  double acc[1] = {(double)nrm.hi + (double)nrm.lo};
  block_sum<1>(acc, smem);
  if (threadIdx.x == 0) rpartial[blockIdx.x] = acc[0];
}

// Stage 2: one block per dot, fixed-order sum over the partials.
__global__ void __launch_bounds__(kReduceThreads)
    k_mdot_final(const double2* __restrict__ partial, int nblocks, double2* __restrict__ out) {
  __shared__ double smem[32 * 2];
  const int i = blockIdx.x;
  double acc[2] = {0, 0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double2 p = partial[(long long)b * kMaxDots + i];
    acc[0] += p.x;
    acc[1] += p.y;
  }
  block_sum<2>(acc, smem);
  if (threadIdx.x == 0) out[i] = make_double2(acc[0], acc[1]);
}

__global__ void __launch_bounds__(kReduceThreads)
    k_rfinal(const double* __restrict__ partial, int nblocks, double* __restrict__ out) {
  __shared__ double smem[32];
  double acc[1] = {0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc[0] += partial[b];
  block_sum<1>(acc, smem);
  if (threadIdx.x == 0) *out = acc[0];
}

// w -= sum_i V_i h_i, FP64 arithmetic, optional |w|^2 partials.
template <typename T2>
__global__ void __launch_bounds__(kReduceThreads)
    k_maxpy(const T2* __restrict__ V, long long ldv, int nv, const double2* __restrict__ h, T2* __restrict__ w,
            long long n, double* __restrict__ rpartial) {
  __shared__ double2 hs[kMaxDots];
  __shared__ double smem[32];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) hs[i] = h[i];
  __syncthreads();
  long long beg, end;
  chunk_bounds(n, beg, end);
  double acc[1] = {0};
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    T2 wr = w[e];
    double wx = (double)wr.x, wy = (double)wr.y;
    for (int i = 0; i < nv; ++i) {
      const double2 v = load_c(V + (long long)i * ldv + e);
      const double2 c = hs[i];
      wx = fma(-v.x, c.x, wx);
      wx = fma(v.y, c.y, wx);
      wy = fma(-v.x, c.y, wy);
      wy = fma(-v.y, c.x, wy);
    }
    T2 o;
    o.x = (decltype(o.x))wx;
    o.y = (decltype(o.y))wy;
    w[e] = o;
    acc[0] = fma((double)o.x, (double)o.x, acc[0]);
    acc[0] = fma((double)o.y, (double)o.y, acc[0]);
  }
  if (rpartial != nullptr) {
    block_sum<1>(acc, smem);
    if (threadIdx.x == 0) rpartial[blockIdx.x] = acc[0];
  }
}

template <typename T2>
__global__ void __launch_bounds__(kReduceThreads)
    k_norm2(const T2* __restrict__ w, long long n, double* __restrict__ rpartial) {
  __shared__ double smem[32];
  long long beg, end;
  chunk_bounds(n, beg, end);
  double acc[1] = {0};
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const double2 v = load_c(w + e);
    acc[0] = fma(v.x, v.x, acc[0]);
    acc[0] = fma(v.y, v.y, acc[0]);
  }
  block_sum<1>(acc, smem);
  if (threadIdx.x == 0) rpartial[blockIdx.x] = acc[0];
}

__global__ void k_scale_f64(const double2* __restrict__ x, double2* __restrict__ y, long long n, double2 a,
                            int accumulate) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const double2 v = x[e];
    double2 o = make_double2(a.x * v.x - a.y * v.y, a.x * v.y + a.y * v.x);
    if (accumulate) {
      const double2 p = y[e];
      o.x += p.x;
      o.y += p.y;
    }
    y[e] = o;
  }
}

__global__ void k_scale_f32(const float2* __restrict__ x, float2* __restrict__ y, long long n, double2 a) {
  const float ar = (float)a.x, ai = (float)a.y;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const float2 v = x[e];
    y[e] = make_float2(ar * v.x - ai * v.y, ar * v.y + ai * v.x);
  }
}

template <typename T2>
__global__ void __launch_bounds__(kReduceThreads)
    k_combine(const T2* __restrict__ V, long long ldv, int nv, const double2* __restrict__ c,
              double2* __restrict__ y, long long n, int accumulate) {
  __shared__ double2 cs[kMaxDots];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) cs[i] = c[i];
  __syncthreads();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    double yx = 0.0, yy = 0.0;
    for (int i = 0; i < nv; ++i) {
      const double2 v = load_c(V + (long long)i * ldv + e);
      const double2 a = cs[i];
      yx = fma(v.x, a.x, yx);
      yx = fma(-v.y, a.y, yx);
      yy = fma(v.x, a.y, yy);
      yy = fma(v.y, a.x, yy);
    }
    if (accumulate) {
      const double2 p = y[e];
      yx += p.x;
      yy += p.y;
    }
    y[e] = make_double2(yx, yy);
  }
}

// t^H x over all block diagonals; a single block, fixed order.
template <typename T2>
__global__ void __launch_bounds__(1024)
    k_trace_dot(const DevSector* __restrict__ sectors, const int* __restrict__ diag_sector,
                const long long* __restrict__ diag_index, int ndiag, const T2* __restrict__ x, int coords,
                double2* __restrict__ out) {
  __shared__ double smem[32 * 2];
  double acc[2] = {0, 0};
  for (int i = threadIdx.x; i < ndiag; i += blockDim.x) {
    const double w = coords ? 1.0 : sectors[diag_sector[i]].sqrt_f;
    const double2 v = load_c(x + diag_index[i]);
    acc[0] = fma(w, v.x, acc[0]);
    acc[1] = fma(w, v.y, acc[1]);
  }
  block_sum<2>(acc, smem);
  if (threadIdx.x == 0) *out = make_double2(acc[0], acc[1]);
}

// Coordinate change between reference coordinates x and population coordinates z.
template <typename TI, typename TO>
__global__ void k_coords(const DevSector* __restrict__ sectors, int nsectors, const TI* __restrict__ in,
                         TO* __restrict__ out, double scale, int to_z, int accumulate) {
  const int s = blockIdx.y;
  if (s >= nsectors) return;
  const DevSector sec = sectors[s];
  const long long cnt = (long long)sec.n * sec.n;
  const double f = (to_z ? sec.sqrt_f : 1.0 / sec.sqrt_f) * scale;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt;
       e += (long long)gridDim.x * blockDim.x) {
    const double2 v = load_c(in + sec.offset + e);
    double ox = f * v.x, oy = f * v.y;
    if (accumulate) {
      const double2 p = load_c((const TO*)out + sec.offset + e);
      ox += p.x;
      oy += p.y;
    }
    TO o;
    o.x = (decltype(o.x))ox;
    o.y = (decltype(o.y))oy;
    out[sec.offset + e] = o;
  }
}

__global__ void k_f64_to_f32(const double2* __restrict__ x, float2* __restrict__ y, long long n, double scale) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const double2 v = x[e];
    y[e] = make_float2((float)(scale * v.x), (float)(scale * v.y));
  }
}

__global__ void __launch_bounds__(kReduceThreads)
    k_weighted_norm2_z(const DevSector* __restrict__ sectors, int nsectors, const double2* __restrict__ z,
                       double* __restrict__ rpartial) {
  // one block per sector: sum |z|^2 / f
  __shared__ double smem[32];
  const int s = blockIdx.x;
  double acc[1] = {0};
  if (s < nsectors) {
    const DevSector sec = sectors[s];
    const long long cnt = (long long)sec.n * sec.n;
    for (long long e = threadIdx.x; e < cnt; e += blockDim.x) {
      const double2 v = z[sec.offset + e];
      acc[0] = fma(v.x, v.x, acc[0]);
      acc[0] = fma(v.y, v.y, acc[0]);
    }
    const double inv = 1.0 / sec.sqrt_f;
    acc[0] *= inv * inv;
  }
  block_sum<1>(acc, smem);
  if (threadIdx.x == 0) rpartial[blockIdx.x] = acc[0];
}

// Element-chunk blocks for a reduction over n entries: at least ~4 entries per thread,
// at most kReduceBlocks in total across the vector-group dimension.
inline int reduce_blocks(long long n, int ygroups) {
  long long b = (n + 4LL * kReduceThreads - 1) / (4LL * kReduceThreads);
  long long cap = std::max(1, kReduceBlocks / std::max(1, ygroups));
  return (int)std::max(1LL, std::min(b, cap));
}

inline int grid_for(long long n) {
  long long g = (n + 255) / 256;
  if (g > 4 * 152) g = 4 * 152;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

cudaError_t mdot_f64(const double2* V, long long ldv, int nv, const double2* w, long long n, ReduceScratch& rs,
                     double2* h_out, cudaStream_t stream) {
  if (nv <= 0) return cudaSuccess;
  if (nv > kMaxDots) return cudaErrorInvalidValue;
  const int gy = (nv + kDotGroup - 1) / kDotGroup;
  const int gx = reduce_blocks(n, gy);
  k_mdot_partial<double2><<<dim3(gx, gy), kReduceThreads, 0, stream>>>(V, ldv, nv, w, n, rs.partial);
  k_mdot_final<<<nv, kReduceThreads, 0, stream>>>(rs.partial, gx, h_out);
  return cudaGetLastError();
}

cudaError_t mdot_f32(const float2* V, long long ldv, int nv, const float2* w, long long n, ReduceScratch& rs,
                     double2* h_out, cudaStream_t stream) {
  if (nv <= 0) return cudaSuccess;
  if (nv > kMaxDots) return cudaErrorInvalidValue;
  const int gy = (nv + kDotGroup - 1) / kDotGroup;
  const int gx = reduce_blocks(n, gy);
  k_mdot_partial_df<<<dim3(gx, gy), kReduceThreads, 0, stream>>>(V, ldv, nv, w, n, rs.partial);
  k_mdot_final<<<nv, kReduceThreads, 0, stream>>>(rs.partial, gx, h_out);
  return cudaGetLastError();
}

cudaError_t maxpy_f64(const double2* V, long long ldv, int nv, const double2* h, double2* w, long long n,
                      ReduceScratch& rs, int norm_slot, cudaStream_t stream) {
  if (nv > kMaxDots) return cudaErrorInvalidValue;
  const int gx = reduce_blocks(n, 1);
  k_maxpy<double2><<<gx, kReduceThreads, 0, stream>>>(V, ldv, nv, h, w, n, norm_slot >= 0 ? rs.rpartial : nullptr);
  if (norm_slot >= 0) k_rfinal<<<1, kReduceThreads, 0, stream>>>(rs.rpartial, gx, rs.rresult + norm_slot);
  return cudaGetLastError();
}

cudaError_t maxpy_f32(const float2* V, long long ldv, int nv, const double2* h, float2* w, long long n,
                      ReduceScratch& rs, int norm_slot, cudaStream_t stream) {
  if (nv > kMaxDots) return cudaErrorInvalidValue;
  const int gx = reduce_blocks(n, 1);
  k_maxpy_f32<<<gx, kReduceThreads, 0, stream>>>(V, ldv, nv, h, w, n, norm_slot >= 0 ? rs.rpartial : nullptr);
  if (norm_slot >= 0) k_rfinal<<<1, kReduceThreads, 0, stream>>>(rs.rpartial, gx, rs.rresult + norm_slot);
  return cudaGetLastError();
}

cudaError_t norm2_f64(const double2* w, long long n, ReduceScratch& rs, int slot, cudaStream_t stream) {
  const int gx = reduce_blocks(n, 1);
  k_norm2<double2><<<gx, kReduceThreads, 0, stream>>>(w, n, rs.rpartial);
  k_rfinal<<<1, kReduceThreads, 0, stream>>>(rs.rpartial, gx, rs.rresult + slot);
  return cudaGetLastError();
}

cudaError_t norm2_f32(const float2* w, long long n, ReduceScratch& rs, int slot, cudaStream_t stream) {
  const int gx = reduce_blocks(n, 1);
  k_norm2_df<<<gx, kReduceThreads, 0, stream>>>(w, n, rs.rpartial);
  k_rfinal<<<1, kReduceThreads, 0, stream>>>(rs.rpartial, gx, rs.rresult + slot);
  return cudaGetLastError();
}

cudaError_t scale_f64(const double2* x, double2* y, long long n, double2 a, int accumulate, cudaStream_t stream) {
  k_scale_f64<<<grid_for(n), 256, 0, stream>>>(x, y, n, a, accumulate);
  return cudaGetLastError();
}

cudaError_t scale_f32(const float2* x, float2* y, long long n, double2 a, cudaStream_t stream) {
  k_scale_f32<<<grid_for(n), 256, 0, stream>>>(x, y, n, a);
  return cudaGetLastError();
}

cudaError_t combine_f64(const double2* V, long long ldv, int nv, const double2* c, double2* y, long long n,
                        int accumulate, cudaStream_t stream) {
  if (nv > kMaxDots) return cudaErrorInvalidValue;
  k_combine<double2><<<grid_for(n), kReduceThreads, 0, stream>>>(V, ldv, nv, c, y, n, accumulate);
  return cudaGetLastError();
}

cudaError_t combine_f32_to_f64(const float2* V, long long ldv, int nv, const double2* c, double2* y, long long n,
                               int accumulate, cudaStream_t stream) {
  if (nv > kMaxDots) return cudaErrorInvalidValue;
  k_combine<float2><<<grid_for(n), kReduceThreads, 0, stream>>>(V, ldv, nv, c, y, n, accumulate);
  return cudaGetLastError();
}

cudaError_t trace_dot(const DevicePlan& dp, const void* x, int is_f32, int coords, double2* out,
                      cudaStream_t stream) {
  if (is_f32)
    k_trace_dot<float2><<<1, 1024, 0, stream>>>(dp.sectors, dp.diag_sector, dp.diag_index, dp.ndiag,
                                                (const float2*)x, coords, out);
  else
    k_trace_dot<double2><<<1, 1024, 0, stream>>>(dp.sectors, dp.diag_sector, dp.diag_index, dp.ndiag,
                                                 (const double2*)x, coords, out);
  return cudaGetLastError();
}

cudaError_t x_to_z_f64(const DevicePlan& dp, const double2* x, double2* z, double scale, cudaStream_t stream) {
  dim3 grid(8, dp.nsectors);
  k_coords<double2, double2><<<grid, 256, 0, stream>>>(dp.sectors, dp.nsectors, x, z, scale, 1, 0);
  return cudaGetLastError();
}

cudaError_t z_to_x_f64(const DevicePlan& dp, const double2* z, double2* x, double scale, int accumulate,
                       cudaStream_t stream) {
  dim3 grid(8, dp.nsectors);
  k_coords<double2, double2><<<grid, 256, 0, stream>>>(dp.sectors, dp.nsectors, z, x, scale, 0, accumulate);
  return cudaGetLastError();
}

cudaError_t x_to_z_f32(const DevicePlan& dp, const double2* x, float2* z, double scale, cudaStream_t stream) {
  dim3 grid(8, dp.nsectors);
  k_coords<double2, float2><<<grid, 256, 0, stream>>>(dp.sectors, dp.nsectors, x, z, scale, 1, 0);
  return cudaGetLastError();
}

cudaError_t f64_to_f32(const double2* x, float2* y, long long n, double scale, cudaStream_t stream) {
  k_f64_to_f32<<<grid_for(n), 256, 0, stream>>>(x, y, n, scale);
  return cudaGetLastError();
}

cudaError_t weighted_norm2_z(const DevicePlan& dp, const double2* z, ReduceScratch& rs, int slot,
                             cudaStream_t stream) {
  if (dp.nsectors > kReduceBlocks) return cudaErrorInvalidValue;
  k_weighted_norm2_z<<<dp.nsectors, kReduceThreads, 0, stream>>>(dp.sectors, dp.nsectors, z, rs.rpartial);
  k_rfinal<<<1, kReduceThreads, 0, stream>>>(rs.rpartial, dp.nsectors, rs.rresult + slot);
  return cudaGetLastError();
}

}  // namespace picuda

// ---------------------------------------------------------------------------------------
// Allocation-free multi-dot.
//
// Some callers cannot allocate device memory at the time they need a reduction: a Julia
// package whose device memory is owned by its own pool (CUDA.jl) and must not see foreign
// cudaMalloc/cudaFree calls, a serving loop that forbids allocation after start-up so its
// memory budget cannot move, or code that enqueues work while a stream is being captured
// (cudaMalloc is not allowed inside a capture).  For them, pi_mdot_f64_noalloc computes
// h[i] = sum_e conj(V_i[e]) w[e] with its partial sums in a fixed device array that lives in
// this library image: kNoAllocBlocks x kNoAllocMaxDots complex doubles (128 KiB), held on
// every GPU that loads the library until the process exits.
// ---------------------------------------------------------------------------------------
namespace picuda {
namespace {

constexpr int kNoAllocBlocks = 256;
constexpr int kNoAllocMaxDots = 32;

static __device__ __align__(256) double2 g_noalloc_partials[kNoAllocBlocks * kNoAllocMaxDots];

// Same arithmetic as the plan-owned multi-dot, with the partial stride of the static array.
__global__ void __launch_bounds__(kReduceThreads)
    k_mdot_partial_noalloc(const double2* __restrict__ V, long long ldv, int nv, const double2* __restrict__ w,
                           long long n, double2* __restrict__ partial) {
  __shared__ double smem[32 * 2 * kDotGroup];
  long long beg, end;
  chunk_bounds(n, beg, end);
  const int g = blockIdx.y * kDotGroup;
  const int cnt = min(kDotGroup, nv - g);
  double acc[2 * kDotGroup];
#pragma unroll
  for (int k = 0; k < 2 * kDotGroup; ++k) acc[k] = 0.0;
  for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const double2 wv = w[e];
#pragma unroll
    for (int k = 0; k < kDotGroup; ++k) {
      if (k < cnt) {
        const double2 v = V[(long long)(g + k) * ldv + e];
        acc[2 * k] = fma(v.x, wv.x, acc[2 * k]);
        acc[2 * k] = fma(v.y, wv.y, acc[2 * k]);
        acc[2 * k + 1] = fma(v.x, wv.y, acc[2 * k + 1]);
        acc[2 * k + 1] = fma(-v.y, wv.x, acc[2 * k + 1]);
      }
    }
  }
  block_sum<2 * kDotGroup>(acc, smem);
  if (threadIdx.x == 0) {
    for (int k = 0; k < cnt; ++k)
      partial[(long long)blockIdx.x * kNoAllocMaxDots + g + k] = make_double2(acc[2 * k], acc[2 * k + 1]);
  }
}

__global__ void __launch_bounds__(kReduceThreads)
    k_mdot_final_noalloc(const double2* __restrict__ partial, int nblocks, double2* __restrict__ out) {
  __shared__ double smem[32 * 2];
  const int i = blockIdx.x;
  double acc[2] = {0, 0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double2 p = partial[(long long)b * kNoAllocMaxDots + i];
    acc[0] += p.x;
    acc[1] += p.y;
  }
  block_sum<2>(acc, smem);
  if (threadIdx.x == 0) out[i] = make_double2(acc[0], acc[1]);
}

}  // namespace

}  // namespace picuda

#include <string>

#include "../../include/picuda.h"

namespace picuda {
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace picuda

extern "C" int pi_mdot_f64_noalloc(const double* V_dev, long long ldv, int nv, const double* w_dev, long long n,
                                   double* h_dev, void* stream) {
  using namespace picuda;
  if (!V_dev || !w_dev || !h_dev) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (nv < 1 || nv > kNoAllocMaxDots)
    return fail(PI_ERR_INVALID_ARGUMENT,
                "nv must lie in 1:32, the capacity of the static scratch of pi_mdot_f64_noalloc");
  if (n < 1 || ldv < n) return fail(PI_ERR_DIMENSION, "need n >= 1 and ldv >= n");
  // An error left pending by earlier, unrelated work is reported as such (and left in place
  // for its owner) rather than mistaken for a failure of the launches below.
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess)
    return fail(PI_ERR_CUDA, std::string("a CUDA error was pending before pi_mdot_f64_noalloc: ") +
                                 cudaGetErrorString(e));
  // The host-side symbol is only a stand-in: the array's device address on the current device
  // is looked up on every call (a host-side table lookup once the module is loaded), so a
  // device reset that loads the module again never leaves a stale address behind.
  void* scratch_addr = nullptr;
  e = cudaGetSymbolAddress(&scratch_addr, g_noalloc_partials);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the static scratch");
  double2* scratch = (double2*)scratch_addr;
  const int gy = (nv + kDotGroup - 1) / kDotGroup;
  long long gx = (n + 4LL * kReduceThreads - 1) / (4LL * kReduceThreads);
  gx = std::max(1LL, std::min(gx, (long long)(kNoAllocBlocks / gy)));
  cudaStream_t s = (cudaStream_t)stream;
  // Every partial that the final pass reads is written by the first pass of the same call,
  // so nothing needs clearing; two calls that overlap on the GPU share the array and race.
  k_mdot_partial_noalloc<<<dim3((unsigned)gx, gy), kReduceThreads, 0, s>>>(
      (const double2*)V_dev, ldv, nv, (const double2*)w_dev, n, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "pi_mdot_f64_noalloc partial-sum launch");
  k_mdot_final_noalloc<<<nv, kReduceThreads, 0, s>>>(scratch, (int)gx, (double2*)h_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "pi_mdot_f64_noalloc final-sum launch");
  return PI_OK;
}
