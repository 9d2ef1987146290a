// Fixed-step RK4 evolution on the device: evolve! (evolution.jl:75-118) and the default
// solve_dynamics algorithm (highlevel.jl:559-566, 623-631, 693-733).
//
// The reference runs, per step, four operator actions and six whole-vector broadcasts over
// three scratch vectors (k1, the stage sum k2, tmp).  Here each stage is ONE launch: the
// stencil apply of that stage (the same tile code as the single-column apply) with the
// stage's vector updates as its epilogue, so the stage derivative never goes to memory:
//
//   stage 0:  acc  = k;          t_B = dest + (h/2) k      (k = L dest)
//   stage 1:  acc += 2k;         t_A = dest + (h/2) k      (k = L t_B)
//   stage 2:  acc += 2k;         t_B = dest + h k          (k = L t_A)
//   stage 3:  dest += (h/6)(acc + k)                       (k = L t_B)
//
// Every stage reads its stencil input from one buffer and writes the next stage's input to
// the other (t_A / t_B ping-pong), so no block reads an entry that another block of the
// same launch writes.  The step size lives in device memory, so the graph of one
// interval's steps is built once per call and replayed for every saved interval.
//
// FP64 form: reference coordinates, everything complex FP64; stage 0 reads dest itself.
// Mixed form (PI_FP32): population coordinates z = sqrt(f) x.  The state is a double-float
// pair (dest_hi + dest_lo, two FP32 planes, ~48-bit significand) and stage 3 adds its
// increment with error-free FP32 transformations (two-sum, FMA two-product), so the state
// keeps FP64-class accuracy while every stage runs on the FP32 pipes: GB300 issues FP64 at
// a small fraction of its FP32 rate, and an FP64 epilogue cost more than the FP32 stencil.
// The applies, the stage sum and the stage inputs are FP32 (their rounding is the FP32
// apply's own), and stage 0 reads dest_hi as its FP32 stencil input.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/picuda.h"
#include "pi_apply_impl.cuh"
#include "pi_handle.hpp"

namespace picuda {
namespace {

struct Rk4Params {
  const DevSector* sectors;
  const DevTerm* terms;
  const void* coef;
  const DevTile* tiles;
  void* dest;      // state: double2 (FP64) or float2 dest_hi (mixed)
  float2* dlo;     // mixed: dest_lo
  void* acc;       // stage sum k1 + 2k2 + 2k3 + k4: double2 (FP64) or float2 (mixed)
  void* ta;        // stage inputs: double2 (FP64) or float2 (mixed)
  void* tb;
  const double* h; // step size (device)
  SplitPlanes planes;  // mixed, canonical plan: merged population-coordinate coefficients
};

// Epilogue of one FP64 RK4 stage for output entry e with stage derivative k = (L input)[e].
template <int STAGE>
struct Rk4Sink64 {
  double2* __restrict__ dest;
  double2* __restrict__ acc;
  double2* __restrict__ next;
  double h;
  __device__ __forceinline__ void operator()(long long e, double2 k) const {
    const double2 d = dest[e];
    if (STAGE == 0) {
      acc[e] = k;
      next[e] = make_double2(d.x + (h / 2) * k.x, d.y + (h / 2) * k.y);
    } else if (STAGE == 1 || STAGE == 2) {
      const double2 a = acc[e];
      acc[e] = make_double2(a.x + 2 * k.x, a.y + 2 * k.y);
      const double c = STAGE == 1 ? h / 2 : h;
      next[e] = make_double2(d.x + c * k.x, d.y + c * k.y);
    } else {
      const double2 a = acc[e];
      const double sr = a.x + k.x, si = a.y + k.y;
      dest[e] = make_double2(d.x + (h / 6) * sr, d.y + (h / 6) * si);
    }
  }
};

// Double-float helpers (Dekker / Knuth error-free transformations on the FP32 pipes).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& err) {
  s = a + b;
  const float bb = s - a;
  err = (a - (s - bb)) + (b - bb);
}
// (hi, lo) + c * v with c = c_hi + c_lo, v a float: the two-product of c_hi * v is exact
__device__ __forceinline__ void df_add_scaled(float& hi, float& lo, float c_hi, float c_lo, float v) {
  const float p = c_hi * v;
  const float pe = fmaf(c_hi, v, -p) + c_lo * v;
  float s, e;
  two_sum(hi, p, s, e);
  e += lo + pe;
  hi = s + e;
  lo = e - (hi - s);
}

// Epilogue of one mixed RK4 stage: FP32 stage arithmetic, double-float state update.
template <int STAGE>
struct Rk4SinkDF {
  float2* __restrict__ dhi;
  float2* __restrict__ dlo;
  float2* __restrict__ acc;
  float2* __restrict__ next;
  float c;             // h/2 (stages 0, 1) or h (stage 2)
  float c6_hi, c6_lo;  // h/6 as a double-float
  __device__ __forceinline__ void operator()(long long e, float2 k) const {
    const float2 d = dhi[e];
    if (STAGE == 0) {
      acc[e] = k;
      next[e] = make_float2(fmaf(c, k.x, d.x), fmaf(c, k.y, d.y));
    } else if (STAGE == 1 || STAGE == 2) {
      const float2 a = acc[e];
      acc[e] = make_float2(fmaf(2.0f, k.x, a.x), fmaf(2.0f, k.y, a.y));
      next[e] = make_float2(fmaf(c, k.x, d.x), fmaf(c, k.y, d.y));
    } else {
      const float2 a = acc[e];
      float2 l = dlo[e];
      float2 hnew = d;
      df_add_scaled(hnew.x, l.x, c6_hi, c6_lo, a.x + k.x);
      df_add_scaled(hnew.y, l.y, c6_hi, c6_lo, a.y + k.y);
      dhi[e] = hnew;
      dlo[e] = l;
    }
  }
};

template <int STAGE>
__global__ void __launch_bounds__(kApplyThreads) k_rk4_stage64(Rk4Params p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* win = reinterpret_cast<double2*>(smem_raw);  // [3][kWinElems] source windows
  __shared__ int4 st[kMaxSectorTerms];
  __shared__ int ge[G_COUNT + 1];
  const double2* x = STAGE == 0 ? (const double2*)p.dest : (const double2*)(STAGE == 2 ? p.ta : p.tb);
  double2* next = (double2*)(STAGE == 1 ? p.ta : p.tb);
  const Rk4Sink64<STAGE> sink{(double2*)p.dest, (double2*)p.acc, next, *p.h};
  const BorderArgs none{1.0, nullptr, 0};
  apply_tile_to<double>(p.sectors, p.terms, (const double2*)p.coef, p.tiles[blockIdx.x], x, sink, none, nullptr,
                        win, st, ge);
}

template <int STAGE>
__global__ void __launch_bounds__(kApplyThreads) k_rk4_stage_mixed(Rk4Params p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* win = reinterpret_cast<float2*>(smem_raw);  // [3][kWinElems] source windows
  __shared__ int4 st[kMaxSectorTerms];
  __shared__ int ge[G_COUNT + 1];
  const float2* x = STAGE == 0 ? (const float2*)p.dest : (const float2*)(STAGE == 2 ? p.ta : p.tb);
  float2* next = (float2*)(STAGE == 1 ? p.ta : p.tb);
  const double h = *p.h;  // FP64 once per thread
  const double h6 = h / 6;
  const float c6_hi = (float)h6;
  const Rk4SinkDF<STAGE> sink{(float2*)p.dest, p.dlo, (float2*)p.acc, next, (float)(STAGE == 2 ? h : h / 2), c6_hi,
                              (float)(h6 - (double)c6_hi)};
  const BorderArgs none{1.0, nullptr, 1};
  // The RK4 stages keep the entry plane: the separable line planes (the batched engine's
  // choice) measured 4% slower here, where one N=120 stage is 0.71 of a wave.
  if (p.planes.eplane != nullptr) {  // merged coefficients: ten staged reads per entry
    if (p.planes.plus)
      apply_tile_planes_to<true>(p.sectors, p.tiles[blockIdx.x], x, sink, none, nullptr, p.planes, win);
    else
      apply_tile_planes_to<false>(p.sectors, p.tiles[blockIdx.x], x, sink, none, nullptr, p.planes, win);
    return;
  }
  apply_tile_to<float>(p.sectors, p.terms, (const float2*)p.coef, p.tiles[blockIdx.x], x, sink, none, nullptr, win,
                       st, ge);
}

// z (FP64) -> (hi, lo) FP32 planes, and back.
__global__ void k_df_split(const double2* __restrict__ z, float2* __restrict__ hi, float2* __restrict__ lo,
                           long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 v = z[i];
    const float2 h = make_float2((float)v.x, (float)v.y);
    hi[i] = h;
    lo[i] = make_float2((float)(v.x - (double)h.x), (float)(v.y - (double)h.y));
  }
}
__global__ void k_df_merge(const float2* __restrict__ hi, const float2* __restrict__ lo, double2* __restrict__ z,
                           long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 h = hi[i], l = lo[i];
    z[i] = make_double2((double)h.x + (double)l.x, (double)h.y + (double)l.y);
  }
}
unsigned elem_grid(long long n) { return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16)); }

using StageKernel = void (*)(Rk4Params);

cudaError_t stage_kernels(bool mixed, StageKernel (&k)[4]) {
  if (mixed) {
    k[0] = k_rk4_stage_mixed<0>;
    k[1] = k_rk4_stage_mixed<1>;
    k[2] = k_rk4_stage_mixed<2>;
    k[3] = k_rk4_stage_mixed<3>;
  } else {
    k[0] = k_rk4_stage64<0>;
    k[1] = k_rk4_stage64<1>;
    k[2] = k_rk4_stage64<2>;
    k[3] = k_rk4_stage64<3>;
  }
  static bool configured[2] = {false, false};  // host side
  if (!configured[mixed]) {
    const int smem = (int)(3 * kWinElems * (mixed ? sizeof(float2) : sizeof(double2)));
    for (int s = 0; s < 4; ++s) {
      cudaError_t e = cudaFuncSetAttribute(k[s], cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e != cudaSuccess) return e;
    }
    configured[mixed] = true;
  }
  return cudaSuccess;
}

// A CUDA graph of `steps` RK4 steps (4 * steps kernel nodes in one chain).
struct StepGraph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~StepGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (g) cudaGraphDestroy(g);
  }
  cudaError_t build(const StageKernel (&k)[4], const Rk4Params& prm, int ntiles, size_t smem, int steps) {
    cudaError_t e = cudaGraphCreate(&g, 0);
    cudaGraphNode_t prev = nullptr;
    Rk4Params arg = prm;
    void* args[] = {&arg};
    for (int s = 0; s < steps && e == cudaSuccess; ++s)
      for (int stage = 0; stage < 4 && e == cudaSuccess; ++stage) {
        cudaKernelNodeParams kp{};
        kp.func = (void*)k[stage];
        kp.gridDim = dim3((unsigned)ntiles);
        kp.blockDim = dim3(kApplyThreads);
        kp.sharedMemBytes = (unsigned)smem;
        kp.kernelParams = args;
        cudaGraphNode_t node;
        e = cudaGraphAddKernelNode(&node, g, prev ? &prev : nullptr, prev ? 1 : 0, &kp);
        prev = node;
      }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    return e;
  }
};

struct DevBufs {
  cudaStream_t s;
  std::vector<void*> ptrs;
  cudaError_t err = cudaSuccess;
  explicit DevBufs(cudaStream_t stream) : s(stream) {}
  void* get(size_t bytes) {
    void* p = nullptr;
    if (err != cudaSuccess) return nullptr;
    err = cudaMallocAsync(&p, bytes ? bytes : 16, s);
    if (err != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return p;
  }
  ~DevBufs() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
    cudaStreamSynchronize(s);
  }
};

// RK4 over the intervals of `times`; state in rho (device, reference coordinates, in place).
// skip_equal: zero-length intervals take no steps (solve_dynamics); evolve! always steps.
int rk4_run(pi_plan* plan, double2* rho, int nt, const double* times, int steps, bool mixed, bool skip_equal,
            int nobs, const double2* obs, double* values_host, pi_rk4_info_t* info) {
  const DevicePlan& dp = plan->dev;
  const long long n = plan->host.dim;
  cudaStream_t s = plan->stream;
  pi_rk4_info_t out;
  std::memset(&out, 0, sizeof(out));
  out.reached_time = times[0];
  cudaError_t err = cudaSuccess;
  auto chk = [&](cudaError_t e) {
    if (e != cudaSuccess && err == cudaSuccess) err = e;
  };
  {
    DevBufs B(s);
    const size_t es = mixed ? sizeof(float2) : sizeof(double2);
    // mixed: dest = dest_hi (float2) plus dest_lo; FP64 evolves rho in place
    void* dest = mixed ? B.get(sizeof(float2) * n) : (void*)rho;
    float2* dlo = mixed ? (float2*)B.get(sizeof(float2) * n) : nullptr;
    double2* zbuf = mixed ? (double2*)B.get(sizeof(double2) * n) : nullptr;  // FP64 z for conversions
    void* acc = B.get(es * n);
    void* ta = B.get(es * n);
    void* tb = B.get(es * n);
    double* hdev = (double*)B.get(sizeof(double) * std::max(nt, 1));
    double* hcur = (double*)B.get(sizeof(double));
    double2* vals = nobs ? (double2*)B.get(sizeof(double2) * (size_t)nt * nobs) : nullptr;
    double2* obsz = (mixed && nobs) ? (double2*)B.get(sizeof(double2) * (size_t)nobs * n) : nullptr;
    if (B.err != cudaSuccess) return cuda_fail(B.err, "RK4 workspace");
    std::vector<double> hs(std::max(nt, 1), 0.0);
    for (int it = 1; it < nt; ++it) hs[it] = (times[it] - times[it - 1]) / steps;
    chk(cudaMemcpyAsync(hdev, hs.data(), sizeof(double) * hs.size(), cudaMemcpyHostToDevice, s));
    const double2* obs_in = obs;
    const double2* state64 = rho;  // FP64 view of the state for observables
    if (mixed) {
      chk(x_to_z_f64(dp, rho, zbuf, 1.0, s));
      k_df_split<<<elem_grid(n), 256, 0, s>>>(zbuf, (float2*)dest, dlo, n);
      chk(cudaGetLastError());
      // dot(op, x) = dot(op / sqrt(f), z): the observables move to population coordinates once
      for (int o = 0; o < nobs; ++o) chk(z_to_x_f64(dp, obs + (size_t)o * n, obsz + (size_t)o * n, 1.0, 0, s));
      if (nobs) obs_in = obsz;
      state64 = zbuf;
    }
    auto record = [&](int it) {
      // dot(op.data, rho.data) for every observable (highlevel.jl:672-677)
      if (!nobs) return;
      if (mixed && it > 0) {
        k_df_merge<<<elem_grid(n), 256, 0, s>>>((const float2*)dest, dlo, zbuf, n);
        chk(cudaGetLastError());
      }
      chk(mdot_f64(obs_in, n, nobs, state64, n, plan->rs, vals + (size_t)it * nobs, s));
    };
    record(0);
    StageKernel k[4];
    chk(stage_kernels(mixed, k));
    const int gsteps = steps <= 128 ? steps : 64;
    const int reps = steps / gsteps, rem = steps % gsteps;
    StepGraph main, tail;
    // Only the step size changes between intervals: the graphs read it from hcur.
    SplitPlanes planes{nullptr, nullptr, nullptr, nullptr, 0};
    if (mixed && dp.canon && em_split_planes(plan, 1, &planes) != PI_OK)
      planes = SplitPlanes{nullptr, nullptr, nullptr, nullptr, 0};
    const Rk4Params prm{dp.sectors, dp.terms, mixed ? (const void*)dp.coef32z : (const void*)dp.coef64, dp.tiles,
                        dest, dlo, acc, ta, tb, hcur, planes};
    const size_t smem = 3 * kWinElems * es;
    if (err == cudaSuccess && dp.ntiles > 0) {
      chk(main.build(k, prm, dp.ntiles, smem, gsteps));
      if (rem) chk(tail.build(k, prm, dp.ntiles, smem, rem));
    }
    for (int it = 1; it < nt && err == cudaSuccess; ++it) {
      if (!(skip_equal && times[it] == times[it - 1]) && dp.ntiles > 0) {
        chk(cudaMemcpyAsync(hcur, hdev + it, sizeof(double), cudaMemcpyDeviceToDevice, s));
        for (int r = 0; r < reps; ++r) chk(cudaGraphLaunch(main.exec, s));
        if (rem) chk(cudaGraphLaunch(tail.exec, s));
        out.steps += steps;
        out.operator_applications += 4LL * steps;
      }
      out.reached_time = times[it];
      record(it);
    }
    if (mixed) {
      k_df_merge<<<elem_grid(n), 256, 0, s>>>((const float2*)dest, dlo, zbuf, n);
      chk(cudaGetLastError());
      chk(z_to_x_f64(dp, zbuf, rho, 1.0, 0, s));
    }
    chk(cudaStreamSynchronize(s));
    if (err == cudaSuccess && nobs)
      chk(cudaMemcpy(values_host, vals, sizeof(double2) * (size_t)nt * nobs, cudaMemcpyDeviceToHost));
  }
  if (info) *info = out;
  if (err != cudaSuccess) return cuda_fail(err, "RK4 evolution");
  return PI_OK;
}

int check_rk4_opts(const pi_rk4_opts_t* opts) {
  if (!opts) return fail(PI_ERR_INVALID_ARGUMENT, "null options");
  if (opts->steps_per_interval <= 0) return fail(PI_ERR_INVALID_ARGUMENT, "steps must be positive");
  if (opts->precision != PI_FP64 && opts->precision != PI_FP32)
    return fail(PI_ERR_INVALID_ARGUMENT, "precision must be PI_FP64 or PI_FP32");
  return PI_OK;
}

}  // namespace
}  // namespace picuda

using namespace picuda;

extern "C" {

void pi_rk4_default_opts(pi_rk4_opts_t* opts) {
  if (!opts) return;
  opts->steps_per_interval = 64;
  opts->precision = PI_FP64;
}

int pi_evolve(pi_plan* plan, double* dest_dev, const double* src_dev, double t0, double t1,
              const pi_rk4_opts_t* opts, pi_rk4_info_t* info) {
  if (!plan || !dest_dev || !src_dev) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  int rc = check_rk4_opts(opts);
  if (rc) return rc;
  if (!std::isfinite(t0) || !std::isfinite(t1)) return fail(PI_ERR_INVALID_ARGUMENT, "tspan must be finite");
  const size_t bytes = sizeof(double2) * (size_t)plan->host.dim;
  const char* d = (const char*)dest_dev;
  const char* s = (const char*)src_dev;
  if (d != s && d < s + bytes && s < d + bytes)
    return fail(PI_ERR_INVALID_ARGUMENT,
                "evolution permits exact in-place use but not partially overlapping source and destination storage");
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  if (d != s) {
    cudaError_t e = cudaMemcpyAsync(dest_dev, src_dev, bytes, cudaMemcpyDeviceToDevice, plan->stream);
    if (e != cudaSuccess) return cuda_fail(e, "evolve copy");
  }
  const double times[2] = {t0, t1};
  return rk4_run(plan, (double2*)dest_dev, 2, times, opts->steps_per_interval, opts->precision == PI_FP32, false, 0,
                 nullptr, nullptr, info);
}

int pi_solve_dynamics_rk4(pi_plan* plan, double* rho_dev, int nt, const double* times, int nobs,
                          const double* obs_dev, double* values_host, const pi_rk4_opts_t* opts,
                          pi_rk4_info_t* info) {
  if (!plan || !rho_dev || !times || nt < 1) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (nobs < 0 || nobs > kMaxDots || (nobs > 0 && (!obs_dev || !values_host)))
    return fail(PI_ERR_INVALID_ARGUMENT, "observables must number 0..128 with device data and a host output");
  int rc = check_rk4_opts(opts);
  if (rc) return rc;
  if (!std::isfinite(times[0])) return fail(PI_ERR_INVALID_ARGUMENT, "saved times must be finite");
  for (int i = 1; i < nt; ++i)
    if (!(times[i] >= times[i - 1]) || !std::isfinite(times[i]))
      return fail(PI_ERR_INVALID_ARGUMENT, "saveat times must be nondecreasing");
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  return rk4_run(plan, (double2*)rho_dev, nt, times, opts->steps_per_interval, opts->precision == PI_FP32, true, nobs,
                 (const double2*)obs_dev, values_host, info);
}

}  // extern "C"
