// Arnoldi factorisation of the Liouvillian for spectra (krylov_liouvillian_spectrum,
// krylov.jl:914-962) and basis combinations for Ritz vectors.
//
// The reference runs one Krylov process of at most m steps with two Gram-Schmidt passes
// per step and hands the projected Hessenberg matrix to LAPACK.  Here every O(dim) step
// runs on the device (fused apply, multi-dot and multi-axpy over the resident basis, norms
// in FP64 with deterministic two-stage reductions) and the host reads back one Hessenberg
// column per step; the small eigenproblem stays with the caller, as in the reference.  The
// two passes are classical Gram-Schmidt (one multi-dot then one multi-axpy each), whose
// orthogonality matches the reference's twice-repeated modified Gram-Schmidt.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "../../include/picuda.h"
#include "pi_handle.hpp"

using namespace picuda;

namespace {

struct Sync {
  pi_plan* p;
  cudaError_t err = cudaSuccess;
  void chk(cudaError_t e) {
    if (e != cudaSuccess && err == cudaSuccess) err = e;
  }
};

}  // namespace

extern "C" {

int pi_arnoldi(pi_plan* plan, const double* v0_dev, int m, double* V_dev, long long ldv, double* H_host,
               pi_arnoldi_info_t* info) {
  if (!plan || !v0_dev || !V_dev || !H_host) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  const long long n = plan->host.dim;
  if (m < 1 || m >= kMaxDots) return fail(PI_ERR_INVALID_ARGUMENT, "krylov dimension must lie in 1..127");
  if (ldv < n) return fail(PI_ERR_INVALID_ARGUMENT, "ldv must be at least the PI dimension");
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  const int ldh = m + 1;
  std::memset(H_host, 0, sizeof(double) * 2 * (size_t)ldh * m);
  cudaStream_t s = plan->stream;
  ReduceScratch& rs = plan->rs;
  double* hp = plan->host_pinned;
  double2* V = reinterpret_cast<double2*>(V_dev);
  auto col = [&](int j) { return V + (size_t)j * (size_t)ldv; };
  Sync z{plan};
  // h1, h2 (kMaxDots complex each) sit in rs.result after the reduction scratch
  double2* h1 = nullptr;
  double2* h2 = nullptr;
  z.chk(cudaMallocAsync((void**)&h1, sizeof(double2) * 2 * kMaxDots, s));
  if (z.err != cudaSuccess) return cuda_fail(z.err, "Arnoldi workspace");
  h2 = h1 + kMaxDots;
  auto fetch = [&](const void* dev, size_t bytes) {
    z.chk(cudaMemcpyAsync(hp, dev, bytes, cudaMemcpyDeviceToHost, s));
    z.chk(cudaStreamSynchronize(s));
  };
  pi_arnoldi_info_t out;
  std::memset(&out, 0, sizeof(out));
  int rc = PI_OK;
  // V[:,0] = v0 / |v0|
  z.chk(norm2_f64(reinterpret_cast<const double2*>(v0_dev), n, rs, 0, s));
  fetch(rs.rresult, sizeof(double));
  const double nq = z.err == cudaSuccess ? std::sqrt(hp[0]) : 0.0;
  if (z.err == cudaSuccess && !(nq > 0.0 && std::isfinite(nq))) rc = fail(PI_ERR_INVALID_ARGUMENT, "initial_vector must be nonzero");
  if (rc == PI_OK) z.chk(scale_f64(reinterpret_cast<const double2*>(v0_dev), col(0), n, make_double2(1.0 / nq, 0.0), 0, s));
  const double breakfactor = std::numeric_limits<double>::epsilon();
  const BorderArgs none{1.0, nullptr, 0};
  for (int j = 0; j < m && rc == PI_OK && z.err == cudaSuccess; ++j) {
    double2* w = col(j + 1);
    z.chk(launch_apply_f64(plan->dev, reinterpret_cast<const double*>(col(j)), reinterpret_cast<double*>(w), 1, n,
                           none, s));
    ++out.operator_applications;
    z.chk(norm2_f64(w, n, rs, 0, s));  // image norm
    const int nv = j + 1;
    z.chk(mdot_f64(V, ldv, nv, w, n, rs, h1, s));
    z.chk(maxpy_f64(V, ldv, nv, h1, w, n, rs, -1, s));
    z.chk(mdot_f64(V, ldv, nv, w, n, rs, h2, s));
    z.chk(maxpy_f64(V, ldv, nv, h2, w, n, rs, 1, s));  // |w|^2 after the second pass
    z.chk(cudaMemcpyAsync(hp, h1, sizeof(double2) * 2 * kMaxDots, cudaMemcpyDeviceToHost, s));
    z.chk(cudaMemcpyAsync(hp + 4 * kMaxDots, rs.rresult, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    z.chk(cudaStreamSynchronize(s));
    if (z.err != cudaSuccess) break;
    const double image_norm = std::sqrt(hp[4 * kMaxDots]);
    const double wn = std::sqrt(hp[4 * kMaxDots + 1]);
    double* Hc = H_host + 2 * (size_t)ldh * j;
    for (int i = 0; i < nv; ++i) {
      Hc[2 * i] = hp[2 * i] + hp[2 * (kMaxDots + i)];
      Hc[2 * i + 1] = hp[2 * i + 1] + hp[2 * (kMaxDots + i) + 1];
    }
    Hc[2 * (j + 1)] = wn;
    out.steps = j + 1;
    if (!std::isfinite(wn) || !std::isfinite(image_norm)) {
      rc = fail(PI_ERR_INVALID_ARGUMENT, "non-finite value in the Arnoldi process");
      break;
    }
    if (j == m - 1) break;
    if (wn <= breakfactor * std::max(image_norm, std::numeric_limits<double>::min())) {
      out.breakdown = 1;
      break;
    }
    z.chk(scale_f64(w, w, n, make_double2(1.0 / wn, 0.0), 0, s));
  }
  z.chk(cudaFreeAsync(h1, s));
  z.chk(cudaStreamSynchronize(s));
  if (info) *info = out;
  if (rc != PI_OK) return rc;
  if (z.err != cudaSuccess) return cuda_fail(z.err, "Arnoldi process");
  return PI_OK;
}

int pi_combine_f64(pi_plan* plan, const double* V_dev, long long ldv, int k, const double* coef_host, int ncols,
                   double* out_dev, long long ldo) {
  if (!plan || !V_dev || !coef_host || !out_dev) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  const long long n = plan->host.dim;
  if (k < 1 || k > kMaxDots || ncols < 0) return fail(PI_ERR_INVALID_ARGUMENT, "k must lie in 1..128");
  if (ldv < n || ldo < n) return fail(PI_ERR_INVALID_ARGUMENT, "leading dimensions must be at least the PI dimension");
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  if (ncols == 0) return PI_OK;
  cudaStream_t s = plan->stream;
  double2* c = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&c, sizeof(double2) * (size_t)k * ncols, s);
  if (e != cudaSuccess) return cuda_fail(e, "combine workspace");
  Sync z{plan};
  z.chk(cudaMemcpyAsync(c, coef_host, sizeof(double2) * (size_t)k * ncols, cudaMemcpyHostToDevice, s));
  for (int j = 0; j < ncols; ++j)
    z.chk(combine_f64(reinterpret_cast<const double2*>(V_dev), ldv, k, c + (size_t)j * k,
                      reinterpret_cast<double2*>(out_dev) + (size_t)j * ldo, n, 0, s));
  z.chk(cudaFreeAsync(c, s));
  z.chk(cudaStreamSynchronize(s));
  if (z.err != cudaSuccess) return cuda_fail(z.err, "basis combination");
  return PI_OK;
}

}  // extern "C"
