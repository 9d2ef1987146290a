// Adaptive restarted-Arnoldi exponential action (krylov_extensions.jl:1346-1573) and the
// expv dynamics loop with streamed observables (highlevel.jl:467-528, 665-733).
//
// The host keeps the reference's step controller verbatim (local tolerance, accept/reject,
// step factor clamps, near-breakdown enlargement, rejected trials reusing the
// factorization); the Arnoldi process, CGS2, norms and the trial combination run on the
// device.  PI_FP32 runs the Arnoldi process in population coordinates z = sqrt(f) x with
// FP32 applies and an FP32 basis; Hessenberg entries, norms, the trial state and the
// controller stay FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>

#include "../../include/picuda.h"
#include "pi_batch.hpp"
#include "pi_dense.hpp"
#include "pi_handle.hpp"

namespace picuda {
namespace {

struct Bufs {
  cudaStream_t s = nullptr;
  std::vector<void*> ptrs;
  cudaError_t err = cudaSuccess;
  void* get(size_t bytes) {
    void* p = nullptr;
    if (err != cudaSuccess) return nullptr;
    err = cudaMallocAsync(&p, bytes ? bytes : 16, s);
    if (err != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return p;
  }
  ~Bufs() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
    cudaStreamSynchronize(s);
  }
};

struct NonFinite {
  const char* what;
};

// Device state of one exponential-action workspace (KrylovExpvWorkspace,
// krylov_extensions.jl:1312-1327): basis V (m+1 columns), image w, current and trial
// states.  `mixed` selects FP32 basis/image in population coordinates.
struct ExpvWork {
  pi_plan* p;
  cudaStream_t s;
  long long n;
  int m;
  bool mixed;
  cudaError_t err = cudaSuccess;
  void* V = nullptr;   // double2 or float2
  void* w = nullptr;
  double2* cur = nullptr;
  double2* trial = nullptr;
  double2* h1 = nullptr;
  double2* h2 = nullptr;
  double2* coef = nullptr;
  int applications = 0;

  void chk(cudaError_t e) {
    if (e != cudaSuccess && err == cudaSuccess) err = e;
  }
  bool ok() const { return err == cudaSuccess; }
  void fetch(void* out, const void* dev, size_t bytes) {
    if (!ok()) return;
    chk(cudaMemcpyAsync(p->host_pinned, dev, bytes, cudaMemcpyDeviceToHost, s));
    chk(cudaStreamSynchronize(s));
    if (ok()) std::memcpy(out, p->host_pinned, bytes);
  }
  double rresult() {
    double v = 0.0;
    fetch(&v, p->rs.rresult, sizeof(double));
    return v;
  }
  double norm64(const double2* x) {
    chk(norm2_f64(x, n, p->rs, 0, s));
    return std::sqrt(rresult());
  }
  double checked(double v, const char* what) {
    if (!std::isfinite(v)) throw NonFinite{what};
    return v;
  }
  size_t esz() const { return mixed ? sizeof(float2) : sizeof(double2); }
  void* col(int j) const { return (char*)V + (size_t)j * (size_t)n * esz(); }
  // w = L V_j; |w|^2 goes to rresult[1] and is read back with the next orthogonalization
  void apply_col(int j) {
    BorderArgs b{1.0, nullptr, mixed ? 1 : 0};
    if (mixed) {
      chk(launch_apply_f32(p->dev, (const float*)col(j), (float*)w, 1, n, b, s));
      chk(norm2_f32((const float2*)w, n, p->rs, 1, s));
    } else {
      chk(launch_apply_f64(p->dev, (const double*)col(j), (double*)w, 1, n, b, s));
      chk(norm2_f64((const double2*)w, n, p->rs, 1, s));
    }
    ++applications;
  }
  // CGS2 of w against V[0..nv): column += h1 + h2; returns |w| after and sets *image to
  // the norm recorded by apply_col.  One synchronization.
  double orthogonalize(int nv, std::vector<cd>& colv, double* image) {
    if (mixed) {
      chk(mdot_f32((const float2*)V, n, nv, (const float2*)w, n, p->rs, h1, s));
      chk(maxpy_f32((const float2*)V, n, nv, h1, (float2*)w, n, p->rs, -1, s));
      chk(mdot_f32((const float2*)V, n, nv, (const float2*)w, n, p->rs, h2, s));
      chk(maxpy_f32((const float2*)V, n, nv, h2, (float2*)w, n, p->rs, 0, s));
    } else {
      chk(mdot_f64((const double2*)V, n, nv, (const double2*)w, n, p->rs, h1, s));
      chk(maxpy_f64((const double2*)V, n, nv, h1, (double2*)w, n, p->rs, -1, s));
      chk(mdot_f64((const double2*)V, n, nv, (const double2*)w, n, p->rs, h2, s));
      chk(maxpy_f64((const double2*)V, n, nv, h2, (double2*)w, n, p->rs, 0, s));
    }
    double* hp = p->host_pinned;
    chk(cudaMemcpyAsync(hp, h1, sizeof(double2) * (kMaxDots + nv), cudaMemcpyDeviceToHost, s));
    chk(cudaMemcpyAsync(hp + 4 * kMaxDots, p->rs.rresult, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    chk(cudaStreamSynchronize(s));
    if (!ok()) return 0.0;
    for (int i = 0; i < nv; ++i)
      colv[i] += cd(hp[2 * i], hp[2 * i + 1]) + cd(hp[2 * (kMaxDots + i)], hp[2 * (kMaxDots + i) + 1]);
    if (image) *image = std::sqrt(hp[4 * kMaxDots + 1]);
    return std::sqrt(hp[4 * kMaxDots]);
  }
  // V_j = src / scale (src is w or, for j = 0, the FP64 current state)
  void set_col_from_w(int j, double scale) {
    if (mixed)
      chk(scale_f32((const float2*)w, (float2*)col(j), n, make_double2(1.0 / scale, 0.0), s));
    else
      chk(scale_f64((const double2*)w, (double2*)col(j), n, make_double2(1.0 / scale, 0.0), 0, s));
  }
  void set_col0_from_current(double beta) {
    if (mixed)
      chk(f64_to_f32(cur, (float2*)col(0), n, 1.0 / beta, s));
    else
      chk(scale_f64(cur, (double2*)col(0), n, make_double2(1.0 / beta, 0.0), 0, s));
  }
  // trial = sum_i c_i V_i, FP64 accumulation
  void combine(int cc) {
    if (mixed)
      chk(combine_f32_to_f64((const float2*)V, n, cc, coef, trial, n, 0, s));
    else
      chk(combine_f64((const double2*)V, n, cc, coef, trial, n, 0, s));
  }
};

struct Factorization {
  double beta = 0;
  bool zero_state = false;
  int k = 0, used = 0;
  bool completed = false, enlarged = false;
  int q = 0, coeff_count = 0;
  double next_remainder = 0;
  CMat S;
};

// _expv_arnoldi_factorization! (krylov_extensions.jl:1346-1401).
Factorization arnoldi(ExpvWork& W) {
  Factorization f;
  f.beta = W.checked(W.norm64(W.cur), "exponential-action state");
  if (f.beta == 0.0) {
    f.zero_state = true;
    f.completed = true;
    return f;
  }
  const int m = W.m;
  std::vector<std::vector<cd>> H(m, std::vector<cd>(m + 1, cd(0, 0)));  // columns
  W.set_col0_from_current(f.beta);
  int k = 0;
  bool exact = false, near = false;
  const double breakfactor = std::sqrt(std::numeric_limits<double>::epsilon());
  for (int j = 0; j < m && W.ok(); ++j) {
    W.apply_col(j);
    double image = 0.0;
    const double rem = W.checked(W.orthogonalize(j + 1, H[j], &image), "exponential-action Arnoldi remainder");
    W.checked(image, "exponential-action Arnoldi image");
    H[j][j + 1] = rem;
    k = j + 1;
    if (rem == 0.0 || (long long)(j + 1) == W.n) {
      exact = true;
      break;
    }
    near |= rem <= breakfactor * std::max(image, std::numeric_limits<double>::min());
    W.set_col_from_w(j + 1, rem);
  }
  const int q = k + (exact ? 0 : 1);
  f.S = CMat(q);
  for (int l = 0; l < k; ++l)
    for (int i = 0; i < k; ++i) f.S(i, l) = H[l][i];
  if (!exact) f.S(k, k - 1) = H[k - 1][k];
  f.used = k;
  if (!exact && near) {
    f.enlarged = true;
    f.used += 1;
    W.apply_col(q - 1);
    std::vector<cd> extra(q, cd(0, 0));
    double image = 0.0;
    f.next_remainder = W.checked(W.orthogonalize(q, extra, &image), "exponential-action enlarged Arnoldi remainder");
    W.checked(image, "exponential-action enlarged Arnoldi image");
    for (int i = 0; i < q; ++i) f.S(i, q - 1) += extra[i];
  }
  f.k = k;
  f.q = q;
  f.coeff_count = f.enlarged ? q : k;
  f.completed = exact || (f.enlarged && ((long long)q == W.n || f.next_remainder == 0.0));
  return f;
}

// _expv_project_factorization! (krylov_extensions.jl:1403-1426); returns the error estimate.
double project(ExpvWork& W, const Factorization& f, double h) {
  if (f.zero_state) {
    W.chk(cudaMemsetAsync(W.trial, 0, sizeof(double2) * W.n, W.s));
    return 0.0;
  }
  CMat A(f.q);
  for (size_t i = 0; i < A.a.size(); ++i) A.a[i] = h * f.S.a[i];
  const CMat E = expm(A);
  std::vector<double2> c(f.coeff_count);
  for (int i = 0; i < f.coeff_count; ++i) {
    const cd v = f.beta * E(i, 0);
    c[i] = make_double2(v.real(), v.imag());
  }
  W.chk(cudaMemcpyAsync(W.coef, c.data(), sizeof(double2) * f.coeff_count, cudaMemcpyHostToDevice, W.s));
  W.combine(f.coeff_count);
  if (f.completed) return 0.0;
  if (f.enlarged) return f.beta * std::abs(h) * f.next_remainder * std::abs(E(f.q - 1, 0));
  return f.beta * std::abs(E(f.k, 0));
}

struct ExpvControls {
  double atol = 1e-10, rtol = 1e-8;
  double initial_step = 0, minimum_step = 0, maximum_step = 0;
  int max_steps = 10000;
  double safety = 0.9;
};

// krylov_expv! (krylov_extensions.jl:1452-1573).  On return W.cur holds the state.
int expv_run(ExpvWork& W, double t, const ExpvControls& c, pi_expv_info_t* info) {
  std::memset(info, 0, sizeof(*info));
  const double time = t;
  const double total = std::abs(time);
  if (total == 0.0) {
    info->converged = 1;
    return PI_OK;
  }
  double hmax = c.maximum_step > 0 ? c.maximum_step : total;
  const double hmin = c.minimum_step > 0 ? c.minimum_step : 0.0;
  const double h0 = c.initial_step > 0 ? c.initial_step : hmax;
  hmax = std::min(hmax, total);
  double h = std::min(h0, hmax);
  if (hmin > hmax) return fail(PI_ERR_INVALID_ARGUMENT, "minimum_step must not exceed the effective maximum step");
  if (h0 < hmin) return fail(PI_ERR_INVALID_ARGUMENT, "initial_step must not be smaller than minimum_step");
  double reached = 0.0, error_sum = 0.0;
  int accepted = 0, rejected = 0, attempts = 0, factorizations = 0;
  const double direction = time < 0 ? -1.0 : 1.0;
  bool have = false;
  Factorization f;
  try {
    while (reached < total && attempts < c.max_steps && W.ok()) {
      ++attempts;
      h = std::min(h, total - reached);
      if (!have) {
        f = arnoldi(W);
        have = true;
        ++factorizations;
      }
      const double error = project(W, f, direction * h);
      double trial_norm = W.norm64(W.trial);
      const bool finite = std::isfinite(trial_norm) && std::isfinite(error);
      if (!finite) trial_norm = W.checked(W.norm64(W.cur), "exponential-action state");
      const double fraction = h / total;
      const double localtol = fraction * (c.atol + c.rtol * trial_norm);
      if (!std::isfinite(localtol))
        return fail(PI_ERR_INVALID_ARGUMENT,
                    "exponential-action local tolerance overflowed; rescale the state or use wider precision");
      const bool accept = finite && (f.completed || error <= localtol);
      if (accept) {
        std::swap(W.cur, W.trial);
        const double remaining = total - reached;
        const double next = (h == remaining) ? total : reached + h;
        if (!(next > reached))
          return fail(PI_ERR_INVALID_ARGUMENT,
                      "exponential-action time step no longer advances; use fewer steps or wider precision");
        reached = next;
        ++accepted;
        error_sum += error;
        have = false;
      } else {
        ++rejected;
      }
      double factor;
      if (!finite)
        factor = 0.2;
      else if (f.completed)
        factor = 5.0;
      else if (error == 0.0)
        factor = 2.0;
      else {
        const double exponent = 1.0 / (double)std::max(f.k, 1);
        factor = c.safety * std::pow(localtol / error, exponent);
        factor = std::min(std::max(factor, 0.2), 5.0);
      }
      if (!accept) factor = std::min(factor, 0.5);
      const double hnew = std::min(hmax, h * factor);
      if (!accept && (hnew < hmin || hnew == 0.0 || (reached > 0.0 && reached + hnew == reached))) break;
      h = std::max(hnew, hmin);
    }
  } catch (const NonFinite& nf) {
    return fail(PI_ERR_INVALID_ARGUMENT, std::string(nf.what) + " is not finite");
  }
  if (!W.ok()) return cuda_fail(W.err, "expv");
  info->converged = reached == total;
  info->reached_time = direction * reached;
  info->accepted_steps = accepted;
  info->rejected_steps = rejected;
  info->operator_applications = W.applications;
  info->arnoldi_factorizations = factorizations;
  info->trial_evaluations = attempts;
  info->estimated_error = error_sum;
  if (!info->converged) {
    char msg[200];
    std::snprintf(msg, sizeof(msg), "adaptive Krylov exponential action reached time %.17g of %.17g after %d attempts",
                  direction * reached, time, attempts);
    return fail(PI_ERR_NOT_CONVERGED, msg);
  }
  return PI_OK;
}

int check_opts(const pi_expv_opts_t* o) {
  if (!o) return fail(PI_ERR_INVALID_ARGUMENT, "null options");
  if (o->krylovdim < 1 || o->krylovdim > kMaxDots - 2) return fail(PI_ERR_INVALID_ARGUMENT, "krylovdim must lie in 1:126");
  if (!(o->atol >= 0) || !(o->rtol >= 0) || !std::isfinite(o->atol) || !std::isfinite(o->rtol))
    return fail(PI_ERR_INVALID_ARGUMENT, "atol and rtol must be finite nonnegative real numbers");
  if (!(o->safety > 0 && o->safety < 1)) return fail(PI_ERR_INVALID_ARGUMENT, "safety must lie strictly between zero and one");
  if (o->max_steps < 1) return fail(PI_ERR_INVALID_ARGUMENT, "max_steps must be positive");
  if (o->precision != PI_FP64 && o->precision != PI_FP32)
    return fail(PI_ERR_INVALID_ARGUMENT, "precision must be PI_FP64 or PI_FP32");
  return PI_OK;
}

ExpvControls controls(const pi_expv_opts_t* o) {
  ExpvControls c;
  c.atol = o->atol;
  c.rtol = o->rtol;
  c.initial_step = o->initial_step;
  c.minimum_step = o->minimum_step;
  c.maximum_step = o->maximum_step;
  c.max_steps = o->max_steps;
  c.safety = o->safety;
  return c;
}

// Allocates the workspace; state (FP64) goes into W.cur.
bool alloc_work(ExpvWork& W, Bufs& B) {
  const size_t e = W.mixed ? sizeof(float2) : sizeof(double2);
  W.V = B.get(e * (size_t)W.n * (W.m + 1));
  W.w = B.get(e * (size_t)W.n);
  W.cur = (double2*)B.get(sizeof(double2) * W.n);
  W.trial = (double2*)B.get(sizeof(double2) * W.n);
  W.h1 = (double2*)B.get(sizeof(double2) * 2 * kMaxDots);  // h2 follows h1 contiguously
  W.h2 = W.h1 ? W.h1 + kMaxDots : nullptr;
  W.coef = (double2*)B.get(sizeof(double2) * kMaxDots);
  return B.err == cudaSuccess;
}

}  // namespace
}  // namespace picuda

using namespace picuda;

extern "C" {

void pi_expv_default_opts(pi_expv_opts_t* o) {
  if (!o) return;
  o->krylovdim = 30;
  o->atol = 1e-10;
  o->rtol = 1e-8;
  o->initial_step = 0;
  o->minimum_step = 0;
  o->maximum_step = 0;
  o->max_steps = 10000;
  o->safety = 0.9;
  o->precision = PI_FP64;
}

int pi_expv(pi_plan* plan, double* x_dev, double t, const pi_expv_opts_t* opts, pi_expv_info_t* info) {
  if (!plan || !x_dev) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  int rc = check_opts(opts);
  if (rc) return rc;
  if (!std::isfinite(t)) return fail(PI_ERR_INVALID_ARGUMENT, "time must be finite");
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  if (opts->krylovdim <= kBatchMaxKrylov) {
    // one job of the plan's batched engine: the whole Arnoldi cycle on the device
    DynamicsJob job(plan, x_dev, {0.0, t}, 0, nullptr, nullptr, *opts, true);
    rc = run_single_job(plan, &job, opts->krylovdim, opts->precision == PI_FP32, "expv");
    if (rc) return rc;
    if (info) *info = job.info();
    return job.rc == PI_OK ? PI_OK : fail(job.rc, job.msg);
  }
  pi_expv_info_t loc;
  ExpvWork W{plan, plan->stream, plan->host.dim, (int)std::min<long long>(opts->krylovdim, plan->host.dim),
             opts->precision == PI_FP32};
  {
    Bufs B;
    B.s = W.s;
    if (!alloc_work(W, B)) return cuda_fail(B.err, "expv workspace");
    const DevicePlan& dp = plan->dev;
    if (W.mixed)
      W.chk(x_to_z_f64(dp, (const double2*)x_dev, W.cur, 1.0, W.s));
    else
      W.chk(cudaMemcpyAsync(W.cur, x_dev, sizeof(double2) * W.n, cudaMemcpyDeviceToDevice, W.s));
    rc = expv_run(W, t, controls(opts), &loc);
    if (rc == PI_OK || rc == PI_ERR_NOT_CONVERGED) {
      if (W.mixed)
        W.chk(z_to_x_f64(dp, W.cur, (double2*)x_dev, 1.0, 0, W.s));
      else
        W.chk(cudaMemcpyAsync(x_dev, W.cur, sizeof(double2) * W.n, cudaMemcpyDeviceToDevice, W.s));
      W.chk(cudaStreamSynchronize(W.s));
      if (!W.ok()) rc = cuda_fail(W.err, "expv result copy");
    }
  }
  if (info) *info = loc;
  return rc;
}

int pi_solve_dynamics(pi_plan* plan, double* rho_dev, int nt, const double* times, int nobs, const double* obs_dev,
                      double* values_host, const pi_expv_opts_t* opts, pi_expv_info_t* info) {
  if (!plan || !rho_dev || !times || nt < 1) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (nobs < 0 || nobs > kMaxDots || (nobs > 0 && (!obs_dev || !values_host)))
    return fail(PI_ERR_INVALID_ARGUMENT, "observables must number 0..128 with device data and a host output");
  int rc = check_opts(opts);
  if (rc) return rc;
  for (int i = 1; i < nt; ++i)
    if (!(times[i] >= times[i - 1]) || !std::isfinite(times[i]))
      return fail(PI_ERR_INVALID_ARGUMENT, "Krylov exponential output times must be nondecreasing");
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  if (opts->krylovdim <= kBatchMaxKrylov && nobs <= kBatchMaxObs) {
    DynamicsJob job(plan, rho_dev, std::vector<double>(times, times + nt), nobs, obs_dev, values_host, *opts, false);
    rc = run_single_job(plan, &job, opts->krylovdim, opts->precision == PI_FP32, "dynamics");
    if (rc) return rc;
    if (info) *info = job.info();
    return job.rc == PI_OK ? PI_OK : fail(job.rc, job.msg);
  }
  ExpvWork W{plan, plan->stream, plan->host.dim, (int)std::min<long long>(opts->krylovdim, plan->host.dim),
             opts->precision == PI_FP32};
  pi_expv_info_t total;
  std::memset(&total, 0, sizeof(total));
  total.converged = 1;
  {
    Bufs B;
    B.s = W.s;
    if (!alloc_work(W, B)) return cuda_fail(B.err, "dynamics workspace");
    double2* xview = (double2*)B.get(sizeof(double2) * W.n);
    if (!xview) return cuda_fail(B.err, "dynamics workspace");
    const DevicePlan& dp = plan->dev;
    const ExpvControls c = controls(opts);
    if (W.mixed)
      W.chk(x_to_z_f64(dp, (const double2*)rho_dev, W.cur, 1.0, W.s));
    else
      W.chk(cudaMemcpyAsync(W.cur, rho_dev, sizeof(double2) * W.n, cudaMemcpyDeviceToDevice, W.s));
    auto record = [&](int it) {
      if (nobs == 0) return;
      const double2* x = W.cur;
      if (W.mixed) {
        W.chk(z_to_x_f64(dp, W.cur, xview, 1.0, 0, W.s));
        x = xview;
      }
      // dot(op.data, rho.data) for every observable (highlevel.jl:672-677)
      W.chk(mdot_f64((const double2*)obs_dev, W.n, nobs, x, W.n, plan->rs, plan->rs.result, W.s));
      W.fetch(values_host + (size_t)it * nobs * 2, plan->rs.result, sizeof(double2) * nobs);
    };
    record(0);
    for (int it = 1; it < nt && rc == PI_OK; ++it) {
      const double dt = times[it] - times[it - 1];
      if (dt != 0.0) {
        pi_expv_info_t one;
        rc = expv_run(W, dt, c, &one);
        total.accepted_steps += one.accepted_steps;
        total.rejected_steps += one.rejected_steps;
        total.arnoldi_factorizations += one.arnoldi_factorizations;
        total.trial_evaluations += one.trial_evaluations;
        total.estimated_error += one.estimated_error;
        total.reached_time = times[it];
        if (rc != PI_OK) total.converged = 0;
      }
      if (rc == PI_OK) record(it);
    }
    total.operator_applications = W.applications;
    if (W.mixed)
      W.chk(z_to_x_f64(dp, W.cur, (double2*)rho_dev, 1.0, 0, W.s));
    else
      W.chk(cudaMemcpyAsync(rho_dev, W.cur, sizeof(double2) * W.n, cudaMemcpyDeviceToDevice, W.s));
    W.chk(cudaStreamSynchronize(W.s));
    if (rc == PI_OK && !W.ok()) rc = cuda_fail(W.err, "dynamics");
  }
  if (info) *info = total;
  return rc;
}

}  // extern "C"
