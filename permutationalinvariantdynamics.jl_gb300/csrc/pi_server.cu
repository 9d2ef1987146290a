// Continuous-batching request loop over the multi-instance engine (pi_batch.hpp).
//
// Clients submit time-evolution and steady-state requests from any thread.  One worker
// thread owns the engine: between engine ticks it admits queued requests in arrival order
// while their device footprint fits the memory budget (and the active-request cap), folds
// them into the next tick's batched launches, and retires finished requests (their state
// written back, their workspaces freed, a completion posted with timestamps).  States and
// Krylov bases of active requests stay resident in HBM for their whole life.  With
// steady_solvers > 0 the worker hands admitted steady-state requests to a pool of solver
// threads instead, which run preconditioned single-instance solves on the plans' own streams
// beside the engine; their footprint stays charged to the budget until they complete.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "pi_batch.hpp"
#include "pi_handle.hpp"
#include "pi_precond.hpp"

using Clock = std::chrono::steady_clock;

namespace picuda {
namespace {

struct Pending {
  pi_request_t req;
  size_t footprint = 0;
  double submit_time = 0;
};

struct Active {
  pi_request_t req;
  std::unique_ptr<Job> job;
  size_t footprint = 0;
  double submit_time = 0, start_time = 0;
};

// Saved-time grid t0:dt:t1 with t1 appended when the range stops short (highlevel.jl:434-465).
std::vector<double> saved_grid(double t1, double dt) {
  std::vector<double> ts;
  const double t0 = 0.0;
  const long long count = (long long)std::floor((t1 - t0) / dt * (1 + 1e-15)) + 1;
  for (long long i = 0; i < count; ++i) {
    const double t = t0 + (double)i * dt;
    if (t <= t1) ts.push_back(t);
  }
  if (ts.empty() || ts.back() < t1) ts.push_back(t1);
  return ts;
}

}  // namespace
}  // namespace picuda

using namespace picuda;

struct pi_server {
  pi_server_opts_t opts{};
  int device = 0;
  std::unique_ptr<Engine> engine;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable wake;       // worker: submissions or stop
  std::condition_variable completed;  // pollers
  std::deque<Pending> incoming;
  std::deque<pi_completion_t> done;
  bool stop = false;
  bool failed = false;
  std::string fail_msg;
  pi_server_stats_t stats{};
  std::thread worker;
  // preconditioned steady-state solver pool (steady_solvers > 0)
  std::deque<Active> steady_queue;
  std::condition_variable steady_wake;
  std::vector<std::thread> solvers;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
  size_t footprint(const pi_request_t& r) const {
    const long long dim = r.plan->host.dim;
    const size_t es = opts.precision == PI_FP32 ? sizeof(float2) : sizeof(double2);
    size_t b = es * (size_t)dim * (opts.krylovdim + 3);  // basis (m + 2 columns) + image
    if (r.kind == PI_REQUEST_DYNAMICS) {
      b += 2 * sizeof(double2) * (size_t)dim;
      if (opts.precision == PI_FP32) b += sizeof(double2) * (size_t)dim * r.nobs;
    } else if (opts.steady_solvers > 0) {
      // GMRES(max(m, 50)) basis and its FP64 vectors, the preconditioner tables and scratch
      b = es * (size_t)dim * (std::max(opts.krylovdim, 50) + 1) + 24 * sizeof(double2) * (size_t)dim;
    } else {
      b += 3 * sizeof(double2) * (size_t)dim;
    }
    return b;
  }
  void post(const Active& a, int status, const std::string& msg) {
    pi_completion_t c;
    std::memset(&c, 0, sizeof(c));
    c.tag = a.req.tag;
    c.kind = a.req.kind;
    c.status = status;
    c.submit_time = a.submit_time;
    c.start_time = a.start_time;
    c.finish_time = now();
    if (a.job) {
      if (a.req.kind == PI_REQUEST_DYNAMICS) {
        const pi_expv_info_t I = static_cast<DynamicsJob*>(a.job.get())->info();
        c.iterations = I.accepted_steps;
        c.operator_applications = I.operator_applications;
        c.residual = I.estimated_error;
      } else {
        const pi_gmres_info_t I = static_cast<SteadyJob*>(a.job.get())->info();
        c.iterations = I.iterations;
        c.operator_applications = I.operator_applications;
        c.residual = I.normalized_residual;
        c.trace_error = I.trace_error;
      }
    }
    std::snprintf(c.message, sizeof(c.message), "%s", msg.c_str());
    finish_post(c, a.footprint);
  }
  void finish_post(const pi_completion_t& c, size_t fp) {
    std::lock_guard<std::mutex> lk(mu);
    done.push_back(c);
    stats.completed += 1;
    stats.active -= 1;
    stats.bytes_in_use -= (double)fp;
    completed.notify_all();
    wake.notify_all();  // freed budget may admit queued requests
  }
  void run();
  void solve_steady();
};

// One solver thread: preconditioned single-instance steady states of admitted requests.
void pi_server::solve_steady() {
  cudaSetDevice(device);
  for (;;) {
    Active a;
    {
      std::unique_lock<std::mutex> lk(mu);
      steady_wake.wait(lk, [&] { return stop || !steady_queue.empty(); });
      if (stop) return;
      a = std::move(steady_queue.front());
      steady_queue.pop_front();
    }
    const pi_request_t& r = a.req;
    a.start_time = now();
    pi_precond* lev = nullptr;
    pi_precond* drv = nullptr;
    // Where the level sweep does not apply (decay and pump channels together: its gains
    // would point both ways) the request is solved with the reference's unpreconditioned
    // method; the drive part alone is no preconditioner for such dissipation-dominated models.
    int rc = pi_precond_create(r.plan, PI_COORDS_POPULATION, 0.0, 0.0, &lev);
    if (rc) lev = nullptr;
    rc = lev ? pi_precond_create_drive(r.plan, PI_COORDS_POPULATION, precond_scale(lev), &drv) : PI_OK;
    pi_gmres_info_t info;
    std::memset(&info, 0, sizeof(info));
    std::string msg;
    if (rc == PI_OK) {
      pi_gmres_opts_t o;
      pi_gmres_default_opts(&o);
      o.krylovdim = std::max(opts.krylovdim, 50);  // GMRES(50), the steady-state restart length
      o.precision = opts.precision;
      o.maxiter = r.maxiter > 0 ? r.maxiter : 2000;
      if (r.atol > 0) o.atol = r.atol;
      if (r.rtol > 0) o.rtol = r.rtol;
      o.coords = lev ? PI_COORDS_POPULATION : PI_COORDS_REFERENCE;
      o.preconditioner = lev;
      o.drive_preconditioner = drv;
      rc = pi_steady_state(r.plan, r.state_dev, &o, &info);
    }
    if (rc != PI_OK) {
      char buf[512];
      pi_last_error(buf, sizeof(buf));
      msg = buf;
    }
    if (lev) pi_precond_destroy(lev);
    if (drv) pi_precond_destroy(drv);
    pi_completion_t c;
    std::memset(&c, 0, sizeof(c));
    c.tag = r.tag;
    c.kind = r.kind;
    c.status = rc;
    c.submit_time = a.submit_time;
    c.start_time = a.start_time;
    c.finish_time = now();
    c.iterations = info.iterations;
    c.operator_applications = info.operator_applications;
    c.residual = info.normalized_residual;
    c.trace_error = info.trace_error;
    std::snprintf(c.message, sizeof(c.message), "%s", msg.c_str());
    finish_post(c, a.footprint);
  }
}

void pi_server::run() {
  cudaSetDevice(device);
  std::vector<Active> active;
  for (;;) {
    // ---- admission (arrival order; stops at the first request that does not fit)
    std::vector<Pending> admit;
    {
      std::unique_lock<std::mutex> lk(mu);
      wake.wait(lk, [&] { return stop || !incoming.empty() || !active.empty(); });
      if (stop) break;
      while (!incoming.empty()) {
        const Pending& p = incoming.front();
        const bool fits = stats.bytes_in_use + (double)p.footprint <= opts.memory_budget;
        const bool slot = opts.max_active <= 0 || stats.active < opts.max_active;
        if (!fits || !slot) break;
        stats.bytes_in_use += (double)p.footprint;
        stats.active += 1;
        stats.queued -= 1;
        stats.admitted += 1;
        admit.push_back(p);
        incoming.pop_front();
      }
    }
    for (Pending& p : admit) {
      Active a;
      a.req = p.req;
      a.footprint = p.footprint;
      a.submit_time = p.submit_time;
      a.start_time = now();
      const pi_request_t& r = p.req;
      if (r.kind == PI_REQUEST_STEADY && opts.steady_solvers > 0) {
        std::lock_guard<std::mutex> lk(mu);
        steady_queue.push_back(std::move(a));
        steady_wake.notify_one();
        continue;
      }
      if (r.kind == PI_REQUEST_DYNAMICS) {
        pi_expv_opts_t o;
        pi_expv_default_opts(&o);
        o.krylovdim = opts.krylovdim;
        o.precision = opts.precision;
        if (r.atol > 0) o.atol = r.atol;
        if (r.rtol > 0) o.rtol = r.rtol;
        a.job.reset(new DynamicsJob(r.plan, r.state_dev, saved_grid(r.t_final, r.dt), r.nobs, r.obs_dev,
                                    r.values_host, o, false));
      } else {
        pi_gmres_opts_t o;
        pi_gmres_default_opts(&o);
        o.krylovdim = opts.krylovdim;
        o.precision = opts.precision;
        if (r.atol > 0) o.atol = r.atol;
        if (r.rtol > 0) o.rtol = r.rtol;
        if (r.maxiter > 0) o.maxiter = r.maxiter;
        a.job.reset(new SteadyJob(r.plan, r.state_dev, o, 0x51ca1eULL ^ r.tag));
      }
      if (!a.job->setup(engine->stream(), engine->m(), engine->f32())) {
        post(a, PI_ERR_OUT_OF_MEMORY, "request workspace allocation failed");
        continue;
      }
      engine->add(a.job.get());
      active.push_back(std::move(a));
    }
    if (active.empty()) continue;
    // ---- one engine tick over every active request
    if (!engine->tick()) {
      const std::string m = std::string("CUDA error in the serving engine: ") + cudaGetErrorString(engine->err);
      {
        std::lock_guard<std::mutex> lk(mu);
        failed = true;
        fail_msg = m;
      }
      for (Active& a : active) post(a, PI_ERR_CUDA, m);
      active.clear();
      break;
    }
    // ---- retire finished requests
    std::vector<Job*> fin = engine->retire();
    if (fin.empty()) continue;
    for (Job* j : fin) j->finish(engine->stream());
    const cudaError_t e = cudaStreamSynchronize(engine->stream());
    std::vector<Active> keep;
    for (Active& a : active) {
      if (!a.job->finished) {
        keep.push_back(std::move(a));
        continue;
      }
      const int status = e != cudaSuccess ? PI_ERR_CUDA : a.job->rc;
      post(a, status, e != cudaSuccess ? cudaGetErrorString(e) : a.job->msg);
    }
    active.swap(keep);
  }
  // stopped: abandon what is left (workspaces freed with the jobs)
  for (Active& a : active) post(a, PI_ERR_BUSY, "server stopped before the request finished");
  active.clear();
  cudaStreamSynchronize(engine->stream());
}

extern "C" {

void pi_server_default_opts(pi_server_opts_t* o) {
  if (!o) return;
  o->krylovdim = 30;
  o->precision = PI_FP64;
  o->memory_budget = 160e9;
  o->max_active = 0;
  o->use_graphs = 1;
  o->steady_solvers = 0;
}

int pi_server_create(const pi_server_opts_t* opts, int device, pi_server** out) {
  if (!opts || !out) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (opts->krylovdim < 1 || opts->krylovdim > kBatchMaxKrylov)
    return fail(PI_ERR_INVALID_ARGUMENT, "krylovdim must lie in 1:120 for the serving engine");
  if (opts->precision != PI_FP64 && opts->precision != PI_FP32)
    return fail(PI_ERR_INVALID_ARGUMENT, "precision must be PI_FP64 or PI_FP32");
  if (!(opts->memory_budget > 0)) return fail(PI_ERR_INVALID_ARGUMENT, "memory_budget must be positive");
  if (opts->steady_solvers < 0 || opts->steady_solvers > 64)
    return fail(PI_ERR_INVALID_ARGUMENT, "steady_solvers must lie in 0:64");
  std::unique_ptr<pi_server> S(new pi_server());
  S->opts = *opts;
  S->device = device;
  S->t0 = Clock::now();
  S->engine.reset(new Engine(device, opts->krylovdim, opts->precision == PI_FP32, opts->use_graphs != 0));
  if (S->engine->err != cudaSuccess) return cuda_fail(S->engine->err, "serving engine");
  pi_server* raw = S.get();
  S->worker = std::thread([raw] { raw->run(); });
  for (int i = 0; i < opts->steady_solvers; ++i) S->solvers.emplace_back([raw] { raw->solve_steady(); });
  *out = S.release();
  return PI_OK;
}

int pi_server_submit(pi_server* S, const pi_request_t* r) {
  if (!S || !r || !r->plan || !r->state_dev) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (r->kind != PI_REQUEST_DYNAMICS && r->kind != PI_REQUEST_STEADY)
    return fail(PI_ERR_INVALID_ARGUMENT, "request kind must be PI_REQUEST_DYNAMICS or PI_REQUEST_STEADY");
  if (r->plan->device != S->device) return fail(PI_ERR_INVALID_ARGUMENT, "the plan lives on another device");
  if (r->kind == PI_REQUEST_DYNAMICS) {
    if (!(std::isfinite(r->t_final) && r->t_final >= 0 && std::isfinite(r->dt) && r->dt > 0))
      return fail(PI_ERR_INVALID_ARGUMENT, "dynamics requests need finite t_final >= 0 and dt > 0");
    if (r->nobs < 0 || r->nobs > kBatchMaxObs || (r->nobs > 0 && (!r->obs_dev || !r->values_host)))
      return fail(PI_ERR_INVALID_ARGUMENT, "observables must number 0..16 with device data and a host output");
  }
  if (!(r->atol >= 0) || !(r->rtol >= 0)) return fail(PI_ERR_INVALID_ARGUMENT, "tolerances must be nonnegative");
  Pending p;
  p.req = *r;
  p.footprint = S->footprint(*r);
  if ((double)p.footprint > S->opts.memory_budget)
    return fail(PI_ERR_OUT_OF_MEMORY, "request needs more device memory than the server's budget");
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->failed) return fail(PI_ERR_CUDA, S->fail_msg);
  if (S->stop) return fail(PI_ERR_BUSY, "server is stopping");
  p.submit_time = S->now();
  S->incoming.push_back(p);
  S->stats.submitted += 1;
  S->stats.queued += 1;
  S->wake.notify_one();
  return PI_OK;
}

int pi_server_poll(pi_server* S, pi_completion_t* out, int max, int* count, int timeout_ms) {
  if (!S || !count || (max > 0 && !out)) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_lock<std::mutex> lk(S->mu);
  auto ready = [&] { return !S->done.empty() || S->failed; };
  if (timeout_ms < 0)
    S->completed.wait(lk, ready);
  else if (timeout_ms > 0)
    S->completed.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
  int n = 0;
  while (n < max && !S->done.empty()) {
    out[n++] = S->done.front();
    S->done.pop_front();
  }
  *count = n;
  return PI_OK;
}

int pi_server_stats(pi_server* S, pi_server_stats_t* st) {
  if (!S || !st) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  *st = S->stats;
  st->ticks = S->engine->ticks;
  st->cycles = S->engine->cycles;
  st->arnoldi_steps = S->engine->steps;
  st->elapsed = S->now();
  return PI_OK;
}

int pi_server_destroy(pi_server* S) {
  if (!S) return PI_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->wake.notify_all();
    S->steady_wake.notify_all();
  }
  if (S->worker.joinable()) S->worker.join();
  for (auto& t : S->solvers)
    if (t.joinable()) t.join();
  // requests handed to the pool but not started
  while (!S->steady_queue.empty()) {
    Active a = std::move(S->steady_queue.front());
    S->steady_queue.pop_front();
    S->post(a, PI_ERR_BUSY, "server stopped before the request finished");
  }
  delete S;
  return PI_OK;
}

}  // extern "C"
