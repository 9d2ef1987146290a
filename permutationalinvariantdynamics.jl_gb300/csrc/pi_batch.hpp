// Multi-instance Krylov engine shared by the batched entry points and the serving loop.
//
// Many independent solves (parameter points, particle numbers, served requests) advance
// together.  Each engine tick runs, over every job that asks for it:
//   stage 1  vector work: basis combinations (expv trial states, GMRES updates), random
//            probes, FP64 applies of arbitrary vectors (residuals, final checks), residual
//            differences, norms, observable dots and trace values;  then one host read;
//   stage 2  host controllers consume those numbers (accept/reject, convergence tests);
//   stage 3  one Arnoldi cycle for every job that needs a factorization: all jobs step in
//            lockstep, one launch per kernel over an (instance, sector-tile) or
//            (instance, element-chunk) work list.  The Arnoldi column index, the stop flags
//            and the GMRES Givens state live in device memory, so the m steps of a cycle
//            run with no host synchronisation (optionally as one CUDA graph); the host reads
//            the Hessenberg records once per cycle.
// Every reduction of an instance covers only that instance's chunks in a fixed order, so a
// job's arithmetic does not depend on which other jobs share the tick.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/picuda.h"
#include "pi_handle.hpp"

namespace picuda {

constexpr int kBatchChunk = 4096;       // elements per reduction chunk, large batches
constexpr int kBatchChunkSmall = 1024;  // when the active jobs hold few elements in total
constexpr int kBatchMaxObs = 16;   // observables per dynamics job
constexpr int kOutSlots = 4 + 2 * kBatchMaxObs;  // per-job stage-1 outputs (doubles)
constexpr int kBatchMaxKrylov = 120;

// Column stride of a Krylov basis: dim rounded up to 64 elements (aligned 16-byte loads of
// element pairs; the padding is zero).
inline long long basis_stride(long long dim) { return (dim + 63) / 64 * 64; }

// Stage-1 operation flags.
enum : unsigned {
  S1_COMBINE = 1u,
  S1_PROBE = 2u,
  S1_AUX = 4u,
  S1_RESID = 8u,
  S1_NORM = 16u,
  S1_OBS = 32u,
  S1_TRACE = 64u,
};

// Device control block of one job in the engine (host copy uploaded before each stage).
struct DevInst {
  // plan tables
  const DevSector* sectors;
  const DevTerm* terms;
  const DevTile* tiles;
  const void* coefb;      // coefficients of the basis precision and coordinates
  const double2* coef64;  // FP64 reference-coordinate coefficients (stage-1 applies)
  const int* diag_sector;
  const long long* diag_index;
  long long dim;
  long long ldv;    // basis column stride: dim rounded up to a multiple of 64, zero padded
  int ndiag;
  int chunk_begin;  // first chunk of this job in the engine's chunk list
  int chunk;        // elements per chunk (the engine's choice, kBatchChunkSmall or kBatchChunk)
  // Krylov cycle
  void* V;  // m + 2 basis columns (FP64 or FP32)
  void* w;
  double2* hA;  // CGS2 projections, pass 1 and 2
  double2* hB;
  double2* H;   // Hessenberg columns, stride ldh
  double2* g;   // GMRES right-hand side (m + 2)
  double2* csn; // GMRES rotations: (cos, 0) at [0, m+2), sin at [m+2, 2m+4)
  double* image;  // |L V_j| per step
  int m;         // steps of this cycle
  int ldh;
  int coords;    // 0: reference coordinates, 1: population coordinates
  int border;    // bordered operator (steady state)
  int givens;    // GMRES rotations and residual stop test
  int j;         // input column of the next step
  int done;      // no further steps this cycle
  int kdone;     // completed steps
  int reorth;    // FP32 basis: this step's second CGS projection ran (selective reorthogonalisation)
  // FP32 basis, canonical plan: merged coefficients of the Arnoldi applies in the coordinate
  // system pwhich (eplane == nullptr: the generic stencil terms)
  SplitPlanes planes;
  int pwhich;
  double scale;  // multiplies L V_j
  double tol;    // GMRES: stop when |g[j+1]| <= tol
  double rem2;
  double image2;
  double2 alpha;
  const double2* v0;  // V_0 = v0 / v0norm (FP64 source)
  double v0norm;
  // stage-1 operands (nullptr: the job takes no part)
  double2* cout;          // cout (+)= sum_k ccoef[k] V_k
  const double2* ccoef;
  int ccount;
  int cacc;
  double2* probe;         // complex normal probe vector
  unsigned long long seed;
  const double2* ax;      // ay = aux_scale L ax (+ (t^H ax) v when aux_border)
  double2* ay;
  double aux_scale;
  int aux_border;
  int nob;                // observable dots conj(ob_o) . obx, o < nob
  double2 aux_alpha;
  const double2* rb;      // rout = rb - ay
  double2* rout;
  const double2* nrm0;    // |nrm0|^2 -> out[0], |nrm1|^2 -> out[1]
  const double2* nrm1;
  const double2* tr;      // t^H tr -> out[2], out[3] (reference coordinates)
  const double2* ob;      // nob vectors of dim entries
  const double2* obx;
  double* out;            // kOutSlots doubles
};

// A job driven by the engine: a resumable controller plus its device vectors.
class Job {
 public:
  virtual ~Job();
  pi_plan* plan = nullptr;
  long long dim = 0;
  int rc = PI_OK;
  std::string msg;
  bool finished = false;
  bool bordered = false;  // cycles apply the trace-bordered operator (steady-state jobs)
  size_t bytes = 0;  // device bytes held by the job
  void* V = nullptr;
  void* w = nullptr;
  long long ldv = 0;
  // Allocates the basis and the job's vectors; false on allocation failure.
  virtual bool setup(cudaStream_t s, int m, bool f32) = 0;
  // Stage 1: sets operands in d and coefficients in coef (when combining); returns flags.
  virtual unsigned stage1(DevInst& d, double2* coef) = 0;
  virtual void after_stage1(const double* out) = 0;
  // Stage 3: configures an Arnoldi cycle in d; false when the job needs none this tick.
  virtual bool cycle(DevInst& d) = 0;
  // Consumes a finished cycle (r: downloaded control block, rec: its Hessenberg record);
  // true asks for one more step with d configured (expv near-breakdown enlargement).
  virtual bool after_cycle(const DevInst& r, const double2* rec, DevInst& d) = 0;
  virtual void after_enlarge(const DevInst& r, const double2* rec) {}
  // Writes results back (stream-ordered) once finished.
  virtual void finish(cudaStream_t s) = 0;
  void fail_job(int code, const std::string& m);
  int ldh = 0;
  int m_engine = 0;

 protected:
  std::vector<void*> allocs_;
  cudaStream_t s_ = nullptr;
  void* alloc(size_t bytes, cudaError_t* err);
};

// Batched dynamics job: the expv controller of krylov_extensions.jl:1452-1573 per saved
// interval (highlevel.jl:665-733), with observable dots at every saved time.
class DynamicsJob : public Job {
 public:
  DynamicsJob(pi_plan* p, double* state, std::vector<double> times, int nobs, const double* obs,
              double* values, const pi_expv_opts_t& o, bool single_interval);
  bool setup(cudaStream_t s, int m, bool f32) override;
  unsigned stage1(DevInst& d, double2* coef) override;
  void after_stage1(const double* out) override;
  bool cycle(DevInst& d) override;
  bool after_cycle(const DevInst& r, const double2* rec, DevInst& d) override;
  void after_enlarge(const DevInst& r, const double2* rec) override;
  void finish(cudaStream_t s) override;
  pi_expv_info_t info() const;

 private:
  void begin_interval();
  void attempt();
  void project();
  void interval_done();
  double* state_;
  std::vector<double> times_;
  int nobs_;
  const double* obs_;
  double* values_;
  pi_expv_opts_t o_;
  bool single_;
  bool mixed_ = false;
  double2* cur_ = nullptr;
  double2* trial_ = nullptr;
  double2* obsz_ = nullptr;
  // progress
  int interval_ = 1;
  int obs_pending_ = -1;
  bool need_norm_ = true;
  bool want_factor_ = false;
  bool pending_trial_ = false;
  double cur_norm_ = 0;
  // interval controller
  double total_ = 0, reached_ = 0, h_ = 0, hmax_ = 0, hmin_ = 0, direction_ = 1;
  int attempts_ = 0;
  // factorization
  bool have_ = false, zero_ = false, completed_ = false, enlarged_ = false;
  int k_ = 0, q_ = 0;
  double beta_ = 0, next_rem_ = 0;
  std::vector<std::complex<double>> S_;  // q x q column-major
  std::vector<std::complex<double>> coef_;
  double err_ = 0;
  // totals
  int accepted_ = 0, rejected_ = 0, factorizations_ = 0, trials_ = 0, applications_ = 0;
  double error_sum_ = 0, reached_time_ = 0;
  bool converged_ = true;
  std::vector<int> zero_copies_;  // saved indices that repeat the pending record
};

// Batched steady-state job: restarted GMRES on the trace-bordered system
// (krylov.jl:732-891), FP64 or FP32 inner cycles with FP64 residual refinement.
class SteadyJob : public Job {
 public:
  // host_probes: draw the operator-scale probes on the host (std::mt19937_64 with the seed,
  // complex normal entries in element order, as the single-instance solver always has);
  // otherwise a counter-based generator on the device.
  SteadyJob(pi_plan* p, double* x, const pi_gmres_opts_t& o, unsigned long long seed, bool host_probes = false);
  bool setup(cudaStream_t s, int m, bool f32) override;
  unsigned stage1(DevInst& d, double2* coef) override;
  void after_stage1(const double* out) override;
  bool cycle(DevInst& d) override;
  bool after_cycle(const DevInst& r, const double2* rec, DevInst& d) override;
  void finish(cudaStream_t s) override {}
  pi_gmres_info_t info() const { return info_; }

 private:
  enum State { INIT, SCALE, RESID, FINAL, DONE };
  double2* x_;
  pi_gmres_opts_t o_;
  unsigned long long seed_;
  bool mixed_ = false;
  double2* b_ = nullptr;
  double2* r_ = nullptr;
  double2* ay_ = nullptr;
  double2* probes_ = nullptr;  // host-drawn probes (3 x dim), when host_probes_
  bool host_probes_ = false;
  State state_ = INIT;
  int probe_ = 0;
  double scale_ = 0, s_op_ = 0, tol_ = 0, beta_ = 0;
  bool want_cycle_ = false, pending_update_ = false, gm_converged_ = false;
  std::vector<std::complex<double>> y_;
  int iterations_ = 0, restarts_ = 0, refinements_ = 0, applications_ = 0, m_ = 30;
  double linear_residual_ = 0;
  pi_gmres_info_t info_{};
};

// Runs one job to completion on the plan's cached engine (Krylov dimension m, FP32 basis
// when f32); returns PI_OK or a CUDA failure status, the job's own status is job->rc.
int run_single_job(pi_plan* plan, Job* job, int m, bool f32, const char* what);
// Releases a plan's cached engine (plan teardown).
void release_plan_engine(pi_plan* plan);

// The engine: membership, work lists, stage execution.
class Engine {
 public:
  Engine(int device, int krylovdim, bool f32, bool use_graphs);
  ~Engine();
  cudaError_t err = cudaSuccess;
  cudaStream_t stream() const { return s_; }
  int m() const { return m_; }
  bool f32() const { return f32_; }
  int ldh() const { return m_ + 2; }
  // Adds a job (setup must have succeeded) / removes finished ones.
  void add(Job* j);
  std::vector<Job*> retire();
  size_t njobs() const { return jobs_.size(); }
  // One tick over every job; returns false on a CUDA error.
  bool tick();
  long long ticks = 0, cycles = 0, steps = 0;

 private:
  void chk(cudaError_t e) {
    if (e != cudaSuccess && err == cudaSuccess) err = e;
  }
  void rebuild();
  template <typename... KArgs, typename... Args>
  void launch(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, Args... args);
  template <typename Tuple, size_t... I>
  static void fill_ptrs(Tuple& t, void** p, std::index_sequence<I...>) {
    ((p[I] = (void*)&std::get<I>(t)), ...);
  }
  void arnoldi_step();
  void run_cycle_steps();
  void reserve(void** p, size_t* cap, size_t bytes, bool pinned);
  int device_;
  int m_;
  bool f32_;
  bool graphs_;
  cudaStream_t s_ = nullptr;
  std::vector<Job*> jobs_;
  bool dirty_ = true;
  int total_tiles_ = 0, total_chunks_ = 0;
  int chunk_ = kBatchChunk;
  bool any_border_ = true;  // some job of the current set runs bordered cycles
  size_t rec_stride_ = 0;  // double2 per job record
  // device work lists and scratch (capacity-managed)
  void* st_ = nullptr; size_t st_cap_ = 0;
  void* tile_inst_ = nullptr; size_t tile_inst_cap_ = 0;
  void* tile_local_ = nullptr; size_t tile_local_cap_ = 0;
  void* chunk_inst_ = nullptr; size_t chunk_inst_cap_ = 0;
  void* nchunks_ = nullptr; size_t nchunks_cap_ = 0;
  void* part1_ = nullptr; size_t part1_cap_ = 0;
  void* partv_ = nullptr; size_t partv_cap_ = 0;
  void* hab_ = nullptr; size_t hab_cap_ = 0;
  void* rec_ = nullptr; size_t rec_cap_ = 0;
  void* out_ = nullptr; size_t out_cap_ = 0;
  void* coefs_ = nullptr; size_t coefs_cap_ = 0;
  // pinned host mirrors
  void* st_h_ = nullptr; size_t st_h_cap_ = 0;
  void* st_dl_ = nullptr; size_t st_dl_cap_ = 0;
  void* rec_h_ = nullptr; size_t rec_h_cap_ = 0;
  void* out_h_ = nullptr; size_t out_h_cap_ = 0;
  void* coefs_h_ = nullptr; size_t coefs_h_cap_ = 0;
  std::vector<DevInst> base_;  // per-job control blocks with the static fields set
  cudaGraphExec_t graph_ = nullptr;
  cudaGraph_t build_ = nullptr;       // graph under construction
  cudaGraphNode_t last_ = nullptr;    // its last node
  // FP32 step-apply schedule: PI_SCHEDULE_PER_TILE (one block per work item) or the blocks
  // per SM of the persistent launch; chosen per job set before its first cycle, by the
  // process-wide setting or by timing the candidates (cached process-wide per device and
  // job-set shape)
  void choose_apply_schedule();
  void launch_step_apply(int schedule);
  int apply_schedule_ = PI_SCHEDULE_PER_TILE;
  bool schedule_chosen_ = false;
  int sm_count_ = 0;
  int persist_max_ = 0;  // resident blocks per SM of the persistent apply (0: unavailable)
};

}  // namespace picuda
