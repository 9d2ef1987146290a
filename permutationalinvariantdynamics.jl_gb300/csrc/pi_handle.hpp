// The opaque pi_plan handle behind the C ABI.
#pragma once

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "pi_internal.hpp"
#include "pi_plan.hpp"

namespace picuda {
class Engine;
}

struct pi_plan {
  picuda::QubitPlan host;
  picuda::DevicePlan dev;
  std::vector<void*> allocations;  // device buffers owned by the plan tables
  size_t device_bytes = 0;
  long long stencil_terms = 0;
  cudaStream_t stream = nullptr;
  int device = 0;
  picuda::ReduceScratch rs;        // reduction scratch (device)
  double* host_pinned = nullptr;   // small pinned staging buffer for reductions
  // Host-buffer applies: grow-only device staging and copy/compute pipeline streams.
  void* stage_x = nullptr;
  void* stage_y = nullptr;
  size_t stage_bytes = 0;
  cudaStream_t pipe[3] = {nullptr, nullptr, nullptr};
  // Calls that use the plan's stream, staging buffers or engine hold call_mu.  By default a
  // second caller waits (the locked MatrixFreeLiouvillian of liouvillian.jl:35-60); with
  // reject_concurrent set it gets PI_ERR_BUSY instead (the workspace rule of
  // threaded_apply.jl:575).  Recursive, like the reference's ReentrantLock.
  std::recursive_mutex call_mu;
  std::atomic<int> reject_concurrent{0};
  // Element-major batched apply (pi_apply_em.cu): tile list and merged coefficient planes,
  // built on first use (FP32 reference / population coordinates).
  std::mutex em_mu;
  const picuda::DevTile* em_tiles = nullptr;
  int em_ntiles = 0;
  const float2* em_planes32[2] = {nullptr, nullptr};
  // Encoded per-sector TMA tensor maps of the last few element-major source batches (host
  // copies, passed to the kernel by value), keyed by source pointer, stride and width.
  struct EmMapSet {
    const void* x;
    long long ld;
    int ncols;
    std::vector<unsigned char> maps;  // nsectors x 128 bytes
  };
  std::vector<EmMapSet> em_maps;
  // Split coefficient planes of the TMA-staged kernel (entry, row and column planes) per
  // coordinate system, and the per-sector offsets of the row and column planes.
  struct EmSplit {
    const float4* eplane = nullptr;
    const float4* lrow = nullptr;
    const float4* rcol = nullptr;
    const float4* srow = nullptr;  // separable line planes of the single-column tile apply
    const float4* scol = nullptr;
  };
  EmSplit em_split[2];
  const int* em_line_off = nullptr;
  int em_nlines = 0;
  const void* em_tma_tiles[3] = {nullptr, nullptr, nullptr};  // tile records, tiles of 16 / 32 / 64 rows
  int em_tma_ntiles[3] = {0, 0, 0};
  // Element-major kernel chosen by the autotuner (or pinned by the caller) per batch width
  // and coordinate system: kind 0 TMA-staged with tiles of `rows` rows, 1 plain loads.
  struct EmChoice {
    int ncols, coords, kind, rows;
    double ms;  // timed duration of one apply (0 when pinned)
  };
  std::vector<EmChoice> em_choices;
  std::mutex em_tune_mu;
  // Single-instance solves run as one job of a batched engine kept with the plan (created on
  // first use for a Krylov dimension and basis precision, replaced when those change).
  picuda::Engine* engine = nullptr;
  int engine_m = 0;
  bool engine_f32 = false;
};

namespace picuda {

// Thread-local error message for pi_last_error.
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// RAII guard around one call on a plan: waits for the plan's other callers (default), or,
// when the plan was switched to rejection, fails at once (ok = false) while another thread
// holds it.
struct BusyGuard {
  pi_plan* p;
  bool ok;
  explicit BusyGuard(pi_plan* plan) : p(plan) {
    if (p->reject_concurrent.load()) {
      ok = p->call_mu.try_lock();
    } else {
      p->call_mu.lock();
      ok = true;
    }
  }
  ~BusyGuard() {
    if (ok) p->call_mu.unlock();
  }
};

// Device allocation tracked by the plan; returns nullptr on failure.
void* plan_alloc(pi_plan* plan, size_t bytes);

// Split coefficient planes of a canonical plan in reference (which 0) or population (which 1)
// FP32 coordinates, built on first use (pi_apply_em.cu); PI_ERR_UNSUPPORTED for a plan whose
// stencil does not sit at the canonical positions.
int em_split_planes(pi_plan* plan, int which, SplitPlanes* out);

}  // namespace picuda
