// Level-sweep preconditioner of the trace-fixed steady-state GMRES (pi_precond.cu): host
// tables, the device view the sweep kernel reads, and the calls the solver drivers use.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <string>
#include <vector>

#include "pi_plan.hpp"

struct pi_plan;
struct pi_precond;

namespace picuda {

// Sectors per level (the thread block's shared-memory level buffers): N <= 318.
constexpr int kPrecondMaxLevel = 160;

// Host tables.  Entries are ordered by charge chain d = b - a, then by level in sweep order,
// then by sector; every entry of the basis appears once.
struct LevelPrecondHost {
  int coords = 0;
  double scale = 1.0;
  double regularization = 0.0;
  int direction = -1;                  // -1: levels swept from high M to low M
  std::vector<int> chain_order;        // thread block -> chain (longest first)
  std::vector<int> chain_lev;          // chain -> first level record (size chains + 1)
  std::vector<int> lev_ent;            // level -> first entry (size levels + 1)
  std::vector<int> elem;               // entry -> element index of the PI vector
  std::vector<std::complex<double>> W, A, C;  // Thomas factors: y_i = W_i r_i + A_i y_{i-1}; u_i = y_i + C_i u_{i+1}
  std::vector<int> gsrc;               // entry -> three 10-bit positions in the previous level (1023: none)
  std::vector<std::complex<double>> G; // entry -> three gain coefficients
  int chain0 = -1;                     // the d = 0 chain (block diagonals)
  int chain0_ent = -1;                 // its first entry
  std::vector<double> t0, v0;          // trace weights and border vector over the d = 0 chain
  std::vector<std::complex<double>> w0;  // over the d = 0 chain: y_v (mode 0) or s L0^-1 v (mode 1)
  std::complex<double> sm_coef = 0.0;  // rho_v (mode 0) or 1 / (1 + t^H w0) (mode 1)
  int mode = 0;                        // 0: singular L0 with a free entry; 1: Sherman-Morrison
  int free_ent = -1;
  std::vector<long long> zero_pivots;
  int max_level = 0;
  double maxdiag = 0.0;
};

// Device view (pointers into the preconditioner's allocations).
struct PrecondDev {
  const int* chain_order;
  const int* chain_lev;
  const int* lev_ent;
  const int* elem;
  const int* gsrc;
  const void* W;  // T2 per entry (T = float or double)
  const void* A;
  const void* C;
  const void* G;  // 3 x T2 per entry
  const double* t0;
  const double* v0;
  const double2* w0;
  double2 sm_coef;
  int chain0;
  int chain0_ent;
  int free_ent;
  int mode;
};

// Builds the host tables of plan hp in the given coordinates (PI_COORDS_*) for operator scale
// `scale`; returns PI_OK or an error status with *err set.
int build_level_precond(const QubitPlan& hp, int coords, double regularization, double scale, LevelPrecondHost* out,
                        std::string* err);

// z = M^-1 r with M = L0/s + v t^H, on `stream`; r and z FP64 (x_f32 = 0) or FP32 (1).
cudaError_t precond_apply(const pi_precond* P, const void* r, int r_f32, void* z, int z_f32, double scale,
                          cudaStream_t stream);
int precond_coords(const pi_precond* P);
int precond_kind(const pi_precond* P);  // PI_PRECOND_LEVEL or PI_PRECOND_DRIVE
double precond_scale(const pi_precond* P);
const pi_plan* precond_plan(const pi_precond* P);

}  // namespace picuda
