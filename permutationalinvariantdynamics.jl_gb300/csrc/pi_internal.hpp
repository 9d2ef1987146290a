// Internal interfaces between the C ABI, the kernels and the solver drivers.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <string>

#include "pi_device.cuh"

namespace picuda {

// Device copies of one plan's tables (owned by pi_plan).
struct DevicePlan {
  const DevSector* sectors = nullptr;
  const DevTerm* terms = nullptr;
  const DevTile* tiles = nullptr;
  const double2* coef64 = nullptr;   // coefficients in reference coordinates
  const double2* coef64z = nullptr;  // FP64 coefficients in population coordinates
  const float2* coef32x = nullptr;   // FP32 coefficients in reference coordinates
  const float2* coef32z = nullptr;   // FP32 coefficients in population coordinates
  const int* diag_sector = nullptr;  // per diagonal entry: its sector
  const long long* diag_index = nullptr;  // per diagonal entry: its element index
  const int4* fterms = nullptr;     // padded fixed-structure term table (batched apply)
  int fast_sr = 0;                   // real sandwich terms per sector of the fixed structure (0: none)
  const int4* canon = nullptr;      // canonical-position table (kCanonEntries per sector) or null
  int canon_plus = 0;                // some sandwich term sits at the +1 diagonal shift
  int nsectors = 0;
  int ntiles = 0;
  int ndiag = 0;
  long long dim = 0;
};

// Applies with at least this many right-hand sides use the fixed-structure batched kernel
// when the plan has one.
constexpr int kFastMinCols = 2;

// Canonical-position table: ADD, LEFT(p = -1, +1), RIGHT(q = -1, +1), then per source slot
// and diagonal shift p = q = -1, 0, +1 up to kCanonPerPos real sandwich terms.
constexpr int kCanonPerPos = 3;
constexpr int kCanonEntries = 5 + 9 * kCanonPerPos;  // 32

// Apply kernels (pi_apply.cu).  Both take border.coords: reference (0) or population (1)
// coordinates.
cudaError_t launch_apply_f64(const DevicePlan& dp, const double* x, double* y, int ncols, long long ld,
                             const BorderArgs& border, cudaStream_t stream);
// FP32 action; border.coords selects reference (0) or population (1) coordinates.
cudaError_t launch_apply_f32(const DevicePlan& dp, const float* x, float* y, int ncols, long long ld,
                             const BorderArgs& border, cudaStream_t stream);

// Reduction workspace used by the linear-algebra kernels (pi_linalg.cu).
struct ReduceScratch {
  double2* partial = nullptr;  // [kReduceBlocks][kMaxDots]
  double2* result = nullptr;   // [kMaxDots]
  double* rpartial = nullptr;  // [kReduceBlocks]
  double* rresult = nullptr;   // [4]
};
constexpr int kReduceBlocks = 608;   // 4 x 152 SMs
constexpr int kReduceThreads = 256;
constexpr int kMaxDots = 128;

// h[i] = sum_e conj(V_i[e]) w[e] for i < nv (FP64 inputs, FP64 accumulation).
cudaError_t mdot_f64(const double2* V, long long ldv, int nv, const double2* w, long long n,
                     ReduceScratch& rs, double2* h_out, cudaStream_t stream);
// w[e] -= sum_i V_i[e] h[i]; optional sum |w|^2 into rs.rresult[slot].
cudaError_t maxpy_f64(const double2* V, long long ldv, int nv, const double2* h, double2* w, long long n,
                      ReduceScratch& rs, int norm_slot, cudaStream_t stream);
// sum |w|^2 -> rs.rresult[slot]
cudaError_t norm2_f64(const double2* w, long long n, ReduceScratch& rs, int slot, cudaStream_t stream);
// y = a * x (+ y if accumulate)
cudaError_t scale_f64(const double2* x, double2* y, long long n, double2 a, int accumulate,
                      cudaStream_t stream);
// y = sum_i c[i] V_i (c on device, complex)
cudaError_t combine_f64(const double2* V, long long ldv, int nv, const double2* c, double2* y, long long n,
                        int accumulate, cudaStream_t stream);
// out = t^H x over the block diagonals (x coordinates weight sqrt_f, z coordinates weight 1)
cudaError_t trace_dot(const DevicePlan& dp, const void* x, int is_f32, int coords, double2* out,
                      cudaStream_t stream);

// Mixed precision (FP32 storage): dots and norms accumulate in double-float (FP32 pairs,
// ~48-bit significand) on the FP32 pipes; basis updates run in FP32.
cudaError_t mdot_f32(const float2* V, long long ldv, int nv, const float2* w, long long n,
                     ReduceScratch& rs, double2* h_out, cudaStream_t stream);
cudaError_t maxpy_f32(const float2* V, long long ldv, int nv, const double2* h, float2* w, long long n,
                      ReduceScratch& rs, int norm_slot, cudaStream_t stream);
cudaError_t norm2_f32(const float2* w, long long n, ReduceScratch& rs, int slot, cudaStream_t stream);
cudaError_t scale_f32(const float2* x, float2* y, long long n, double2 a, cudaStream_t stream);
// FP64 combination of FP32 basis vectors into an FP64 vector: y (+)= sum_i c[i] V_i
cudaError_t combine_f32_to_f64(const float2* V, long long ldv, int nv, const double2* c, double2* y,
                               long long n, int accumulate, cudaStream_t stream);
// Coordinate changes between x (reference, FP64) and z = sqrt(f) x.
cudaError_t x_to_z_f64(const DevicePlan& dp, const double2* x, double2* z, double scale, cudaStream_t stream);
cudaError_t z_to_x_f64(const DevicePlan& dp, const double2* z, double2* x, double scale, int accumulate,
                       cudaStream_t stream);
cudaError_t f64_to_f32(const double2* x, float2* y, long long n, double scale, cudaStream_t stream);
cudaError_t x_to_z_f32(const DevicePlan& dp, const double2* x, float2* z, double scale, cudaStream_t stream);
// sum over sectors of (1/f_s) |z_s|^2 : the reference-coordinate norm of a z vector
cudaError_t weighted_norm2_z(const DevicePlan& dp, const double2* z, ReduceScratch& rs, int slot,
                             cudaStream_t stream);

}  // namespace picuda
