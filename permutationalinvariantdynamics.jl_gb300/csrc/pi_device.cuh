// Device-side plan layout shared by the apply and solver kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace picuda {

// One output sector of the stencil plan.
struct DevSector {
  long long offset;    // 0-based element offset of the column-major block
  int n;               // block dimension
  int term_begin;      // first stencil term
  int term_count;      // number of stencil terms
  int pad;
  double border_x;     // normalized trace vector v = t/|t|^2 on the diagonal, x coordinates
  double border_z;     // the same vector in population coordinates (f / |t|^2)
  double sqrt_f;       // sqrt(f^nu): z = sqrt_f * x
};

// One separable stencil term (see pi_plan.hpp).
struct DevTerm {
  long long src_off;   // block offset of the source sector
  int src_n;           // block dimension of the source sector
  int kind;            // 0 ADD, 1 LEFT, 2 RIGHT, 3 SAND
  int cls;             // 0 real, 1 imaginary, 2 complex combined coefficient
  int dr;              // row offset into the source block: e + p
  int dc;              // column offset into the source block: e + q
  int alpha_off;       // offset of alpha[0..n) in the coefficient pool
  int beta_off;        // offset of beta[0..n) in the coefficient pool
  int pad;
};

// Output tile: 32 rows x TILE_COLS columns of one sector block.
struct DevTile {
  int sector;
  int a0;
  int b0;
  int pad;
};

constexpr int kTileRows = 32;
constexpr int kTileCols = 8;
constexpr int kApplyThreads = kTileRows * kTileCols;

// Trace-border epilogue: y = scale * (L x) + border ? alpha * v : 0, where alpha is a
// device scalar t^H x computed beforehand (krylov.jl:855-860).
struct BorderArgs {
  double scale;            // multiplies L x (1/s in the bordered steady-state system)
  const double2* alpha;    // device complex scalar per column, or nullptr (no border)
  int coords;              // 0: x coordinates (border_x), 1: population coordinates (border_z)
};

}  // namespace picuda
