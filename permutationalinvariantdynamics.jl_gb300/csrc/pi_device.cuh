// Device-side plan layout shared by the apply and solver kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace picuda {

// Stencil term groups, in the order the apply kernel walks them: every group runs one
// branch-free code path (kind = how the separable coefficient combines, class = whether it
// is real, imaginary or complex).
enum TermGroup : int {
  G_ADD = 0,      // (alpha[a] + beta[b]) x[a, b]
  G_LEFT_IM,      // i Im(alpha[a]) x[a + dr, b]
  G_LEFT_RE,      // Re(alpha[a]) x[a + dr, b]
  G_LEFT_CX,      // alpha[a] x[a + dr, b]
  G_RIGHT_IM,     // i Im(beta[b]) x[a, b + dc]
  G_RIGHT_RE,
  G_RIGHT_CX,
  G_SAND_RE,      // Re(alpha[a]) Re(beta[b]) x[a + dr, b + dc]
  G_SAND_CX,      // alpha[a] beta[b] x[a + dr, b + dc]
  G_COUNT
};

// One output sector of the stencil plan.
struct DevSector {
  long long offset;    // 0-based element offset of the column-major block
  int n;               // block dimension
  int term_begin;      // first stencil term (terms are stored group by group)
  int group_end[G_COUNT];  // absolute end index of each group
  int src[3];          // source sector for index shift e = j_src - j_out = -1, 0, +1 (-1: none)
  double border_x;     // normalized trace vector v = t/|t|^2 on the diagonal, x coordinates
  double border_z;     // the same vector in population coordinates (f / |t|^2)
  double sqrt_f;       // sqrt(f^nu): z = sqrt_f * x
};

// One separable stencil term (see pi_plan.hpp); its group fixes kind and class.  The
// source entry x_src[a + e + p, b + e + q] is read from the staged window of slot e + 1.
struct DevTerm {
  int woff;            // (e+1)*kWinElems + p + q*kWinRows: offset into the staged windows
  int alpha_off;       // offset of alpha[0..n) in the coefficient pool (0 when unused)
  int beta_off;        // offset of beta[0..n) in the coefficient pool, a multiple of 4
  int pad;
};

// Output tile: 32 rows x 32 columns of one sector block; each of the 8 warps owns 4
// consecutive columns and each lane one row.
struct DevTile {
  int sector;
  int a0;
  int b0;
  int pad;
};

constexpr int kTileRows = 32;
constexpr int kColsPerThread = 4;
constexpr int kApplyWarps = 8;
constexpr int kTileCols = kColsPerThread * kApplyWarps;
constexpr int kApplyThreads = 32 * kApplyWarps;
constexpr int kMaxSectorTerms = 128;  // stencil terms of one sector staged in shared memory
constexpr int kHalo = 2;                // band half-width of every stencil term
constexpr int kWinRows = kTileRows + 2 * kHalo;
constexpr int kWinCols = kTileCols + 2 * kHalo;
constexpr int kWinElems = kWinRows * kWinCols;

// Trace-border epilogue: y = scale * (L x) + border ? alpha * v : 0, where alpha is a
// device scalar t^H x computed beforehand (krylov.jl:855-860).
struct BorderArgs {
  double scale;            // multiplies L x (1/s in the bordered steady-state system)
  const double2* alpha;    // device complex scalar per column, or nullptr (no border)
  int coords;              // 0: x coordinates (border_x), 1: population coordinates (border_z)
};

// Split coefficient planes of a plan whose stencil sits at the canonical positions (built by
// the element-major apply): per entry (centre re, centre im, own (-1,-1), smaller (-2,-2)),
// (smaller (-1,-1), larger (0,0), larger (1,1), own (1,1)) [, (smaller (0,0), larger (2,2))];
// per row (LEFT -1, LEFT +1); per column (RIGHT -1, RIGHT +1).
struct SplitPlanes {
  const float4* eplane;
  const float4* lrow;
  const float4* rcol;
  const int* line_off;  // per sector: start of its row and column planes
  int plus;             // three entry float4 (pumping terms at the +1 diagonal shifts)
  // Separable line planes (kSepF4 or kSepF4Plus float4 per row and per column): every merged
  // coefficient is (alpha_add[a] + beta_add[b]) or a sum of at most three real products
  // alpha_t[a] beta_t[b], so a single-column tile rebuilds it from its row's and column's
  // factors instead of streaming 32-48 bytes per entry.  Row floats: alpha_add (re, im),
  // LEFT -1 (re, im), LEFT +1 (re, im), then alpha_t of the sandwich positions own centre,
  // own (-1,-1), smaller (-2,-2), smaller (-1,-1), larger (0,0), larger (1,1)[, own (1,1),
  // smaller (0,0), larger (2,2)], three terms each; column floats the same with beta_add,
  // RIGHT -1, RIGHT +1 and beta_t.
  const float4* srow;
  const float4* scol;
};

constexpr int kSepF4 = 6;      // 24 floats: 6 + 3 x 6 positions
constexpr int kSepF4Plus = 9;  // 36 floats: 6 + 3 x 9 positions, padded

}  // namespace picuda
