// Host-side lowering of a qubit PI model into the device stencil plan.
//
// This is the native replacement for the reference's compile step
// (src/liouvillian.jl:1290-1371 compile_term, :1700-1738 _fuse_fixed_kernels,
// src/geometry.jl:405-562 one-body geometry, :840-865 collective blocks).  It keeps the
// reference's exact-rational Clebsch-Gordan route (src/cgc.jl:6-39) and branch weights
// (src/partitions.jl:519-543), then rewrites the fused Schur-block operator as a list of
// separable stencil terms per output sector:
//
//   y_s[a,b] += alpha[a] * beta[b] * x_src[a + e + p, b + e + q]      (kind SAND/LEFT/RIGHT)
//   y_s[a,b] += (alpha[a] + beta[b]) * x_s[a, b]                        (kind ADD)
//
// where e = j_src - j_s aligns equal magnetic quantum numbers between sectors.
#pragma once

#include <complex>
#include <cstdint>
#include <string>
#include <vector>

namespace picuda {

using cd = std::complex<double>;

enum TermKind : int { TERM_HAMILTONIAN = 0, TERM_LOCAL_JUMP = 1, TERM_COLLECTIVE_JUMP = 2 };

struct TermSpec {
  int kind = TERM_HAMILTONIAN;
  cd op[2][2];  // op[i][j]: row i, column j; level 0 = |g>, level 1 = |e>
  double rate = 1.0;
  double hbar = 1.0;
};

enum StencilKind : int { ST_ADD = 0, ST_LEFT = 1, ST_RIGHT = 2, ST_SAND = 3 };
enum CoefClass : int { CC_REAL = 0, CC_IMAG = 1, CC_CPLX = 2 };

struct StencilTerm {
  int src = 0;         // source sector (index into the plan's sector list)
  int kind = ST_SAND;  // StencilKind
  int cls = CC_CPLX;   // CoefClass of the combined coefficient
  int e = 0;           // index alignment j_src - j_out
  int p = 0, q = 0;    // row / column offsets
  std::vector<cd> alpha;  // length n_out (unused for ST_RIGHT)
  std::vector<cd> beta;   // length n_out (unused for ST_LEFT)
};

struct Sector {
  int k = 0;               // partition (N-k, k)
  int n = 0;               // block dimension N - 2k + 1
  long long offset = 0;    // 0-based element offset of the column-major block
  double f = 1.0;          // f^lambda rounded to double
  double sqrt_f = 1.0;     // sqrt(f^lambda)
  std::vector<StencilTerm> terms;
};

struct QubitPlan {
  int N = 0;
  long long dim = 0;
  std::vector<Sector> sectors;
  double trace_norm2 = 0.0;  // sum_s n_s f_s = ||t||^2
  int max_terms = 0;
  int max_n = 0;
};

// Builds the plan.  ks lists the retained sectors as k values (partition (N-k, k)),
// in any order; they are sorted into the reference's descending partition order.
// Throws std::invalid_argument on unsupported input.
QubitPlan build_qubit_plan(int N, std::vector<int> ks, const std::vector<TermSpec>& terms);

// Exact f^(N-k,k) as a decimal string (for tests of the combinatorics).
std::string symmetric_group_dimension_decimal(int N, int k);
// f^(N-k,k) correctly rounded to double.
double sector_multiplicity_double(int N, int k);

// Exact squared CG coefficient and sign for d = 2 (child pattern entries {m, mu1, mu2},
// local label j, parent {m', lam1, lam2}); returns false for a structural zero.
bool cgc_qubit_exact(const int child[3], int j, const int parent[3], int* sign, long long* num,
                     long long* den);

// Collective block of sum_i X_i in sector k of an N-qubit basis, dense column-major n x n.
std::vector<cd> collective_block_dense(int N, int k, const cd X[2][2]);

}  // namespace picuda
