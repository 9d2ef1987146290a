// Drive preconditioner of the trace-fixed steady-state GMRES (pi_drive.cu).
//
// Per Schur sector s the within-sector operator holds the Hamiltonian commutator -i[H_s, X],
// the loss anticommutator -(Q_s X + X Q_s)/2 and the sector's own sandwich gains.  In the
// orthogonal eigenbasis U_s of H_s (the sector's real symmetric tridiagonal Hamiltonian
// block, H_s = U_s diag(h) U_s^T) the commutator is diagonal and the loss is kept as its
// diagonal part, the loss q_i = (U_s^T Q_s U_s)_ii each eigenmode sees (floored at half the
// sector's mean loss); that operator is solved exactly:
//   X = U_s [ (U_s^T R U_s) ./ d ] U_s^T,   d_ij = (-i (h_i - h_j) - (q_i + q_j) / 2) / s,
// and the trace border v t^H of the bordered operator L/s + v t^H is added by Sherman-Morrison
// over the whole block-diagonal map.  The loss variation along a sector, the sandwich gains and
// the coupling between sectors are left out: this part carries the drive exactly, which is what
// the charge-keeping level sweep (pi_precond.cu) leaves out.  No counterpart in the reference,
// whose Schur-sector preconditioner LU-factors every sector block densely (krylov.jl:594-699),
// n^2 x n^2 per sector and infeasible at N = 200.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pi_plan.hpp"

struct pi_plan;

namespace picuda {

struct DriveHost {
  int coords = 0;
  double scale = 1.0;
  std::vector<int> n;             // per sector: block dimension
  std::vector<long long> offset;  // per sector: element offset of the block
  std::vector<long long> u_off;   // per sector: offset of U_s (column-major, column i = eigenvector i)
  std::vector<long long> h_off;   // per sector: offset of its eigenvalues
  std::vector<double> c;          // per sector: c_s = -2 x mean loss (before the 1/s scaling)
  std::vector<double> U, h;       // pools
  std::vector<double> q;          // per eigenmode (pool like h): the loss it sees, floored
  double max_asymmetry = 0.0;     // largest |H_ab - H_ba| of the lowered Hamiltonian blocks
  double max_nonhermitian = 0.0;  // largest real part of a row-shift +-1 coefficient (left out)
};

// Symmetric tridiagonal eigendecomposition by implicit QL with shifts (the algorithm of
// Bowdler, Martin, Reinsch and Wilkinson, Numer. Math. 11 (1968) 293-306): d[0..n) the
// diagonal, e[0..n-1) the off-diagonal T[i][i+1] (e has n entries; e[n-1] is scratch).  On
// return d holds the eigenvalues and Z (n x n, column-major) the orthonormal eigenvectors
// (column i belongs to d[i]).  Returns false if an eigenvalue takes more than 60 iterations.
bool tridiag_eigen(int n, double* d, double* e, double* Z);

// Host tables of plan hp in coordinates `coords` (PI_COORDS_*) for operator scale `scale`;
// PI_OK or an error status with *err set.
int build_drive_precond(const QubitPlan& hp, int coords, double scale, DriveHost* out, std::string* err);

struct DriveState;
int drive_create(pi_plan* plan, int coords, double scale, DriveState** out, std::string* err);
// z = M^-1 r for M = blockdiag(A_s X + X A_s^H)/s + v t^H (one application), on `stream`; r
// and z both FP64 (FP64 arithmetic) or both FP32 (FP32 arithmetic).  Uses the state's scratch:
// one application at a time per state (the solves of a plan are serialised by the plan).
cudaError_t drive_apply(DriveState* D, const void* r, int r_f32, void* z, int z_f32, cudaStream_t stream);
void drive_free(DriveState* D);
size_t drive_bytes(const DriveState* D);
const DriveHost& drive_host(const DriveState* D);
double drive_setup_seconds(const DriveState* D);

}  // namespace picuda
