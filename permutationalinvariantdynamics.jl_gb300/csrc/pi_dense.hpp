// Small dense complex linear algebra for the projected Krylov problems (host, FP64):
// the matrix exponential of the (m+1) x (m+1) Hessenberg matrix used by expv
// (krylov_extensions.jl:1412, Julia's LinearAlgebra.exp) and helpers.
//
// The exponential is an implementation of the scaling-and-squaring algorithm with
// [m/m] Pade approximants of N. J. Higham, "The scaling and squaring method for the
// matrix exponential revisited", SIAM J. Matrix Anal. Appl. 26 (2005) 1179-1193,
// Algorithm 2.3: degrees 3, 5, 7, 9, 13 chosen by the 1-norm against the published
// theta_m bounds; Pade coefficients b_j = (2m-j)! m! / ((2m)! j! (m-j)!).
#pragma once

#include <cmath>
#include <complex>
#include <stdexcept>
#include <vector>

namespace picuda {

using cd = std::complex<double>;

struct CMat {
  int n = 0;
  std::vector<cd> a;  // row-major
  CMat() = default;
  explicit CMat(int n_) : n(n_), a((size_t)n_ * n_, cd(0, 0)) {}
  cd& operator()(int i, int j) { return a[(size_t)i * n + j]; }
  const cd& operator()(int i, int j) const { return a[(size_t)i * n + j]; }
  static CMat identity(int n) {
    CMat m(n);
    for (int i = 0; i < n; ++i) m(i, i) = 1.0;
    return m;
  }
};

inline CMat matmul(const CMat& x, const CMat& y) {
  CMat r(x.n);
  for (int i = 0; i < x.n; ++i)
    for (int k = 0; k < x.n; ++k) {
      const cd xv = x(i, k);
      if (xv == cd(0, 0)) continue;
      for (int j = 0; j < x.n; ++j) r(i, j) += xv * y(k, j);
    }
  return r;
}

inline CMat lincomb(const CMat& x, cd a, const CMat& y, cd b) {
  CMat r(x.n);
  for (size_t i = 0; i < r.a.size(); ++i) r.a[i] = a * x.a[i] + b * y.a[i];
  return r;
}

inline double norm1(const CMat& x) {
  double best = 0.0;
  for (int j = 0; j < x.n; ++j) {
    double s = 0.0;
    for (int i = 0; i < x.n; ++i) s += std::abs(x(i, j));
    best = std::max(best, s);
  }
  return best;
}

// Solves P X = Q by LU with partial pivoting.
inline CMat solve(CMat P, CMat Q) {
  const int n = P.n;
  for (int k = 0; k < n; ++k) {
    int piv = k;
    double best = std::abs(P(k, k));
    for (int i = k + 1; i < n; ++i)
      if (std::abs(P(i, k)) > best) {
        best = std::abs(P(i, k));
        piv = i;
      }
    if (best == 0.0) throw std::runtime_error("singular Pade denominator");
    if (piv != k) {
      for (int j = 0; j < n; ++j) {
        std::swap(P(k, j), P(piv, j));
        std::swap(Q(k, j), Q(piv, j));
      }
    }
    for (int i = k + 1; i < n; ++i) {
      const cd f = P(i, k) / P(k, k);
      if (f == cd(0, 0)) continue;
      for (int j = k; j < n; ++j) P(i, j) -= f * P(k, j);
      for (int j = 0; j < n; ++j) Q(i, j) -= f * Q(k, j);
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    for (int j = 0; j < n; ++j) {
      cd s = Q(k, j);
      for (int i = k + 1; i < n; ++i) s -= P(k, i) * Q(i, j);
      Q(k, j) = s / P(k, k);
    }
  }
  return Q;
}

inline std::vector<double> pade_coefficients(int m) {
  std::vector<double> b(m + 1);
  // b_j = (2m-j)! m! / ((2m)! j! (m-j)!) evaluated as a running product
  b[0] = 1.0;
  for (int j = 1; j <= m; ++j) b[j] = b[j - 1] * (double)(m - j + 1) / ((double)j * (double)(2 * m - j + 1));
  return b;
}

inline CMat expm(const CMat& A0) {
  const int n = A0.n;
  static const double theta[5] = {1.495585217958292e-2, 2.539398330063230e-1, 9.504178996162932e-1,
                                  2.097847961257068e0, 5.371920351148152e0};
  static const int degrees[5] = {3, 5, 7, 9, 13};
  const double nrm = norm1(A0);
  const CMat I = CMat::identity(n);
  for (int d = 0; d < 4; ++d) {
    if (nrm <= theta[d]) {
      const int m = degrees[d];
      const auto b = pade_coefficients(m);
      const CMat A2 = matmul(A0, A0);
      CMat U_in = lincomb(I, b[1], I, 0.0), V = lincomb(I, b[0], I, 0.0);
      CMat P = I;
      for (int k = 2; k <= m; k += 2) {
        P = matmul(P, A2);
        U_in = lincomb(U_in, 1.0, P, b[k + 1]);
        V = lincomb(V, 1.0, P, b[k]);
      }
      const CMat U = matmul(A0, U_in);
      return solve(lincomb(V, 1.0, U, -1.0), lincomb(V, 1.0, U, 1.0));
    }
  }
  int s = 0;
  if (nrm > theta[4]) s = (int)std::ceil(std::log2(nrm / theta[4]));
  if (s < 0) s = 0;
  const double scale = std::ldexp(1.0, -s);
  CMat A(n);
  for (size_t i = 0; i < A.a.size(); ++i) A.a[i] = A0.a[i] * scale;
  const auto b = pade_coefficients(13);
  const CMat A2 = matmul(A, A), A4 = matmul(A2, A2), A6 = matmul(A4, A2);
  CMat U1(n), V1(n);
  for (size_t i = 0; i < U1.a.size(); ++i) {
    U1.a[i] = b[13] * A6.a[i] + b[11] * A4.a[i] + b[9] * A2.a[i];
    V1.a[i] = b[12] * A6.a[i] + b[10] * A4.a[i] + b[8] * A2.a[i];
  }
  CMat U2 = matmul(A6, U1), V2 = matmul(A6, V1);
  for (size_t i = 0; i < U2.a.size(); ++i) {
    U2.a[i] += b[7] * A6.a[i] + b[5] * A4.a[i] + b[3] * A2.a[i] + b[1] * I.a[i];
    V2.a[i] += b[6] * A6.a[i] + b[4] * A4.a[i] + b[2] * A2.a[i] + b[0] * I.a[i];
  }
  const CMat U = matmul(A, U2);
  CMat X = solve(lincomb(V2, 1.0, U, -1.0), lincomb(V2, 1.0, U, 1.0));
  for (int k = 0; k < s; ++k) X = matmul(X, X);
  return X;
}

// Complex Givens rotation (krylov.jl:710-716).
inline void complex_givens(cd a, cd b, double* c, cd* s) {
  if (b == cd(0, 0)) {
    *c = 1.0;
    *s = cd(0, 0);
    return;
  }
  if (a == cd(0, 0)) {
    *c = 0.0;
    *s = cd(1, 0);
    return;
  }
  const double scale = std::abs(a) + std::abs(b);
  const double normab = scale * std::sqrt(std::norm(a / scale) + std::norm(b / scale));
  const cd alpha = a / std::abs(a);
  *c = std::abs(a) / normab;
  *s = alpha * std::conj(b) / normab;
}

}  // namespace picuda
