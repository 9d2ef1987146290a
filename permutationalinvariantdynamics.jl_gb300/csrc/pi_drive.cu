// Drive preconditioner: per-sector normal-part Lyapunov solves through the eigenvectors of
// the sector Hamiltonian blocks, plus the trace border by Sherman-Morrison (see pi_drive.hpp).
#include "pi_drive.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <limits>
#include <thread>

#include "../../include/picuda.h"
#include "pi_handle.hpp"
#include "pi_internal.hpp"

namespace picuda {

bool tridiag_eigen(int n, double* d, double* e, double* Z) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) Z[i + (size_t)j * n] = i == j ? 1.0 : 0.0;
  if (n <= 1) return true;
  e[n - 1] = 0.0;
  const double eps = std::numeric_limits<double>::epsilon();
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      int m = l;
      for (; m < n - 1; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= eps * dd) break;
      }
      if (m == l) break;
      if (++iter > 60) return false;
      // shift: the eigenvalue of the leading 2 x 2 block at l nearer to d[l]
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
      double s = 1.0, c = 1.0, p = 0.0;
      bool split = false;
      for (int i = m - 1; i >= l; --i) {
        double f = s * e[i];
        const double b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // the rotation underflowed: the matrix splits at i + 1
          d[i + 1] -= p;
          e[m] = 0.0;
          split = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        double* zi = Z + (size_t)i * n;
        double* zj = Z + (size_t)(i + 1) * n;
        for (int k = 0; k < n; ++k) {
          const double t = zj[k];
          zj[k] = s * zi[k] + c * t;
          zi[k] = c * zi[k] - s * t;
        }
      }
      if (split) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  return true;
}

int build_drive_precond(const QubitPlan& hp, int coords, double scale, DriveHost* out, std::string* err) {
  DriveHost& D = *out;
  D = DriveHost{};
  const int S = (int)hp.sectors.size();
  if (S < 1) {
    *err = "empty basis";
    return PI_ERR_INVALID_ARGUMENT;
  }
  if (!(std::isfinite(scale) && scale > 0)) {
    *err = "operator_scale must be finite and positive";
    return PI_ERR_INVALID_ARGUMENT;
  }
  D.coords = coords;
  D.scale = scale;
  D.n.resize(S);
  D.offset.resize(S);
  D.u_off.resize(S);
  D.h_off.resize(S);
  D.c.resize(S);
  long long uo = 0, ho = 0;
  for (int s = 0; s < S; ++s) {
    D.n[s] = hp.sectors[s].n;
    D.offset[s] = hp.sectors[s].offset;
    D.u_off[s] = uo;
    D.h_off[s] = ho;
    uo += (long long)D.n[s] * D.n[s];
    ho += D.n[s];
  }
  D.U.assign(uo, 0.0);
  D.h.assign(ho, 0.0);
  D.q.assign(ho, 0.0);
  // per sector: the Hamiltonian block from the own-sector stencil terms
  std::vector<std::vector<double>> diag(S), off(S), loss(S);
  for (int s = 0; s < S; ++s) {
    const int n = D.n[s];
    std::vector<cd> al(n, 0.0), be(n, 0.0);
    std::vector<double> up(n, 0.0), dn(n, 0.0);  // H[a][a+1] from row shift +1, H[a][a-1] from -1
    for (const StencilTerm& t : hp.sectors[s].terms) {
      if (t.src != s || t.e != 0 || t.q != 0) continue;
      if (t.p == 0) {
        if (t.kind == ST_ADD) {
          for (int a = 0; a < n; ++a) {
            al[a] += t.alpha[a];
            be[a] += t.beta[a];
          }
        } else if (t.kind == ST_LEFT) {
          for (int a = 0; a < n; ++a) al[a] += t.alpha[a];
        } else if (t.kind == ST_RIGHT) {
          for (int a = 0; a < n; ++a) be[a] += t.beta[a];
        }
      } else if ((t.p == 1 || t.p == -1) && t.kind == ST_LEFT) {
        // -i H[a][a+p] x[a+p, b]: H[a][a+p] = Re(i c) = -Im(c); Re(c) would be a
        // non-Hermitian row coupling (not part of the normal part)
        for (int a = 0; a < n; ++a) {
          if (a + t.p < 0 || a + t.p >= n) continue;
          const cd c = t.alpha[a];
          (t.p == 1 ? up : dn)[a] += -c.imag();
          D.max_nonhermitian = std::max(D.max_nonhermitian, std::fabs(c.real()));
        }
      }
    }
    diag[s].resize(n);
    off[s].assign(n, 0.0);
    loss[s].resize(n);
    double mre = 0.0;
    for (int a = 0; a < n; ++a) {
      // -i h_a in alpha and +i h_b in beta, up to a constant split that cancels in h_i - h_j
      diag[s][a] = 0.5 * (-al[a].imag() + be[a].imag());
      mre += al[a].real() + be[a].real();
      loss[s][a] = -(al[a].real() + be[a].real());  // q_a: the split's constant cancels at a = b
    }
    for (int a = 0; a + 1 < n; ++a) {
      off[s][a] = 0.5 * (up[a] + dn[a + 1]);
      D.max_asymmetry = std::max(D.max_asymmetry, std::fabs(up[a] - dn[a + 1]));
    }
    // mean of the pointwise loss coefficient alpha_a + beta_b over the block is mre / n;
    // c_s = 2 x that mean = -2 x the mean loss
    double c = 2.0 * mre / n;
    // a sector without loss has a singular normal part: keep a shift of 1e-6 s
    c = std::min(c, -1e-6 * scale);
    D.c[s] = c;
  }
  // eigendecompositions, sectors spread over the host threads
  std::atomic<int> next{0};
  std::atomic<int> failed{-1};
  auto worker = [&]() {
    std::vector<double> d, e;
    for (int s = next.fetch_add(1); s < S; s = next.fetch_add(1)) {
      const int n = D.n[s];
      d = diag[s];
      e = off[s];
      const double* U = D.U.data() + D.u_off[s];
      if (!tridiag_eigen(n, d.data(), e.data(), D.U.data() + D.u_off[s])) failed.store(s);
      std::copy(d.begin(), d.end(), D.h.begin() + D.h_off[s]);
      // the loss each eigenmode sees, (U^T Q U)_ii, floored at half the mean loss -c_s / 2
      const double floor_q = -0.25 * D.c[s];
      for (int i = 0; i < n; ++i) {
        double qi = 0.0;
        for (int a = 0; a < n; ++a) qi += U[a + (size_t)i * n] * U[a + (size_t)i * n] * loss[s][a];
        D.q[D.h_off[s] + i] = std::max(qi, floor_q);
      }
    }
  };
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  for (unsigned i = 1; i < hw; ++i) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  if (failed.load() >= 0) {
    *err = "the eigendecomposition of a sector Hamiltonian block did not converge";
    return PI_ERR_NOT_CONVERGED;
  }
  return PI_OK;
}

// ---------------------------------------------------------------------------------------
// Device side
// ---------------------------------------------------------------------------------------

namespace {

constexpr int kDT = 32;  // tile edge: lane = row, 8 warps x 4 columns

template <typename T>
struct Cx;
template <>
struct Cx<float> {
  using type = float2;
};
template <>
struct Cx<double> {
  using type = double2;
};

// Tables of one arithmetic precision T.
template <typename T>
struct DriveDev {
  const int4* tiles;        // (sector, i0, j0, 0)
  const int* n;
  const long long* offset;
  const long long* u_off;
  const long long* h_off;
  const T* U;
  const T* h;               // eigenvalues / s
  const T* q;               // per eigenmode: its loss / s
};

template <typename T2>
__device__ __forceinline__ T2 cvt2(float2 v);
template <>
__device__ __forceinline__ float2 cvt2<float2>(float2 v) { return v; }
template <typename T2>
__device__ __forceinline__ T2 cvt2(double2 v);
template <>
__device__ __forceinline__ float2 cvt2<float2>(double2 v) { return make_float2((float)v.x, (float)v.y); }
template <>
__device__ __forceinline__ double2 cvt2<double2>(double2 v) { return v; }

// One 32 x 32 tile of a sector product with the real eigenvector matrix U (n x n), in
// arithmetic T:  LEFT: C = op(U) B,  RIGHT: C = B op(U),  op(U) = U^T when TRANS;
// B and C complex n x n column-major at the sector's offset; DIVIDE divides C[i][j] by
// d_ij = -(q_i + q_j)/(2 s) - i (h_i - h_j)/s.
template <typename T, bool RIGHT, bool TRANS, bool DIVIDE, typename TI, typename TO>
__global__ void __launch_bounds__(256) k_drive_mm(DriveDev<T> D, const TI* __restrict__ in, TO* __restrict__ out) {
  using T2 = typename Cx<T>::type;
  __shared__ T sU[kDT][kDT + 1];
  __shared__ T2 sB[kDT][kDT + 1];
  const int4 tl = D.tiles[blockIdx.x];
  const int s = tl.x, i0 = tl.y, j0 = tl.z;
  const int n = D.n[s];
  const long long off = D.offset[s];
  const T* U = D.U + D.u_off[s];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const T2 zero{0, 0};
  T2 acc[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) acc[c] = zero;
  for (int k0 = 0; k0 < n; k0 += kDT) {
    for (int q = w; q < kDT; q += 8) {
      if (!RIGHT) {
        // sU[kk][ii] = op(U)(i0 + ii, k0 + kk); sB[kk][jj] = B(k0 + kk, j0 + jj)
        if (TRANS) {  // U[k][i]: contiguous in k
          const int k = k0 + lane, i = i0 + q;
          sU[lane][q] = (k < n && i < n) ? U[k + (long long)i * n] : T(0);
        } else {      // U[i][k]: contiguous in i
          const int i = i0 + lane, k = k0 + q;
          sU[q][lane] = (k < n && i < n) ? U[i + (long long)k * n] : T(0);
        }
        const int k = k0 + lane, j = j0 + q;
        sB[lane][q] = (k < n && j < n) ? cvt2<T2>(in[off + k + (long long)j * n]) : zero;
      } else {
        // sB[ii][kk] = B(i0 + ii, k0 + kk); sU[kk][jj] = op(U)(k0 + kk, j0 + jj)
        const int i = i0 + lane, k = k0 + q;
        sB[lane][q] = (i < n && k < n) ? cvt2<T2>(in[off + i + (long long)k * n]) : zero;
        if (TRANS) {  // U[j][k]: contiguous in j
          const int j = j0 + lane, kk = k0 + q;
          sU[q][lane] = (j < n && kk < n) ? U[j + (long long)kk * n] : T(0);
        } else {      // U[k][j]: contiguous in k
          const int kk = k0 + lane, j = j0 + q;
          sU[lane][q] = (j < n && kk < n) ? U[kk + (long long)j * n] : T(0);
        }
      }
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kDT; ++kk) {
      if (!RIGHT) {
        const T a = sU[kk][lane];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const T2 b = sB[kk][4 * w + c];
          acc[c].x = fma(a, b.x, acc[c].x);
          acc[c].y = fma(a, b.y, acc[c].y);
        }
      } else {
        const T2 b = sB[lane][kk];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const T a = sU[kk][4 * w + c];
          acc[c].x = fma(a, b.x, acc[c].x);
          acc[c].y = fma(a, b.y, acc[c].y);
        }
      }
    }
    __syncthreads();
  }
  const int i = i0 + lane;
  if (i >= n) return;
  const T* h = D.h + D.h_off[s];
  const T* q = D.q + D.h_off[s];
  const T hi = DIVIDE ? h[i] : T(0);
  const T qi = DIVIDE ? q[i] : T(0);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int j = j0 + 4 * w + c;
    if (j >= n) break;
    T2 v = acc[c];
    if (DIVIDE) {
      // v / (dr - i dm) = v (dr + i dm) / (dr^2 + dm^2), dr = -(q_i + q_j)/2, dm = h_i - h_j
      const T dm = hi - h[j];
      const T dr = T(-0.5) * (qi + q[j]);
      const T inv = T(1) / fma(dr, dr, dm * dm);
      v = T2{(v.x * dr - v.y * dm) * inv, (v.x * dm + v.y * dr) * inv};
    }
    out[off + i + (long long)j * n] = cvt2<TO>(v);
  }
}

// z -= Dv (t^H z) / den, with t^H z read from the device scalar `alpha`; in z's precision.
template <typename T2>
__global__ void k_drive_border(T2* __restrict__ z, const T2* __restrict__ dv, const double2* __restrict__ alpha,
                               double2 inv_den, long long n) {
  const double2 a = *alpha;
  const double gr = a.x * inv_den.x - a.y * inv_den.y, gi = a.x * inv_den.y + a.y * inv_den.x;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const T2 d = dv[e];
    T2 v = z[e];
    v.x -= d.x * gr - d.y * gi;
    v.y -= d.x * gi + d.y * gr;
    z[e] = v;
  }
}

// v = t / |t|^2 on the diagonal entries, zero elsewhere (the caller zeroes v first).
template <typename T2>
__global__ void k_drive_fill_border(const DevSector* __restrict__ sectors, const int* __restrict__ diag_sector,
                                    const long long* __restrict__ diag_index, int ndiag, T2* __restrict__ v,
                                    int coords) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndiag; i += gridDim.x * blockDim.x) {
    const DevSector& sec = sectors[diag_sector[i]];
    v[diag_index[i]] = cvt2<T2>(make_double2(coords ? sec.border_z : sec.border_x, 0.0));
  }
}

inline int grid_for(long long n) { return (int)std::max(1LL, std::min((n + 255) / 256, 4LL * 152)); }

// One arithmetic precision's device state: tables, scratch, the border vector D^-1 v.
template <typename T>
struct Chain {
  using T2 = typename Cx<T>::type;
  DriveDev<T> dev{};
  T2* t1 = nullptr;
  T2* t2 = nullptr;
  T2* dv = nullptr;
  double2 inv_den{1.0, 0.0};
};

}  // namespace

struct DriveState {
  pi_plan* plan = nullptr;
  DriveHost host;
  int ntiles = 0;
  long long dim = 0;
  Chain<float> c32;    // FP32 vectors: FP32 arithmetic
  Chain<double> c64;   // FP64 vectors: FP64 arithmetic
  double2* alpha = nullptr;
  std::vector<void*> allocs;
  size_t bytes = 0;
  double setup_seconds = 0.0;
};

namespace {

cudaError_t dalloc(DriveState* D, size_t bytes, void** p) {
  *p = nullptr;
  cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
  if (e != cudaSuccess) return e;
  D->allocs.push_back(*p);
  D->bytes += std::max<size_t>(bytes, 16);
  return cudaSuccess;
}

template <typename X>
cudaError_t upload(DriveState* D, const std::vector<X>& v, const X** out) {
  void* p = nullptr;
  cudaError_t e = dalloc(D, sizeof(X) * v.size(), &p);
  if (e != cudaSuccess) return e;
  if (!v.empty()) e = cudaMemcpy(p, v.data(), sizeof(X) * v.size(), cudaMemcpyHostToDevice);
  *out = (const X*)p;
  return e;
}

// out = D_blockdiag^-1 in (no border), in the chain's arithmetic
template <typename T, typename TI, typename TO>
cudaError_t block_solve(DriveState* D, Chain<T>& C, const TI* in, TO* out, cudaStream_t st) {
  using T2 = typename Cx<T>::type;
  const int g = D->ntiles;
  k_drive_mm<T, false, true, false, TI, T2><<<g, 256, 0, st>>>(C.dev, in, C.t1);     // U^T R
  k_drive_mm<T, true, false, true, T2, T2><<<g, 256, 0, st>>>(C.dev, C.t1, C.t2);    // (.) U ./ d
  k_drive_mm<T, false, false, false, T2, T2><<<g, 256, 0, st>>>(C.dev, C.t2, C.t1);  // U (.)
  k_drive_mm<T, true, true, false, T2, TO><<<g, 256, 0, st>>>(C.dev, C.t1, out);     // (.) U^T
  return cudaGetLastError();
}

// Uploads one precision's tables and scratch, forms D^-1 v and 1 / (1 + t^H D^-1 v).
template <typename T>
int setup_chain(DriveState* D, Chain<T>& C, const std::vector<int4>& tiles, const int* nn, const long long* of,
                const long long* uo, const long long* ho, int coords, std::string* err) {
  using T2 = typename Cx<T>::type;
  const DriveHost& H = D->host;
  std::vector<T> Ut(H.U.begin(), H.U.end()), ht(H.h.size()), qt(H.q.size());
  for (size_t i = 0; i < H.h.size(); ++i) ht[i] = (T)(H.h[i] / H.scale);
  for (size_t i = 0; i < H.q.size(); ++i) qt[i] = (T)(H.q[i] / H.scale);
  cudaError_t e = cudaSuccess;
  const int4* tl = nullptr;
  const T *Ud = nullptr, *hd = nullptr, *cd_ = nullptr;
  if (e == cudaSuccess) e = upload(D, tiles, &tl);
  if (e == cudaSuccess) e = upload(D, Ut, &Ud);
  if (e == cudaSuccess) e = upload(D, ht, &hd);
  if (e == cudaSuccess) e = upload(D, qt, &cd_);
  C.dev = DriveDev<T>{tl, nn, of, uo, ho, Ud, hd, cd_};
  void* p = nullptr;
  const size_t vb = sizeof(T2) * (size_t)D->dim;
  if (e == cudaSuccess && (e = dalloc(D, vb, &p)) == cudaSuccess) C.t1 = (T2*)p;
  if (e == cudaSuccess && (e = dalloc(D, vb, &p)) == cudaSuccess) C.t2 = (T2*)p;
  if (e == cudaSuccess && (e = dalloc(D, vb, &p)) == cudaSuccess) C.dv = (T2*)p;
  cudaStream_t st = D->plan->stream;
  const DevicePlan& dp = D->plan->dev;
  // the border vector v, a temporary of the setup
  T2* v = nullptr;
  if (e == cudaSuccess && (e = dalloc(D, vb, &p)) == cudaSuccess) v = (T2*)p;
  if (e == cudaSuccess) e = cudaMemsetAsync(v, 0, vb, st);
  if (e == cudaSuccess && dp.ndiag > 0) {
    k_drive_fill_border<T2><<<grid_for(dp.ndiag), 256, 0, st>>>(dp.sectors, dp.diag_sector, dp.diag_index, dp.ndiag,
                                                                v, coords);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = block_solve<T, T2, T2>(D, C, v, C.dv, st);
  if (e == cudaSuccess) e = trace_dot(dp, C.dv, sizeof(T) == sizeof(float) ? 1 : 0, coords, D->alpha, st);
  double2 tdv{0.0, 0.0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&tdv, D->alpha, sizeof(double2), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) {
    // the border vector's buffer is not needed after setup
    D->allocs.erase(std::find(D->allocs.begin(), D->allocs.end(), (void*)v));
    D->bytes -= std::max<size_t>(vb, 16);
    e = cudaFree(v);
  }
  if (e != cudaSuccess) {
    *err = std::string("drive preconditioner setup: ") + cudaGetErrorString(e);
    return PI_ERR_CUDA;
  }
  const std::complex<double> den(1.0 + tdv.x, tdv.y);
  if (!(std::abs(den) > 1e-12) || !std::isfinite(std::abs(den))) {
    *err = "the drive preconditioner's trace border is singular";
    return PI_ERR_NOT_CONVERGED;
  }
  const std::complex<double> inv = 1.0 / den;
  C.inv_den = make_double2(inv.real(), inv.imag());
  return PI_OK;
}

}  // namespace

int drive_create(pi_plan* plan, int coords, double scale, DriveState** out, std::string* err) {
  const auto t0 = std::chrono::steady_clock::now();
  *out = nullptr;
  DriveState* D = new DriveState;
  D->plan = plan;
  D->dim = plan->host.dim;
  int rc = build_drive_precond(plan->host, coords, scale, &D->host, err);
  if (rc) {
    delete D;
    return rc;
  }
  const DriveHost& H = D->host;
  const int S = (int)H.n.size();
  std::vector<int4> tiles;
  for (int s = 0; s < S; ++s) {
    const int nt = (H.n[s] + kDT - 1) / kDT;
    for (int a = 0; a < nt; ++a)
      for (int b = 0; b < nt; ++b) tiles.push_back(make_int4(s, a * kDT, b * kDT, 0));
  }
  D->ntiles = (int)tiles.size();
  cudaError_t e = cudaSuccess;
  const int* nn = nullptr;
  const long long *of = nullptr, *uo = nullptr, *ho = nullptr;
  void* p = nullptr;
  if (e == cudaSuccess) e = upload(D, H.n, &nn);
  if (e == cudaSuccess) e = upload(D, H.offset, &of);
  if (e == cudaSuccess) e = upload(D, H.u_off, &uo);
  if (e == cudaSuccess) e = upload(D, H.h_off, &ho);
  if (e == cudaSuccess && (e = dalloc(D, sizeof(double2) * 2, &p)) == cudaSuccess) D->alpha = (double2*)p;
  if (e != cudaSuccess) {
    drive_free(D);
    *err = std::string("drive preconditioner upload: ") + cudaGetErrorString(e);
    return PI_ERR_CUDA;
  }
  rc = setup_chain<float>(D, D->c32, tiles, nn, of, uo, ho, coords, err);
  if (!rc) rc = setup_chain<double>(D, D->c64, tiles, nn, of, uo, ho, coords, err);
  if (rc) {
    drive_free(D);
    return rc;
  }
  D->setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *out = D;
  return PI_OK;
}

cudaError_t drive_apply(DriveState* D, const void* r, int r_f32, void* z, int z_f32, cudaStream_t st) {
  if (r_f32 != z_f32) return cudaErrorInvalidValue;
  cudaError_t e = r_f32 ? block_solve<float, float2, float2>(D, D->c32, (const float2*)r, (float2*)z, st)
                        : block_solve<double, double2, double2>(D, D->c64, (const double2*)r, (double2*)z, st);
  if (e != cudaSuccess) return e;
  e = trace_dot(D->plan->dev, z, z_f32, D->host.coords, D->alpha, st);
  if (e != cudaSuccess) return e;
  if (z_f32)
    k_drive_border<float2><<<grid_for(D->dim), 256, 0, st>>>((float2*)z, D->c32.dv, D->alpha, D->c32.inv_den, D->dim);
  else
    k_drive_border<double2><<<grid_for(D->dim), 256, 0, st>>>((double2*)z, D->c64.dv, D->alpha, D->c64.inv_den,
                                                              D->dim);
  return cudaGetLastError();
}

void drive_free(DriveState* D) {
  if (!D) return;
  for (void* p : D->allocs) cudaFree(p);
  delete D;
}

size_t drive_bytes(const DriveState* D) { return D->bytes; }
const DriveHost& drive_host(const DriveState* D) { return D->host; }
double drive_setup_seconds(const DriveState* D) { return D->setup_seconds; }

}  // namespace picuda
