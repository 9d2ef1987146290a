// Krylov solver drivers behind the C ABI: restarted GMRES for the trace-bordered steady
// state (krylov.jl:732-891), adaptive Krylov expv (krylov_extensions.jl:1346-1573) and the
// expv dynamics loop with streamed observables (highlevel.jl:467-528, 665-733).
//
// The host drives the reference's control flow exactly (restart loop, Givens updates,
// accept/reject controller, small dense exponential); all O(dim) work runs on the device on
// the plan's stream: the fused apply, CGS2 (classical Gram-Schmidt with one full
// re-orthogonalisation, in place of the reference's MGS x2), norms and basis combinations.
// Per Arnoldi step the host reads back one Hessenberg column.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

#include "../../include/picuda.h"
#include "pi_batch.hpp"
#include "pi_dense.hpp"
#include "pi_handle.hpp"
#include "pi_precond.hpp"

namespace picuda {
namespace {

struct DeviceBuffers {
  cudaStream_t s = nullptr;
  std::vector<void*> ptrs;
  cudaError_t err = cudaSuccess;
  void* get(size_t bytes) {
    void* p = nullptr;
    if (err != cudaSuccess) return nullptr;
    err = cudaMallocAsync(&p, bytes ? bytes : 16, s);
    if (err != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return p;
  }
  ~DeviceBuffers() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
    cudaStreamSynchronize(s);
  }
};

// Sticky error wrapper for a sequence of stream-ordered launches.
struct Run {
  pi_plan* p;
  cudaStream_t s;
  long long n;
  cudaError_t err = cudaSuccess;
  int applications = 0;
  int coords = 0;  // PI_COORDS_* of every vector of the solve
  explicit Run(pi_plan* plan, int c = 0) : p(plan), s(plan->stream), n(plan->host.dim), coords(c) {}
  bool ok() const { return err == cudaSuccess; }
  void chk(cudaError_t e) {
    if (e != cudaSuccess && err == cudaSuccess) err = e;
  }
  // Reads back rs.rresult[0..cnt) and optionally device complex arrays.
  void fetch(double* out, const void* dev, size_t bytes) {
    if (!ok()) return;
    chk(cudaMemcpyAsync(p->host_pinned, dev, bytes, cudaMemcpyDeviceToHost, s));
    chk(cudaStreamSynchronize(s));
    if (ok()) std::memcpy(out, p->host_pinned, bytes);
  }
  double norm2(const double2* w) {
    chk(norm2_f64(w, n, p->rs, 0, s));
    double v = 0.0;
    fetch(&v, p->rs.rresult, sizeof(double));
    return v;
  }
  double norm(const double2* w) { return std::sqrt(norm2(w)); }
  // y = L x (unbordered)
  void apply(const double2* x, double2* y) {
    BorderArgs b{1.0, nullptr, coords};
    chk(launch_apply_f64(p->dev, (const double*)x, (double*)y, 1, n, b, s));
    ++applications;
  }
  // y = L x / scale + (t^H x) v  (krylov.jl:855-860)
  void apply_bordered(const double2* x, double2* y, double invscale, double2* alpha_dev) {
    chk(trace_dot(p->dev, x, 0, coords, alpha_dev, s));
    BorderArgs b{invscale, alpha_dev, coords};
    chk(launch_apply_f64(p->dev, (const double*)x, (double*)y, 1, n, b, s));
    ++applications;
  }
  void apply_bordered_f32(const float2* x, float2* y, double invscale, double2* alpha_dev) {
    chk(trace_dot(p->dev, x, 1, coords, alpha_dev, s));
    BorderArgs b{invscale, alpha_dev, coords};
    chk(launch_apply_f32(p->dev, (const float*)x, (float*)y, 1, n, b, s));
    ++applications;
  }
  // Left preconditioning of the bordered system B = L/s + v t^H.  Stage 0 applies `level`
  // (or the only preconditioner); stage 1 the drive part twice, z = D r, z += D (r - B z);
  // stage 2 drive, level and drive in turn, each on the current residual r - B z.  FP64 or
  // FP32 in and out; the extra bordered applies count as operator applications.
  double invscale = 1.0;
  double2* palpha = nullptr;        // border scalar of the extra applies
  void* pscr[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [f32][0..1]: n-vectors
  void bapply(const void* x, void* y, int f32) {
    if (f32)
      apply_bordered_f32((const float2*)x, (float2*)y, invscale, palpha);
    else
      apply_bordered((const double2*)x, (double2*)y, invscale, palpha);
  }
  // z += M (r - B z) for one preconditioner M
  void correct(const pi_precond* M, const void* r, void* z, int f32) {
    void* t = pscr[f32][0];
    void* u = pscr[f32][1];
    bapply(z, t, f32);
    chk(axpby(r, t, t, f32, 1.0, -1.0));  // t = r - B z
    chk(precond_apply(M, t, f32, u, f32, precond_scale(M), s));
    chk(axpby(z, u, z, f32, 1.0, 1.0));   // z += u
  }
  void precondition(const pi_precond* level, const pi_precond* drive, int stage, const void* r, void* z, int f32) {
    const pi_precond* first = stage == 0 ? (level ? level : drive) : drive;
    chk(precond_apply(first, r, f32, z, f32, precond_scale(first), s));
    if (stage == 0 && (level || precond_kind(first) == PI_PRECOND_LEVEL)) return;
    if (stage == 2) correct(level, r, z, f32);
    correct(drive, r, z, f32);
  }
  // out = a x + b y elementwise (n complex entries, FP64 or FP32)
  cudaError_t axpby(const void* x, const void* y, void* out, int f32, double a, double b);
  cd trace(const double2* x) {
    double2* out = p->rs.result;
    chk(trace_dot(p->dev, x, 0, coords, out, s));
    double h[2] = {0, 0};
    fetch(h, out, sizeof(double2));
    return cd(h[0], h[1]);
  }
};

// Dense normalized trace vector v = t / (t^H t) in x coordinates (coords 0) or its image
// in population coordinates (coords 1).
__global__ void k_fill_border(const DevSector* __restrict__ sectors, const int* __restrict__ diag_sector,
                              const long long* __restrict__ diag_index, int ndiag, double2* __restrict__ v,
                              int coords) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndiag; i += gridDim.x * blockDim.x) {
    const DevSector& sec = sectors[diag_sector[i]];
    v[diag_index[i]] = make_double2(coords ? sec.border_z : sec.border_x, 0.0);
  }
}

// r = b - w
__global__ void k_sub(const double2* __restrict__ b, const double2* __restrict__ w, double2* __restrict__ r,
                      long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    r[e] = make_double2(b[e].x - w[e].x, b[e].y - w[e].y);
}

inline int grid_n(long long n) {
  long long g = (n + 255) / 256;
  return (int)std::max(1LL, std::min(g, 4LL * 152));
}

template <typename T2>
__global__ void k_axpby(const T2* __restrict__ x, const T2* __restrict__ y, T2* __restrict__ out, double a, double b,
                        long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const T2 u = x[e], v = y[e];
    out[e].x = a * u.x + b * v.x;
    out[e].y = a * u.y + b * v.y;
  }
}

cudaError_t Run::axpby(const void* x, const void* y, void* out, int f32, double a, double b) {
  if (f32)
    k_axpby<float2><<<grid_n(n), 256, 0, s>>>((const float2*)x, (const float2*)y, (float2*)out, a, b, n);
  else
    k_axpby<double2><<<grid_n(n), 256, 0, s>>>((const double2*)x, (const double2*)y, (double2*)out, a, b, n);
  return cudaGetLastError();
}

// One CGS2 orthogonalisation of w against V[0..nv) (FP64): H column += h1 + h2 and
// *rem2 = |w|^2 after both passes.
template <typename VT>
void cgs2_fetch(Run& R, int nv, double2* h1d, std::vector<cd>& hcol, double* rem2) {
  // h1 and h2 are contiguous (h2 = h1 + kMaxDots); one pinned copy of both plus the
  // remainder norm, then a single synchronization.
  pi_plan* p = R.p;
  double* hp = p->host_pinned;
  R.chk(cudaMemcpyAsync(hp, h1d, sizeof(double2) * (kMaxDots + nv), cudaMemcpyDeviceToHost, R.s));
  R.chk(cudaMemcpyAsync(hp + 2 * (2 * kMaxDots), p->rs.rresult, sizeof(double) * 2, cudaMemcpyDeviceToHost, R.s));
  R.chk(cudaStreamSynchronize(R.s));
  if (!R.ok()) return;
  for (int i = 0; i < nv; ++i)
    hcol[i] += cd(hp[2 * i], hp[2 * i + 1]) + cd(hp[2 * (kMaxDots + i)], hp[2 * (kMaxDots + i) + 1]);
  *rem2 = hp[4 * kMaxDots];
}

// One CGS2 orthogonalisation of w against V[0..nv) (FP64): H column += h1 + h2 and
// *rem2 = |w|^2 after both passes.
void cgs2_f64(Run& R, const double2* V, int nv, double2* w, double2* h1d, double2* h2d, std::vector<cd>& hcol,
              double* rem2) {
  pi_plan* p = R.p;
  R.chk(mdot_f64(V, R.n, nv, w, R.n, p->rs, h1d, R.s));
  R.chk(maxpy_f64(V, R.n, nv, h1d, w, R.n, p->rs, -1, R.s));
  R.chk(mdot_f64(V, R.n, nv, w, R.n, p->rs, h2d, R.s));
  R.chk(maxpy_f64(V, R.n, nv, h2d, w, R.n, p->rs, 0, R.s));
  cgs2_fetch<double2>(R, nv, h1d, hcol, rem2);
}

// Classical Gram-Schmidt of an FP32 w against V[0..nv) with selective reorthogonalisation
// (Daniel-Gragg-Kaufman-Stewart): the second pass runs only when the first removed more than
// half of |w|^2, i.e. |w_1|^2 < |w_0|^2 / 2; otherwise w_1 is already orthogonal to the basis
// to working precision.  H column += h1 (+ h2) and *rem2 = |w|^2 at the end.  The mixed
// precision solves use it (as the batched engine does); the plain FP64 path keeps two passes.
void cgs_dgks_f32(Run& R, const float2* V, int nv, float2* w, double2* h1d, double2* h2d, std::vector<cd>& hcol,
                  double* rem2) {
  pi_plan* p = R.p;
  double* hp = p->host_pinned;
  R.chk(norm2_f32(w, R.n, p->rs, 1, R.s));  // |w_0|^2 -> rresult[1]
  R.chk(mdot_f32(V, R.n, nv, w, R.n, p->rs, h1d, R.s));
  R.chk(maxpy_f32(V, R.n, nv, h1d, w, R.n, p->rs, 0, R.s));  // |w_1|^2 -> rresult[0]
  R.chk(cudaMemcpyAsync(hp, h1d, sizeof(double2) * nv, cudaMemcpyDeviceToHost, R.s));
  R.chk(cudaMemcpyAsync(hp + 2 * kMaxDots, p->rs.rresult, sizeof(double) * 2, cudaMemcpyDeviceToHost, R.s));
  R.chk(cudaStreamSynchronize(R.s));
  if (!R.ok()) return;
  for (int i = 0; i < nv; ++i) hcol[i] += cd(hp[2 * i], hp[2 * i + 1]);
  const double w1 = hp[2 * kMaxDots], w0 = hp[2 * kMaxDots + 1];
  *rem2 = w1;
  if (!(w1 < 0.5 * w0)) return;
  R.chk(mdot_f32(V, R.n, nv, w, R.n, p->rs, h2d, R.s));
  R.chk(maxpy_f32(V, R.n, nv, h2d, w, R.n, p->rs, 0, R.s));
  R.chk(cudaMemcpyAsync(hp, h2d, sizeof(double2) * nv, cudaMemcpyDeviceToHost, R.s));
  R.chk(cudaMemcpyAsync(hp + 2 * kMaxDots, p->rs.rresult, sizeof(double), cudaMemcpyDeviceToHost, R.s));
  R.chk(cudaStreamSynchronize(R.s));
  if (!R.ok()) return;
  for (int i = 0; i < nv; ++i) hcol[i] += cd(hp[2 * i], hp[2 * i + 1]);
  *rem2 = hp[2 * kMaxDots];
}

void upper_triangular_solve(const std::vector<std::vector<cd>>& H, const std::vector<cd>& g, int k,
                            std::vector<cd>& y) {
  y.assign(k, cd(0, 0));
  for (int i = k - 1; i >= 0; --i) {
    cd s = g[i];
    for (int j = i + 1; j < k; ++j) s -= H[j][i] * y[j];  // H stored by column
    if (H[i][i] == cd(0, 0)) throw std::runtime_error("singular GMRES triangular factor");
    y[i] = s / H[i][i];
  }
}

// Raw-residual reduction per restart cycle below which the preconditioner ladder moves on:
// the level sweep gives way to the drive part after a cycle that gained less than 3x; the
// drive part (which converges steadily where the drive dominates) gives way to drive, level
// and drive only when it nearly stagnates (less than 1.25x), where the loss is as strong as
// the drive.
inline double ladder_factor(int stage) { return stage == 0 ? 3.0 : 1.25; }

struct GmresResult {
  bool converged = false;
  int iterations = 0, restarts = 0;
  double residual = 0.0;
};

// Operator-scale estimate (krylov.jl:156-169): max |L r| / |r| over 3 complex normal probes.
// The reference draws probes from Julia's MersenneTwister(0x51ca1e); this uses
// std::mt19937_64 with the same seed, so the scale agrees to tolerance, not bitwise.
double estimate_scale(Run& R, double2* probe, double2* image) {
  std::mt19937_64 rng(0x51ca1e);
  std::normal_distribution<double> nd(0.0, 1.0);
  std::vector<double2> h(R.n);
  double scale = 0.0;
  for (int k = 0; k < 3 && R.ok(); ++k) {
    for (long long e = 0; e < R.n; ++e) h[e] = make_double2(nd(rng) * M_SQRT1_2, nd(rng) * M_SQRT1_2);
    R.chk(cudaMemcpyAsync(probe, h.data(), sizeof(double2) * R.n, cudaMemcpyHostToDevice, R.s));
    const double nx = R.norm(probe);
    R.apply(probe, image);
    const double ny = R.norm(image);
    scale = std::max(scale, ny / nx);
  }
  return scale;
}

// Restarted GMRES(m) on the bordered system (krylov.jl:732-787), FP64.  With a
// preconditioner P it runs the reference's left-preconditioned form: the Krylov space of
// P A, the preconditioned residual |P r| tested against atol + rtol |P b| and the raw residual
// |r| against atol + rtol |b|, both after every restart (krylov.jl:737-786).
GmresResult gmres_f64(Run& R, double2* x, const double2* b, int m, double atol, double rtol, int maxiter,
                      double invscale, DeviceBuffers& buf, const pi_precond* Plev, const pi_precond* Pdrv,
                      int* stage_out) {
  GmresResult res;
  const long long n = R.n;
  const pi_precond* P = Plev ? Plev : Pdrv;
  const bool ladder = Plev && Pdrv;
  int stage = 0;
  double2* V = (double2*)buf.get(sizeof(double2) * n * (m + 1));
  double2* w = (double2*)buf.get(sizeof(double2) * n);
  double2* r = (double2*)buf.get(sizeof(double2) * n);
  double2* pz = P ? (double2*)buf.get(sizeof(double2) * n) : nullptr;
  double2* hd = (double2*)buf.get(sizeof(double2) * 2 * kMaxDots);
  double2* alpha = (double2*)buf.get(sizeof(double2) * 4);
  double2* yd = (double2*)buf.get(sizeof(double2) * kMaxDots);
  if (Pdrv) {
    R.pscr[0][0] = buf.get(sizeof(double2) * n);
    R.pscr[0][1] = buf.get(sizeof(double2) * n);
  }
  if (!V || !w || !r || !hd || !alpha || !yd || (P && !pz) || (Pdrv && (!R.pscr[0][0] || !R.pscr[0][1]))) {
    R.chk(buf.err);
    return res;
  }
  R.invscale = invscale;
  R.palpha = alpha + 2;
  auto prec = [&](const void* in, void* out) { R.precondition(Plev, Pdrv, stage, in, out, 0); };
  double2* h1d = hd;
  double2* h2d = hd + kMaxDots;
  const double raw_bnorm = R.norm(b);
  const double rawtol = atol + rtol * raw_bnorm;
  double bnorm = raw_bnorm;
  if (P) {
    prec(b, pz);
    bnorm = R.norm(pz);
  }
  double tol = atol + rtol * bnorm;
  // residual of the current x: r = b - A x, its raw and (preconditioned) norms
  auto residual = [&](double* rawbeta) {
    R.apply_bordered(x, w, invscale, alpha);
    R.chk((k_sub<<<grid_n(n), 256, 0, R.s>>>(b, w, r, n), cudaGetLastError()));
    *rawbeta = R.norm(r);
    if (!P) return *rawbeta;
    prec(r, pz);
    return R.norm(pz);
  };
  double rawbeta = 0.0;
  double beta = residual(&rawbeta);
  res.residual = beta;
  *stage_out = stage;
  if (beta <= tol && rawbeta <= rawtol) {
    res.converged = true;
    return res;
  }
  double prev_raw = rawbeta;
  std::vector<std::vector<cd>> H(m, std::vector<cd>(m + 1));  // H[j] = column j
  std::vector<cd> g(m + 1), sn(m), y;
  std::vector<double> cs(m);
  while (res.iterations < maxiter && R.ok()) {
    for (auto& col : H) std::fill(col.begin(), col.end(), cd(0, 0));
    std::fill(g.begin(), g.end(), cd(0, 0));
    R.chk(scale_f64(P ? pz : r, V, n, make_double2(1.0 / beta, 0.0), 0, R.s));
    g[0] = beta;
    // With a preconditioner the recomputed |P r| after a restart differs from the cycle's
    // estimate |g| by the preconditioner's rounding (FP32 parts, combined stages); a cycle that
    // stops exactly at tol can then restart just above it, cycle after cycle.  Preconditioned
    // cycles target tol / 2, as the mixed-precision inner solves do.
    const double ctol = P ? 0.5 * tol : tol;
    int kdone = 0;
    const int steps = std::min(m, maxiter - res.iterations);
    for (int j = 0; j < steps && R.ok(); ++j) {
      R.apply_bordered(V + (long long)j * n, w, invscale, alpha);
      double2* q = w;
      if (P) {
        prec(w, pz);
        q = pz;
      }
      double rem2 = 0.0;
      cgs2_f64(R, V, j + 1, q, h1d, h2d, H[j], &rem2);
      H[j][j + 1] = std::sqrt(rem2);
      if (H[j][j + 1] != cd(0, 0))
        R.chk(scale_f64(q, V + (long long)(j + 1) * n, n, make_double2(1.0 / H[j][j + 1].real(), 0.0), 0, R.s));
      for (int i = 0; i < j; ++i) {
        const cd h1 = H[j][i], h2 = H[j][i + 1];
        H[j][i] = cs[i] * h1 + sn[i] * h2;
        H[j][i + 1] = -std::conj(sn[i]) * h1 + cs[i] * h2;
      }
      double c;
      cd sg;
      complex_givens(H[j][j], H[j][j + 1], &c, &sg);
      cs[j] = c;
      sn[j] = sg;
      const cd h1 = H[j][j], h2 = H[j][j + 1];
      H[j][j] = c * h1 + sg * h2;
      H[j][j + 1] = 0.0;
      const cd g1 = g[j], g2 = g[j + 1];
      g[j] = c * g1 + sg * g2;
      g[j + 1] = -std::conj(sg) * g1 + c * g2;
      ++res.iterations;
      kdone = j + 1;
      if (std::abs(g[j + 1]) <= ctol) break;
    }
    if (!R.ok()) break;
    upper_triangular_solve(H, g, kdone, y);
    R.chk(cudaMemcpyAsync(yd, y.data(), sizeof(double2) * kdone, cudaMemcpyHostToDevice, R.s));
    R.chk(combine_f64(V, n, kdone, yd, x, n, 1, R.s));
    ++res.restarts;
    beta = residual(&rawbeta);
    res.residual = beta;
    if (beta <= tol && rawbeta <= rawtol) {
      res.converged = true;
      return res;
    }
    if (ladder && stage < 2 && rawbeta > prev_raw / ladder_factor(stage)) {
      // the cycle made too little progress: the next preconditioner stage, with the
      // preconditioned tests rescaled to it
      ++stage;
      *stage_out = stage;
      prec(b, pz);
      bnorm = R.norm(pz);
      tol = atol + rtol * bnorm;
      prec(r, pz);
      beta = R.norm(pz);
      res.residual = beta;
    }
    prev_raw = rawbeta;
  }
  return res;
}

// Mixed-precision GMRES with FP64 iterative refinement: every restart cycle computes the
// true bordered residual b - A x in FP64 and solves the correction equation with FP32
// applies, an FP32 Krylov basis and FP64-accumulated CGS2; the update x += d is FP64.  With
// a preconditioner the correction equation is solved left-preconditioned (FP32 sweeps) and
// the outer tests are the reference's pair: |P r| <= atol + rtol |P b| and
// |r| <= atol + rtol |b|, with P r and r in FP64.
GmresResult gmres_mixed(Run& R, double2* x, const double2* b, int m, double atol, double rtol, int maxiter,
                        int max_refinements, double invscale, DeviceBuffers& buf, int* refinements,
                        const pi_precond* Plev, const pi_precond* Pdrv, int* stage_out) {
  GmresResult res;
  const long long n = R.n;
  const pi_precond* P = Plev ? Plev : Pdrv;
  const bool ladder = Plev && Pdrv;
  int stage = 0;
  float2* V = (float2*)buf.get(sizeof(float2) * n * (m + 1));
  float2* w = (float2*)buf.get(sizeof(float2) * n);
  float2* pw = P ? (float2*)buf.get(sizeof(float2) * n) : nullptr;
  double2* w64 = (double2*)buf.get(sizeof(double2) * n);
  double2* r = (double2*)buf.get(sizeof(double2) * n);
  double2* pz = P ? (double2*)buf.get(sizeof(double2) * n) : nullptr;
  double2* hd = (double2*)buf.get(sizeof(double2) * 2 * kMaxDots);
  double2* alpha = (double2*)buf.get(sizeof(double2) * 4);
  double2* yd = (double2*)buf.get(sizeof(double2) * kMaxDots);
  if (Pdrv) {
    for (int k = 0; k < 2; ++k) {
      R.pscr[0][k] = buf.get(sizeof(double2) * n);
      R.pscr[1][k] = buf.get(sizeof(float2) * n);
    }
  }
  if (!V || !w || !w64 || !r || !hd || !alpha || !yd || (P && (!pw || !pz)) ||
      (Pdrv && (!R.pscr[0][0] || !R.pscr[0][1] || !R.pscr[1][0] || !R.pscr[1][1]))) {
    R.chk(buf.err);
    return res;
  }
  R.invscale = invscale;
  R.palpha = alpha + 2;
  auto prec = [&](const void* in, void* out, int f32) { R.precondition(Plev, Pdrv, stage, in, out, f32); };
  double2* h1d = hd;
  double2* h2d = hd + kMaxDots;
  const double raw_bnorm = R.norm(b);
  const double rawtol = atol + rtol * raw_bnorm;
  double bnorm = raw_bnorm;
  if (P) {
    prec(b, pz, 0);
    bnorm = R.norm(pz);
  }
  double tol = atol + rtol * bnorm;
  double prev_raw = -1.0;
  *stage_out = stage;
  // Inner solves stop at this relative reduction: FP32 applies cannot resolve the
  // correction much below it, and the FP64 outer residual restores the rest.
  const double inner_rtol = 1e-5;
  std::vector<std::vector<cd>> H(m, std::vector<cd>(m + 1));
  std::vector<cd> g(m + 1), sn(m), y;
  std::vector<double> cs(m);
  *refinements = 0;
  while (R.ok()) {
    R.apply_bordered(x, w64, invscale, alpha);
    R.chk((k_sub<<<grid_n(n), 256, 0, R.s>>>(b, w64, r, n), cudaGetLastError()));
    const double rawbeta = R.norm(r);
    if (ladder && stage < 2 && prev_raw > 0 && rawbeta > prev_raw / ladder_factor(stage)) {
      // the last refinement cycle made too little progress: the next preconditioner stage,
      // with the preconditioned tests rescaled to it
      ++stage;
      *stage_out = stage;
      prec(b, pz, 0);
      bnorm = R.norm(pz);
      tol = atol + rtol * bnorm;
    }
    prev_raw = rawbeta;
    double beta = rawbeta;
    if (P) {
      prec(r, pz, 0);
      beta = R.norm(pz);
    }
    res.residual = beta;
    if (beta <= tol && rawbeta <= rawtol) {
      res.converged = true;
      return res;
    }
    if (res.iterations >= maxiter || *refinements >= max_refinements) break;
    ++*refinements;
    for (auto& col : H) std::fill(col.begin(), col.end(), cd(0, 0));
    std::fill(g.begin(), g.end(), cd(0, 0));
    R.chk(f64_to_f32(P ? pz : r, V, n, 1.0 / beta, R.s));
    g[0] = beta;
    const double itol = std::max(tol * 0.5, inner_rtol * beta);
    int kdone = 0;
    const int steps = std::min(m, maxiter - res.iterations);
    for (int j = 0; j < steps && R.ok(); ++j) {
      R.apply_bordered_f32(V + (long long)j * n, w, invscale, alpha);
      float2* q = w;
      if (P) {
        prec(w, pw, 1);
        q = pw;
      }
      double rem2 = 0.0;
      cgs_dgks_f32(R, V, j + 1, q, h1d, h2d, H[j], &rem2);
      H[j][j + 1] = std::sqrt(rem2);
      if (H[j][j + 1] != cd(0, 0))
        R.chk(scale_f32(q, V + (long long)(j + 1) * n, n, make_double2(1.0 / H[j][j + 1].real(), 0.0), R.s));
      for (int i = 0; i < j; ++i) {
        const cd h1 = H[j][i], h2 = H[j][i + 1];
        H[j][i] = cs[i] * h1 + sn[i] * h2;
        H[j][i + 1] = -std::conj(sn[i]) * h1 + cs[i] * h2;
      }
      double c;
      cd sg;
      complex_givens(H[j][j], H[j][j + 1], &c, &sg);
      cs[j] = c;
      sn[j] = sg;
      const cd h1 = H[j][j], h2 = H[j][j + 1];
      H[j][j] = c * h1 + sg * h2;
      H[j][j + 1] = 0.0;
      const cd g1 = g[j], g2 = g[j + 1];
      g[j] = c * g1 + sg * g2;
      g[j + 1] = -std::conj(sg) * g1 + c * g2;
      ++res.iterations;
      kdone = j + 1;
      if (std::abs(g[j + 1]) <= itol) break;
    }
    if (!R.ok() || kdone == 0) break;
    upper_triangular_solve(H, g, kdone, y);
    R.chk(cudaMemcpyAsync(yd, y.data(), sizeof(double2) * kdone, cudaMemcpyHostToDevice, R.s));
    R.chk(combine_f32_to_f64(V, n, kdone, yd, x, n, 1, R.s));
    ++res.restarts;
  }
  return res;
}

}  // namespace

// Operator scale of the plan in the given coordinates (3 complex normal probes,
// krylov.jl:156-169), for a preconditioner built before the solve.
int estimate_operator_scale(pi_plan* plan, int coords, double* out) {
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  Run R(plan, coords);
  DeviceBuffers buf;
  buf.s = R.s;
  double2* t1 = (double2*)buf.get(sizeof(double2) * R.n);
  double2* t2 = (double2*)buf.get(sizeof(double2) * R.n);
  if (!t1 || !t2) return cuda_fail(buf.err, "operator-scale workspace");
  const double s = estimate_scale(R, t1, t2);
  if (!R.ok()) return cuda_fail(R.err, "operator-scale estimate");
  if (!(std::isfinite(s) && s > 0))
    return fail(PI_ERR_INVALID_ARGUMENT, "operator_scale must be finite and positive");
  *out = s;
  return PI_OK;
}

}  // namespace picuda

using namespace picuda;

extern "C" {

void pi_gmres_default_opts(pi_gmres_opts_t* o) {
  if (!o) return;
  o->krylovdim = 30;
  o->maxiter = 500;
  o->atol = 1e-10;
  o->rtol = 1e-8;
  o->operator_scale = 0.0;
  o->precision = PI_FP64;
  o->use_initial = 0;
  o->max_refinements = 200;
  o->coords = PI_COORDS_REFERENCE;
  o->preconditioner = nullptr;
  o->drive_preconditioner = nullptr;
}

int pi_steady_state(pi_plan* plan, double* x_dev, const pi_gmres_opts_t* opts, pi_gmres_info_t* info) {
  if (!plan || !x_dev || !opts) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (opts->krylovdim < 1 || opts->krylovdim > kMaxDots - 1)
    return fail(PI_ERR_INVALID_ARGUMENT, "krylovdim must lie in 1:127");
  if (opts->maxiter < 1) return fail(PI_ERR_INVALID_ARGUMENT, "maxiter must be positive");
  if (!(opts->atol >= 0) || !(opts->rtol >= 0)) return fail(PI_ERR_INVALID_ARGUMENT, "tolerances must be nonnegative");
  if (opts->precision != PI_FP64 && opts->precision != PI_FP32)
    return fail(PI_ERR_INVALID_ARGUMENT, "precision must be PI_FP64 or PI_FP32");
  if (opts->coords != PI_COORDS_REFERENCE && opts->coords != PI_COORDS_POPULATION)
    return fail(PI_ERR_INVALID_ARGUMENT, "coords must be PI_COORDS_REFERENCE or PI_COORDS_POPULATION");
  const pi_precond* P = opts->preconditioner;
  if (P) {
    if (precond_plan(P) != plan)
      return fail(PI_ERR_INVALID_ARGUMENT, "the preconditioner was built for another compiled model");
    if (precond_coords(P) != opts->coords)
      return fail(PI_ERR_INVALID_ARGUMENT, "the preconditioner was built for other coordinates than the solve's");
    const double ps = precond_scale(P);
    if (opts->operator_scale > 0 && std::abs(opts->operator_scale - ps) > std::sqrt(2.2e-16) * ps)
      return fail(PI_ERR_INVALID_ARGUMENT, "operator_scale is inconsistent with the prepared preconditioner");
  }
  const pi_precond* Pd = opts->drive_preconditioner;
  if (Pd) {
    if (!P || precond_kind(P) != PI_PRECOND_LEVEL || precond_kind(Pd) != PI_PRECOND_DRIVE)
      return fail(PI_ERR_INVALID_ARGUMENT,
                  "drive_preconditioner needs a PI_PRECOND_DRIVE preconditioner beside a PI_PRECOND_LEVEL one");
    if (precond_plan(Pd) != plan || precond_coords(Pd) != opts->coords)
      return fail(PI_ERR_INVALID_ARGUMENT, "the drive preconditioner was built for another model or coordinates");
    const double ps = precond_scale(P);
    if (std::abs(precond_scale(Pd) - ps) > std::sqrt(2.2e-16) * ps)
      return fail(PI_ERR_INVALID_ARGUMENT, "the two preconditioners were built for different operator scales");
  }
  const pi_precond* Plev = P && precond_kind(P) == PI_PRECOND_LEVEL ? P : nullptr;
  const pi_precond* Pdrv = P && precond_kind(P) == PI_PRECOND_DRIVE ? P : Pd;
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  if (opts->krylovdim <= kBatchMaxKrylov && !P && opts->coords == PI_COORDS_REFERENCE) {
    // one job of the plan's batched engine: each GMRES cycle on the device, Givens included
    SteadyJob job(plan, x_dev, *opts, 0x51ca1eULL, true);
    const int rc = run_single_job(plan, &job, opts->krylovdim, opts->precision == PI_FP32, "GMRES");
    if (rc) return rc;
    if (info) *info = job.info();
    return job.rc == PI_OK ? PI_OK : fail(job.rc, job.msg);
  }
  const int coords = opts->coords;
  Run R(plan, coords);
  const long long n = R.n;
  const int m = (int)std::min<long long>(opts->krylovdim, n);
  pi_gmres_info_t loc;
  std::memset(&loc, 0, sizeof(loc));
  int rc = PI_OK;
  {
    DeviceBuffers buf;
    buf.s = R.s;
    double2* v = (double2*)buf.get(sizeof(double2) * n);
    double2* t1 = (double2*)buf.get(sizeof(double2) * n);
    double2* t2 = (double2*)buf.get(sizeof(double2) * n);
    // the solve's vector: x itself, or z = sqrt(f) x in population coordinates
    double2* x = coords == PI_COORDS_POPULATION ? (double2*)buf.get(sizeof(double2) * n) : (double2*)x_dev;
    if (!v || !t1 || !t2 || !x) return cuda_fail(buf.err, "solver workspace");
    R.chk(cudaMemsetAsync(v, 0, sizeof(double2) * n, R.s));
    R.chk((k_fill_border<<<grid_n(plan->dev.ndiag), 256, 0, R.s>>>(plan->dev.sectors, plan->dev.diag_sector,
                                                                    plan->dev.diag_index, plan->dev.ndiag, v,
                                                                    coords),
           cudaGetLastError()));
    if (!opts->use_initial)
      R.chk(cudaMemcpyAsync(x, v, sizeof(double2) * n, cudaMemcpyDeviceToDevice, R.s));
    else if (coords == PI_COORDS_POPULATION)
      R.chk(x_to_z_f64(plan->dev, (const double2*)x_dev, x, 1.0, R.s));
    double s = P ? precond_scale(P) : (opts->operator_scale > 0 ? opts->operator_scale : estimate_scale(R, t1, t2));
    if (!R.ok()) return cuda_fail(R.err, "operator-scale estimate");
    if (!(std::isfinite(s) && s > 0))
      return fail(PI_ERR_INVALID_ARGUMENT,
                  "operator_scale must be finite and positive; a numerically zero Liouvillian does not define a "
                  "unique trace-fixed Krylov solve");
    GmresResult gr;
    int refinements = 0;
    int stage = 0;
    try {
      if (opts->precision == PI_FP64)
        gr = gmres_f64(R, x, v, m, opts->atol, opts->rtol, opts->maxiter, 1.0 / s, buf, Plev, Pdrv, &stage);
      else
        gr = gmres_mixed(R, x, v, m, opts->atol, opts->rtol, opts->maxiter, std::max(1, opts->max_refinements),
                         1.0 / s, buf, &refinements, Plev, Pdrv, &stage);
    } catch (const std::exception& ex) {
      return fail(PI_ERR_NOT_CONVERGED, ex.what());
    }
    if (!R.ok()) return cuda_fail(R.err, "GMRES");
    // Final checks in the reference's terms (krylov.jl:868-873), in the solve's coordinates.
    R.apply(x, t1);
    const double residual = R.norm(t1);
    const double normalized = residual / s;
    const cd tr = R.trace(x);
    const double terr = std::abs(tr - cd(1, 0));
    const double xn = R.norm(x);
    const double tol = opts->atol + opts->rtol * std::max(xn, 1.0);
    if (coords == PI_COORDS_POPULATION) R.chk(z_to_x_f64(plan->dev, x, (double2*)x_dev, 1.0, 0, R.s));
    R.chk(cudaStreamSynchronize(R.s));
    if (!R.ok()) return cuda_fail(R.err, "GMRES final check");
    loc.converged = gr.converged && normalized <= tol && terr <= opts->atol + opts->rtol;
    loc.iterations = gr.iterations;
    loc.restarts = gr.restarts;
    loc.refinements = refinements;
    loc.operator_applications = R.applications;
    loc.residual = residual;
    loc.normalized_residual = normalized;
    loc.trace_error = terr;
    loc.operator_scale = s;
    loc.linear_residual = gr.residual;
    loc.preconditioner_stage = stage;
    if (!loc.converged) {
      char msg[256];
      std::snprintf(msg, sizeof(msg),
                    "matrix-free Krylov steady-state solve did not converge in %d iterations; "
                    "normalized_residual=%.3e, trace_error=%.3e",
                    gr.iterations, normalized, terr);
      rc = fail(PI_ERR_NOT_CONVERGED, msg);
    }
  }
  if (info) *info = loc;
  return rc;
}

}  // extern "C"
