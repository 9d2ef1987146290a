// C ABI of libpicuda.so: plan upload, capability, basis maps, apply and dot entry points.
// The Krylov solver entry points live in pi_solvers.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/picuda.h"
#include "pi_batch.hpp"
#include "pi_handle.hpp"
#include "pi_precond.hpp"
#include "pi_drive.hpp"

namespace picuda {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? PI_ERR_OUT_OF_MEMORY : PI_ERR_CUDA;
}

void* plan_alloc(pi_plan* plan, size_t bytes) {
  void* p = nullptr;
  if (bytes == 0) bytes = 16;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
  plan->allocations.push_back(p);
  plan->device_bytes += bytes;
  return p;
}

namespace {

template <typename T>
int upload(pi_plan* plan, const std::vector<T>& host, const T** out) {
  void* d = plan_alloc(plan, host.size() * sizeof(T));
  if (!d) return fail(PI_ERR_OUT_OF_MEMORY, "device allocation of plan tables failed");
  if (!host.empty()) {
    cudaError_t e = cudaMemcpy(d, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "plan upload");
  }
  *out = (const T*)d;
  return PI_OK;
}

void free_plan(pi_plan* plan) {
  if (!plan) return;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(plan->device);
  if (plan->stream) cudaStreamSynchronize(plan->stream);
  release_plan_engine(plan);
  for (void* p : plan->allocations) cudaFree(p);
  if (plan->stage_x) cudaFree(plan->stage_x);
  if (plan->stage_y) cudaFree(plan->stage_y);
  for (auto& ps : plan->pipe)
    if (ps) cudaStreamDestroy(ps);
  if (plan->host_pinned) cudaFreeHost(plan->host_pinned);
  if (plan->stream) cudaStreamDestroy(plan->stream);
  cudaSetDevice(cur);
  delete plan;
}

bool overlap(const void* a, size_t abytes, const void* b, size_t bbytes) {
  const char* pa = (const char*)a;
  const char* pb = (const char*)b;
  return pa < pb + bbytes && pb < pa + abytes;
}

}  // namespace

// Flattens the host plan into device tables (explicit_once transfer policy,
// accelerators.jl:9-11: the plan is uploaded once; applies move no host data).
int upload_plan(pi_plan* plan) {
  const QubitPlan& hp = plan->host;
  const int S = (int)hp.sectors.size();
  std::vector<DevSector> sectors(S);
  std::vector<DevTerm> terms;
  std::vector<double2> coef64, coef64z;
  std::vector<float2> coef32x, coef32z;
  std::vector<DevTile> tiles;
  std::vector<int> diag_sector;
  std::vector<long long> diag_index;
  auto group_of = [](const StencilTerm& t) -> int {
    switch (t.kind) {
      case ST_ADD: return G_ADD;
      case ST_LEFT: return t.cls == CC_IMAG ? G_LEFT_IM : t.cls == CC_REAL ? G_LEFT_RE : G_LEFT_CX;
      case ST_RIGHT: return t.cls == CC_IMAG ? G_RIGHT_IM : t.cls == CC_REAL ? G_RIGHT_RE : G_RIGHT_CX;
      default: return t.cls == CC_REAL ? G_SAND_RE : G_SAND_CX;
    }
  };
  // grouped terms of every sector, kept for the fixed-structure table below
  std::vector<std::array<std::vector<DevTerm>, G_COUNT>> by_group(S);
  for (int s = 0; s < S; ++s) {
    const Sector& sec = hp.sectors[s];
    DevSector& ds = sectors[s];
    std::memset(&ds, 0, sizeof(ds));
    ds.offset = sec.offset;
    ds.n = sec.n;
    ds.term_begin = (int)terms.size();
    ds.border_x = sec.sqrt_f / hp.trace_norm2;
    ds.border_z = sec.f / hp.trace_norm2;
    ds.sqrt_f = sec.sqrt_f;
    if ((int)sec.terms.size() > kMaxSectorTerms)
      return fail(PI_ERR_UNSUPPORTED, "a sector has more stencil terms than the apply kernel stages");
    ds.src[0] = ds.src[1] = ds.src[2] = -1;
    for (const StencilTerm& t : sec.terms) {
      if (t.e < -1 || t.e > 1 || t.p < -kHalo || t.p > kHalo || t.q < -kHalo || t.q > kHalo)
        return fail(PI_ERR_UNSUPPORTED, "stencil term outside the staged band");
      if (ds.src[t.e + 1] >= 0 && ds.src[t.e + 1] != t.src)
        return fail(PI_ERR_UNSUPPORTED, "two source sectors share one index shift");
      ds.src[t.e + 1] = t.src;
    }
    for (int g = 0; g < G_COUNT; ++g) {
      for (const StencilTerm& t : sec.terms) {
        if (group_of(t) != g) continue;
        DevTerm dt;
        const Sector& src = hp.sectors[t.src];
        dt.woff = (t.e + 1) * kWinElems + t.p + t.q * kWinRows;
        dt.pad = 0;
        const double ratio = sec.sqrt_f / src.sqrt_f;  // population-coordinate rescaling
        dt.alpha_off = 0;
        dt.beta_off = 0;
        // every coefficient array starts on a 4-element boundary and is padded to a
        // multiple of 4, so the kernel reads beta[b0 .. b0+3] with aligned vector loads
        auto pad4 = [&]() {
          while (coef64.size() % 4) {
            coef64.push_back(make_double2(0, 0));
            coef64z.push_back(make_double2(0, 0));
            coef32x.push_back(make_float2(0, 0));
            coef32z.push_back(make_float2(0, 0));
          }
        };
        pad4();
        if (!t.alpha.empty()) {
          dt.alpha_off = (int)coef64.size();
          for (const auto& z : t.alpha) {
            coef64.push_back(make_double2(z.real(), z.imag()));
            coef32x.push_back(make_float2((float)z.real(), (float)z.imag()));
            coef32z.push_back(make_float2((float)(z.real() * ratio), (float)(z.imag() * ratio)));
            coef64z.push_back(make_double2(z.real() * ratio, z.imag() * ratio));
          }
          pad4();
        }
        if (!t.beta.empty()) {
          dt.beta_off = (int)coef64.size();
          for (const auto& z : t.beta) {
            // ratio is applied once, on alpha (or on beta for a RIGHT term, which has no alpha)
            const double r = t.alpha.empty() ? ratio : 1.0;
            coef64.push_back(make_double2(z.real(), z.imag()));
            coef32x.push_back(make_float2((float)z.real(), (float)z.imag()));
            coef32z.push_back(make_float2((float)(z.real() * r), (float)(z.imag() * r)));
            coef64z.push_back(make_double2(z.real() * r, z.imag() * r));
          }
          pad4();
        }
        terms.push_back(dt);
        by_group[s][g].push_back(dt);
      }
      ds.group_end[g] = (int)terms.size();
    }
    for (int a0 = 0; a0 < sec.n; a0 += kTileRows)
      for (int b0 = 0; b0 < sec.n; b0 += kTileCols) tiles.push_back(DevTile{s, a0, b0, 0});
    for (int a = 0; a < sec.n; ++a) {
      diag_sector.push_back(s);
      diag_index.push_back(sec.offset + a + (long long)a * sec.n);
    }
  }
  // Fixed-structure table for the batched kernel: one ADD, two imaginary LEFT, two
  // imaginary RIGHT and fast_sr real sandwich terms per sector, padded with zero terms.
  std::vector<DevTerm> fterms;
  int fast_sr = 0;
  int fast_zero_off = -1;  // zero coefficient pool of the fixed-structure tables
  {
    bool ok = true;
    int max_sr = 0;
    for (int s = 0; s < S && ok; ++s) {
      const auto& g = by_group[s];
      ok = g[G_LEFT_RE].empty() && g[G_LEFT_CX].empty() && g[G_RIGHT_RE].empty() && g[G_RIGHT_CX].empty() &&
           g[G_SAND_CX].empty() && g[G_ADD].size() <= 1 && g[G_LEFT_IM].size() <= 2 && g[G_RIGHT_IM].size() <= 2;
      max_sr = std::max(max_sr, (int)g[G_SAND_RE].size());
    }
    if (ok && max_sr <= 13) {
      fast_sr = max_sr <= 5 ? 5 : (max_sr <= 9 ? 9 : 13);
      while (coef64.size() % 4) {
        coef64.push_back(make_double2(0, 0));
        coef64z.push_back(make_double2(0, 0));
        coef32x.push_back(make_float2(0, 0));
        coef32z.push_back(make_float2(0, 0));
      }
      const int zero_off = (int)coef64.size();
      fast_zero_off = zero_off;
      const int zlen = ((hp.max_n + 3) / 4) * 4 + 4;
      for (int i = 0; i < zlen; ++i) {
        coef64.push_back(make_double2(0, 0));
        coef64z.push_back(make_double2(0, 0));
        coef32x.push_back(make_float2(0, 0));
        coef32z.push_back(make_float2(0, 0));
      }
      const DevTerm zero{kWinElems, zero_off, zero_off, 0};  // centre of the own-sector window
      auto put = [&](const std::vector<DevTerm>& v, int count) {
        for (int i = 0; i < count; ++i) fterms.push_back(i < (int)v.size() ? v[i] : zero);
      };
      for (int s = 0; s < S; ++s) {
        const auto& g = by_group[s];
        put(g[G_ADD], 1);
        put(g[G_LEFT_IM], 2);
        put(g[G_RIGHT_IM], 2);
        put(g[G_SAND_RE], fast_sr);
      }
    }
  }
  // Canonical-position table for the register-reuse batched kernel (pi_apply.cu,
  // k_apply_canon): per sector kCanonEntries int4 (alpha_off, beta_off, 0, 0):
  //   [0] ADD; [1], [2] imaginary LEFT at row shift p = -1, +1; [3], [4] imaginary RIGHT at
  //   column shift q = -1, +1; then, for each source slot (0..2) and diagonal shift
  //   p = q = -1, 0, +1, kCanonPerPos real sandwich terms (zero-padded).
  // Built only when every term of every sector sits at one of these positions.
  std::vector<int4> canon;
  int canon_plus = 0;
  if (fast_sr > 0) {
    bool ok = true;
    std::vector<int4> table;
    const int zoff = fast_zero_off;
    for (int s = 0; s < S && ok; ++s) {
      std::vector<int4> e(kCanonEntries, make_int4(zoff, zoff, 0, 0));
      int nsand[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      bool have_add = false, have_l[2] = {false, false}, have_r[2] = {false, false};
      for (int g = 0; g < G_COUNT && ok; ++g) {
        for (const DevTerm& dt : by_group[s][g]) {
          // woff = slot * kWinElems + p + q * kWinRows, |p|, |q| <= kHalo
          const int span = kHalo + kHalo * kWinRows;
          const int slot = (dt.woff + span) / kWinElems;
          const int rem = dt.woff - slot * kWinElems;
          // rem = p + q * kWinRows with p, q in [-2, 2]
          int q = (rem + 2 + 2 * kWinRows) / kWinRows - 2;
          int p = rem - q * kWinRows;
          if (g == G_ADD) {
            ok = slot == 1 && p == 0 && q == 0 && !have_add;
            e[0] = make_int4(dt.alpha_off, dt.beta_off, 0, 0);
            have_add = true;
          } else if (g == G_LEFT_IM) {
            const int i = p < 0 ? 0 : 1;
            ok = slot == 1 && q == 0 && (p == -1 || p == 1) && !have_l[i];
            e[1 + i] = make_int4(dt.alpha_off, dt.beta_off, 0, 0);
            have_l[i] = true;
          } else if (g == G_RIGHT_IM) {
            const int i = q < 0 ? 0 : 1;
            ok = slot == 1 && p == 0 && (q == -1 || q == 1) && !have_r[i];
            e[3 + i] = make_int4(dt.alpha_off, dt.beta_off, 0, 0);
            have_r[i] = true;
          } else if (g == G_SAND_RE) {
            ok = p == q && p >= -1 && p <= 1;
            if (!ok) break;
            const int pos = slot * 3 + (p + 1);
            if (nsand[pos] >= kCanonPerPos) {
              ok = false;
              break;
            }
            e[5 + pos * kCanonPerPos + nsand[pos]] = make_int4(dt.alpha_off, dt.beta_off, 0, 0);
            ++nsand[pos];
            if (p == 1) canon_plus = 1;
          } else {
            ok = false;
          }
          if (!ok) break;
        }
      }
      table.insert(table.end(), e.begin(), e.end());
    }
    if (ok && zoff >= 0) canon.swap(table);
  }
  // Largest sectors first: their tiles are the longest-running.
  std::stable_sort(tiles.begin(), tiles.end(), [&](const DevTile& x, const DevTile& y) {
    return hp.sectors[x.sector].n > hp.sectors[y.sector].n;
  });
  if (coef64.size() > (size_t)0x7fffffff) return fail(PI_ERR_UNSUPPORTED, "coefficient pool too large");
  int rc;
  if ((rc = upload(plan, sectors, &plan->dev.sectors))) return rc;
  if ((rc = upload(plan, terms, &plan->dev.terms))) return rc;
  if ((rc = upload(plan, tiles, &plan->dev.tiles))) return rc;
  if ((rc = upload(plan, coef64, &plan->dev.coef64))) return rc;
  if ((rc = upload(plan, coef64z, &plan->dev.coef64z))) return rc;
  if ((rc = upload(plan, coef32x, &plan->dev.coef32x))) return rc;
  if ((rc = upload(plan, coef32z, &plan->dev.coef32z))) return rc;
  if ((rc = upload(plan, diag_sector, &plan->dev.diag_sector))) return rc;
  if (fast_sr > 0) {
    const DevTerm* ft = nullptr;
    if ((rc = upload(plan, fterms, &ft))) return rc;
    plan->dev.fterms = reinterpret_cast<const int4*>(ft);
    plan->dev.fast_sr = fast_sr;
  }
  if (!canon.empty()) {
    if ((rc = upload(plan, canon, &plan->dev.canon))) return rc;
    plan->dev.canon_plus = canon_plus;
  }
  if ((rc = upload(plan, diag_index, &plan->dev.diag_index))) return rc;
  plan->dev.nsectors = S;
  plan->dev.ntiles = (int)tiles.size();
  plan->dev.ndiag = (int)diag_index.size();
  plan->dev.dim = hp.dim;
  plan->stencil_terms = (long long)terms.size();
  plan->rs.partial = (double2*)plan_alloc(plan, sizeof(double2) * kReduceBlocks * kMaxDots);
  plan->rs.result = (double2*)plan_alloc(plan, sizeof(double2) * kMaxDots);
  plan->rs.rpartial = (double*)plan_alloc(plan, sizeof(double) * kReduceBlocks);
  plan->rs.rresult = (double*)plan_alloc(plan, sizeof(double) * 16);
  if (!plan->rs.partial || !plan->rs.result || !plan->rs.rpartial || !plan->rs.rresult)
    return fail(PI_ERR_OUT_OF_MEMORY, "device allocation of reduction scratch failed");
  cudaError_t e = cudaMallocHost((void**)&plan->host_pinned, sizeof(double) * 8 * kMaxDots);
  if (e != cudaSuccess) return cuda_fail(e, "pinned staging allocation");
  return PI_OK;
}

}  // namespace picuda

using namespace picuda;

extern "C" {

int pi_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return PI_ERR_INVALID_ARGUMENT;
  std::strncpy(buf, g_last_error.c_str(), len - 1);
  buf[len - 1] = '\0';
  return PI_OK;
}

int pi_capability(pi_capability_t* out) {
  if (!out) return fail(PI_ERR_INVALID_ARGUMENT, "null capability pointer");
  std::memset(out, 0, sizeof(*out));
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    out->functional = 0;
    return fail(PI_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
  out->device_count = count;
  out->sm_count = prop.multiProcessorCount;
  out->cc_major = prop.major;
  out->cc_minor = prop.minor;
  out->total_memory = prop.totalGlobalMem;
  size_t nl = 0;  // device name, truncated to the field
  for (; nl + 1 < sizeof(out->device_name) && prop.name[nl]; ++nl) out->device_name[nl] = prop.name[nl];
  out->device_name[nl] = '\0';
  // The kernels are built for sm_103a only.
  out->functional = (prop.major == 10 && prop.minor == 3) ? 1 : 0;
  out->supports_matrixfree_pi = out->functional;
  if (!out->functional) return fail(PI_ERR_NO_DEVICE, "libpicuda is built for sm_103a only");
  return PI_OK;
}

static int build_host_plan(int N, int d, int nsectors, const int* sector_ks, int nterms, const int* term_kind,
                           const double* ops, const double* rates, const double* hbar, QubitPlan* out) {
  if (d != 2) return fail(PI_ERR_UNSUPPORTED, "the CUDA backend supports qubit ensembles (d == 2) only");
  if (N < 1) return fail(PI_ERR_INVALID_ARGUMENT, "N must be positive");
  if (nterms < 0 || (nterms > 0 && (!term_kind || !ops || !rates)))
    return fail(PI_ERR_INVALID_ARGUMENT, "term arrays are missing");
  if (nsectors < 0 || (nsectors > 0 && !sector_ks)) return fail(PI_ERR_INVALID_ARGUMENT, "sector list is missing");
  std::vector<int> ks(sector_ks, sector_ks + (nsectors > 0 ? nsectors : 0));
  std::vector<TermSpec> terms(nterms);
  for (int t = 0; t < nterms; ++t) {
    terms[t].kind = term_kind[t];
    // column-major interleaved: element (i, j) at (i + 2j) * 2
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        terms[t].op[i][j] = std::complex<double>(ops[t * 8 + (i + 2 * j) * 2], ops[t * 8 + (i + 2 * j) * 2 + 1]);
    terms[t].rate = rates[t];
    terms[t].hbar = hbar ? hbar[t] : 1.0;
  }
  try {
    *out = build_qubit_plan(N, ks, terms);
  } catch (const std::invalid_argument& ex) {
    return fail(PI_ERR_INVALID_ARGUMENT, ex.what());
  } catch (const std::exception& ex) {
    return fail(PI_ERR_UNSUPPORTED, ex.what());
  }
  return PI_OK;
}

static QubitPlan adjoint_host_plan(const QubitPlan& hp);

static int export_plan(const QubitPlan& hp, long long* counts, int* term_table, double* coef) {
  long long nt = 0, nc = 0;
  for (const auto& sec : hp.sectors)
    for (const auto& t : sec.terms) {
      ++nt;
      nc += (long long)t.alpha.size() + (long long)t.beta.size();
    }
  counts[0] = nt;
  counts[1] = nc;
  if (!term_table || !coef) return PI_OK;
  long long it = 0, ic = 0;
  for (size_t s = 0; s < hp.sectors.size(); ++s)
    for (const auto& t : hp.sectors[s].terms) {
      int* row = term_table + 8 * it++;
      row[0] = (int)s;
      row[1] = t.src;
      row[2] = t.kind;
      row[3] = t.cls;
      row[4] = t.e + t.p;
      row[5] = t.e + t.q;
      row[6] = -1;
      row[7] = -1;
      if (!t.alpha.empty()) {
        row[6] = (int)ic;
        for (const auto& z : t.alpha) {
          coef[2 * ic] = z.real();
          coef[2 * ic + 1] = z.imag();
          ++ic;
        }
      }
      if (!t.beta.empty()) {
        row[7] = (int)ic;
        for (const auto& z : t.beta) {
          coef[2 * ic] = z.real();
          coef[2 * ic + 1] = z.imag();
          ++ic;
        }
      }
    }
  return PI_OK;
}

int pi_stencil_export(int N, int d, int nsectors, const int* sector_ks, int nterms, const int* term_kind,
                      const double* ops, const double* rates, const double* hbar, long long* counts,
                      int* term_table, double* coef) {
  if (!counts) return fail(PI_ERR_INVALID_ARGUMENT, "null counts");
  QubitPlan hp;
  int rc = build_host_plan(N, d, nsectors, sector_ks, nterms, term_kind, ops, rates, hbar, &hp);
  if (rc) return rc;
  return export_plan(hp, counts, term_table, coef);
}

int pi_stencil_export_adjoint(int N, int d, int nsectors, const int* sector_ks, int nterms, const int* term_kind,
                              const double* ops, const double* rates, const double* hbar, long long* counts,
                              int* term_table, double* coef) {
  if (!counts) return fail(PI_ERR_INVALID_ARGUMENT, "null counts");
  QubitPlan hp;
  int rc = build_host_plan(N, d, nsectors, sector_ks, nterms, term_kind, ops, rates, hbar, &hp);
  if (rc) return rc;
  return export_plan(adjoint_host_plan(hp), counts, term_table, coef);
}

int pi_precond_drive_export(int N, int d, int nsectors, const int* sector_ks, int nterms, const int* term_kind,
                            const double* ops, const double* rates, const double* hbar, long long* counts,
                            double* U, double* h, double* c, double* q) {
  if (!counts) return fail(PI_ERR_INVALID_ARGUMENT, "null counts");
  QubitPlan hp;
  int rc = build_host_plan(N, d, nsectors, sector_ks, nterms, term_kind, ops, rates, hbar, &hp);
  if (rc) return rc;
  DriveHost D;
  std::string err;
  rc = build_drive_precond(hp, PI_COORDS_REFERENCE, 1.0, &D, &err);
  if (rc) return fail(rc, err);
  counts[0] = (long long)D.n.size();
  counts[1] = (long long)D.U.size();
  counts[2] = (long long)D.h.size();
  if (U) std::copy(D.U.begin(), D.U.end(), U);
  if (h) std::copy(D.h.begin(), D.h.end(), h);
  if (c) std::copy(D.c.begin(), D.c.end(), c);
  if (q) std::copy(D.q.begin(), D.q.end(), q);
  return PI_OK;
}

int pi_precond_export(int N, int d, int nsectors, const int* sector_ks, int nterms, const int* term_kind,
                      const double* ops, const double* rates, const double* hbar, int coords, double regularization,
                      double operator_scale, long long* counts, pi_precond_tables_t* tables) {
  if (!counts) return fail(PI_ERR_INVALID_ARGUMENT, "null counts");
  if (coords != PI_COORDS_REFERENCE && coords != PI_COORDS_POPULATION)
    return fail(PI_ERR_INVALID_ARGUMENT, "coords must be PI_COORDS_REFERENCE or PI_COORDS_POPULATION");
  if (!(std::isfinite(regularization) && regularization >= 0))
    return fail(PI_ERR_INVALID_ARGUMENT, "regularization must be finite and nonnegative");
  if (!(std::isfinite(operator_scale) && operator_scale > 0))
    return fail(PI_ERR_INVALID_ARGUMENT, "operator_scale must be finite and positive");
  QubitPlan hp;
  int rc = build_host_plan(N, d, nsectors, sector_ks, nterms, term_kind, ops, rates, hbar, &hp);
  if (rc) return rc;
  LevelPrecondHost H;
  std::string err;
  rc = build_level_precond(hp, coords, regularization, operator_scale, &H, &err);
  if (rc) return fail(rc, err);
  const long long n0 = (long long)H.t0.size();
  counts[0] = (long long)H.chain_lev.size() - 1;
  counts[1] = (long long)H.lev_ent.size() - 1;
  counts[2] = (long long)H.elem.size();
  counts[3] = n0;
  if (!tables) return PI_OK;
  auto put = [](double* out, const std::vector<std::complex<double>>& v) {
    if (!out) return;
    for (size_t i = 0; i < v.size(); ++i) {
      out[2 * i] = v[i].real();
      out[2 * i + 1] = v[i].imag();
    }
  };
  if (tables->chain_lev) std::copy(H.chain_lev.begin(), H.chain_lev.end(), tables->chain_lev);
  if (tables->lev_ent) std::copy(H.lev_ent.begin(), H.lev_ent.end(), tables->lev_ent);
  if (tables->elem) std::copy(H.elem.begin(), H.elem.end(), tables->elem);
  if (tables->gsrc) std::copy(H.gsrc.begin(), H.gsrc.end(), tables->gsrc);
  put(tables->W, H.W);
  put(tables->A, H.A);
  put(tables->C, H.C);
  put(tables->G, H.G);
  if (tables->t0) std::copy(H.t0.begin(), H.t0.end(), tables->t0);
  if (tables->v0) std::copy(H.v0.begin(), H.v0.end(), tables->v0);
  if (tables->w0) {
    for (long long i = 0; i < n0; ++i) {
      const std::complex<double> w = H.w0[i];
      tables->w0[2 * i] = w.real();
      tables->w0[2 * i + 1] = w.imag();
    }
  }
  tables->meta[0] = H.chain0;
  tables->meta[1] = H.chain0_ent;
  tables->meta[2] = H.mode;
  tables->meta[3] = H.free_ent;
  tables->meta[4] = H.direction;
  tables->meta[5] = H.max_level;
  tables->meta[6] = 0;
  tables->meta[7] = 0;
  tables->sm_coef[0] = H.sm_coef.real();
  tables->sm_coef[1] = H.sm_coef.imag();
  return PI_OK;
}

int pi_collective_block(int N, int k, const double* op, double* out) {
  if (!op || !out) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (N < 1 || k < 0 || 2 * k > N) return fail(PI_ERR_INVALID_ARGUMENT, "sector is not a two-row partition of N");
  std::complex<double> X[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) X[i][j] = std::complex<double>(op[(i + 2 * j) * 2], op[(i + 2 * j) * 2 + 1]);
  try {
    auto B = collective_block_dense(N, k, X);
    for (size_t e = 0; e < B.size(); ++e) {
      out[2 * e] = B[e].real();
      out[2 * e + 1] = B[e].imag();
    }
  } catch (const std::exception& ex) {
    return fail(PI_ERR_INVALID_ARGUMENT, ex.what());
  }
  return PI_OK;
}

int pi_sector_multiplicity(int N, int k, double* f, double* sqrt_f) {
  if (N < 0 || k < 0 || 2 * k > N) return fail(PI_ERR_INVALID_ARGUMENT, "sector is not a two-row partition of N");
  const double v = sector_multiplicity_double(N, k);
  if (f) *f = v;
  if (sqrt_f) *sqrt_f = std::sqrt(v);
  return PI_OK;
}

// Device resources and tables of a plan whose host lowering is in plan->host; takes
// ownership of plan (freed on failure).
static int finish_plan(pi_plan* plan, pi_plan** out) {
  if (plan->host.dim > (long long)1 << 31) {
    delete plan;
    return fail(PI_ERR_UNSUPPORTED, "PI dimension exceeds the 32-bit tile addressing of this build");
  }
  cudaError_t e = cudaGetDevice(&plan->device);
  if (e != cudaSuccess) {
    delete plan;
    return cuda_fail(e, "cudaGetDevice");
  }
  e = cudaStreamCreateWithFlags(&plan->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete plan;
    return cuda_fail(e, "cudaStreamCreate");
  }
  for (auto& ps : plan->pipe) {
    e = cudaStreamCreateWithFlags(&ps, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      free_plan(plan);
      return cuda_fail(e, "cudaStreamCreate");
    }
  }
  int rc = upload_plan(plan);
  if (rc != PI_OK) {
    std::string msg = g_last_error;
    free_plan(plan);
    return fail(rc, msg);
  }
  *out = plan;
  return PI_OK;
}

int pi_plan_create(int N, int d, int nsectors, const int* sector_ks, int nterms, const int* term_kind,
                   const double* ops, const double* rates, const double* hbar, pi_plan** out) {
  if (!out) return fail(PI_ERR_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  pi_plan* plan = new (std::nothrow) pi_plan();
  if (!plan) return fail(PI_ERR_OUT_OF_MEMORY, "host allocation failed");
  int brc = build_host_plan(N, d, nsectors, sector_ks, nterms, term_kind, ops, rates, hbar, &plan->host);
  if (brc != PI_OK) {
    delete plan;
    return brc;
  }
  return finish_plan(plan, out);
}

// Conjugate transpose of a lowered plan (liouvillian.jl:3107-3143, 3275-3324: apply_adjoint!
// is the adjoint of the PI-coordinate matrix).  A stencil term of output sector s,
//   y_s[a, b] += c(a, b) x_r[a + e + p, b + e + q],
// contributes to the adjoint the term of output sector r with source s
//   y_r[a', b'] += conj(c(a' - e - p, b' - e - q)) x_s[a' - e - p, b' - e - q],
// i.e. shift -e, offsets (-p, -q) and the coefficient arrays conjugated and shifted (zero
// where the shifted index leaves sector s).  Kinds and coefficient classes are preserved,
// so every kernel runs the adjoint plan unchanged.
static QubitPlan adjoint_host_plan(const QubitPlan& hp) {
  QubitPlan out = hp;
  for (auto& sec : out.sectors) sec.terms.clear();
  out.max_terms = 0;
  for (int s = 0; s < (int)hp.sectors.size(); ++s) {
    const int ns = hp.sectors[s].n;
    for (const StencilTerm& t : hp.sectors[s].terms) {
      const int r = t.src;
      const int nr = hp.sectors[r].n;
      auto shifted = [&](const std::vector<cd>& v, int shift) {
        std::vector<cd> w(nr, cd(0, 0));
        for (int i = 0; i < nr; ++i) {
          const int src_i = i - shift;
          if (src_i >= 0 && src_i < ns) w[i] = std::conj(v[src_i]);
        }
        return w;
      };
      StencilTerm u;
      u.src = s;
      u.kind = t.kind;
      u.cls = t.cls;
      u.e = -t.e;
      u.p = -t.p;
      u.q = -t.q;
      if (t.kind != ST_RIGHT) u.alpha = shifted(t.alpha, t.e + t.p);
      if (t.kind != ST_LEFT) u.beta = shifted(t.beta, t.e + t.q);
      out.sectors[r].terms.push_back(std::move(u));
    }
  }
  for (const auto& sec : out.sectors) out.max_terms = std::max(out.max_terms, (int)sec.terms.size());
  return out;
}

int pi_plan_adjoint(const pi_plan* plan, pi_plan** out) {
  if (!plan || !out) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  pi_plan* adj = new (std::nothrow) pi_plan();
  if (!adj) return fail(PI_ERR_OUT_OF_MEMORY, "host allocation failed");
  adj->host = adjoint_host_plan(plan->host);
  return finish_plan(adj, out);
}

int pi_plan_destroy(pi_plan* plan) {
  free_plan(plan);
  return PI_OK;
}

int pi_plan_set_concurrency(pi_plan* plan, int mode) {
  if (!plan) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (mode != PI_CONCURRENCY_WAIT && mode != PI_CONCURRENCY_REJECT)
    return fail(PI_ERR_INVALID_ARGUMENT, "mode must be PI_CONCURRENCY_WAIT or PI_CONCURRENCY_REJECT");
  plan->reject_concurrent.store(mode == PI_CONCURRENCY_REJECT ? 1 : 0);
  return PI_OK;
}

int pi_plan_info(const pi_plan* plan, pi_plan_info_t* out) {
  if (!plan || !out) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  out->N = plan->host.N;
  out->nsectors = (int)plan->host.sectors.size();
  out->dim = plan->host.dim;
  out->max_block = plan->host.max_n;
  out->max_terms = plan->host.max_terms;
  out->stencil_terms = plan->stencil_terms;
  out->device_bytes = plan->device_bytes;
  out->batched_kernel = plan->dev.canon ? 2 : (plan->dev.fast_sr > 0 ? 1 : 0);
  return PI_OK;
}

int pi_plan_sectors(const pi_plan* plan, int* ks, long long* offsets, int* dims) {
  if (!plan) return fail(PI_ERR_INVALID_ARGUMENT, "null plan");
  const auto& sec = plan->host.sectors;
  for (size_t s = 0; s < sec.size(); ++s) {
    if (ks) ks[s] = sec[s].k;
    if (offsets) offsets[s] = sec[s].offset;
    if (dims) dims[s] = sec[s].n;
  }
  return PI_OK;
}

int pi_plan_gt_patterns(const pi_plan* plan, int sector, int* entries) {
  if (!plan || !entries) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (sector < 0 || sector >= (int)plan->host.sectors.size()) return fail(PI_ERR_INVALID_ARGUMENT, "sector out of range");
  const auto& sec = plan->host.sectors[sector];
  const int N = plan->host.N;
  for (int a = 0; a < sec.n; ++a) {
    entries[3 * a] = sec.k + a;  // row 1 entry m, ascending
    entries[3 * a + 1] = N - sec.k;
    entries[3 * a + 2] = sec.k;
  }
  return PI_OK;
}

int pi_plan_trace_functional(const pi_plan* plan, long long* idx, double* vals) {
  if (!plan || !idx || !vals) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  long long i = 0;
  for (const auto& sec : plan->host.sectors)
    for (int a = 0; a < sec.n; ++a, ++i) {
      idx[i] = sec.offset + a + (long long)a * sec.n;
      vals[i] = sec.sqrt_f;
    }
  return PI_OK;
}

int pi_plan_sector_scales(const pi_plan* plan, double* sqrt_f) {
  if (!plan || !sqrt_f) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  for (size_t s = 0; s < plan->host.sectors.size(); ++s) sqrt_f[s] = plan->host.sectors[s].sqrt_f;
  return PI_OK;
}

static int check_apply_args(pi_plan* plan, const void* y, const void* x, int ncols, long long ld, size_t elem) {
  if (!plan || !x || !y) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (ncols < 1 || ncols > 65535) return fail(PI_ERR_INVALID_ARGUMENT, "ncols must lie in 1:65535");
  if (ld < plan->host.dim) return fail(PI_ERR_DIMENSION, "leading dimension is smaller than the PI dimension");
  const size_t bytes = ((size_t)(ncols - 1) * (size_t)ld + (size_t)plan->host.dim) * elem;
  if (overlap(x, bytes, y, bytes))
    return fail(PI_ERR_INVALID_ARGUMENT, "source and destination must not share storage");
  return PI_OK;
}

int pi_apply_f64(pi_plan* plan, double* y_dev, const double* x_dev, int ncols, long long ld, void* stream) {
  int rc = check_apply_args(plan, y_dev, x_dev, ncols, ld, sizeof(double2));
  if (rc) return rc;
  BorderArgs border{1.0, nullptr, 0};
  cudaStream_t s = (cudaStream_t)stream;  // NULL is the CUDA default stream
  cudaError_t e = launch_apply_f64(plan->dev, x_dev, y_dev, ncols, ld, border, s);
  if (e != cudaSuccess) return cuda_fail(e, "apply launch");
  return PI_OK;
}

int pi_apply_f32(pi_plan* plan, float* y_dev, const float* x_dev, int ncols, long long ld, int coords,
                 void* stream) {
  int rc = check_apply_args(plan, y_dev, x_dev, ncols, ld, sizeof(float2));
  if (rc) return rc;
  if (coords != PI_COORDS_REFERENCE && coords != PI_COORDS_POPULATION)
    return fail(PI_ERR_INVALID_ARGUMENT, "coords must be PI_COORDS_REFERENCE or PI_COORDS_POPULATION");
  BorderArgs border{1.0, nullptr, coords};
  cudaStream_t s = (cudaStream_t)stream;  // NULL is the CUDA default stream
  cudaError_t e = launch_apply_f32(plan->dev, x_dev, y_dev, ncols, ld, border, s);
  if (e != cudaSuccess) return cuda_fail(e, "apply launch");
  return PI_OK;
}

}  // extern "C"

// Host-buffer apply: the columns are split into chunks that cycle through three streams,
// so the host-to-device copy of one chunk, the apply of the previous one and the
// device-to-host copy of the one before overlap on the link and the SMs.  Device staging
// is grow-only and owned by the plan.
template <typename T>
static int apply_host(pi_plan* plan, void* y_host, const void* x_host, int ncols, int coords) {
  if (!plan || !y_host || !x_host) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  if (ncols < 1 || ncols > 65535) return fail(PI_ERR_INVALID_ARGUMENT, "ncols must lie in 1:65535");
  if (coords != PI_COORDS_REFERENCE && coords != PI_COORDS_POPULATION)
    return fail(PI_ERR_INVALID_ARGUMENT, "coords must be PI_COORDS_REFERENCE or PI_COORDS_POPULATION");
  const size_t col_bytes = (size_t)plan->host.dim * 2 * sizeof(T);
  const size_t bytes = (size_t)ncols * col_bytes;
  if (overlap(x_host, bytes, y_host, bytes))
    return fail(PI_ERR_INVALID_ARGUMENT, "source and destination must not share storage");
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  cudaError_t e = cudaSuccess;
  if (plan->stage_bytes < bytes) {
    if (plan->stage_x) cudaFree(plan->stage_x);
    if (plan->stage_y) cudaFree(plan->stage_y);
    plan->stage_x = plan->stage_y = nullptr;
    plan->stage_bytes = 0;
    e = cudaMalloc(&plan->stage_x, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&plan->stage_y, bytes);
    if (e != cudaSuccess) {
      if (plan->stage_x) cudaFree(plan->stage_x);
      plan->stage_x = nullptr;
      return cuda_fail(e, "host-apply staging allocation");
    }
    plan->stage_bytes = bytes;
  }
  // Chunks of at least 1 column.  The first upload and the last download overlap nothing, so
  // smaller chunks shorten them, while each chunk adds launch and copy setup.  At 128 columns
  // of N=120: FP64 (compute-heavy chunks) 16 chunks measured 5% faster than 8 and 32 chunks
  // 6% slower; FP32 (copy-bound chunks) 8 chunks measured faster than 16 (2.13 vs 2.33 ms).
  const int nchunks = sizeof(T) == sizeof(double) ? 16 : 8;
  const int chunk = std::max(1, (ncols + nchunks - 1) / nchunks);
  BorderArgs border{1.0, nullptr, coords};
  int k = 0;
  for (int c0 = 0; c0 < ncols && e == cudaSuccess; c0 += chunk, ++k) {
    const int nc = std::min(chunk, ncols - c0);
    cudaStream_t s = plan->pipe[k % 3];
    char* dx = (char*)plan->stage_x + (size_t)c0 * col_bytes;
    char* dy = (char*)plan->stage_y + (size_t)c0 * col_bytes;
    e = cudaMemcpyAsync(dx, (const char*)x_host + (size_t)c0 * col_bytes, (size_t)nc * col_bytes,
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      if (sizeof(T) == sizeof(double))
        e = launch_apply_f64(plan->dev, (const double*)dx, (double*)dy, nc, plan->host.dim, border, s);
      else
        e = launch_apply_f32(plan->dev, (const float*)dx, (float*)dy, nc, plan->host.dim, border, s);
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync((char*)y_host + (size_t)c0 * col_bytes, dy, (size_t)nc * col_bytes, cudaMemcpyDeviceToHost, s);
  }
  cudaError_t e2 = cudaSuccess;
  for (auto& ps : plan->pipe) {
    cudaError_t e3 = cudaStreamSynchronize(ps);
    if (e3 != cudaSuccess && e2 == cudaSuccess) e2 = e3;
  }
  if (e != cudaSuccess) return cuda_fail(e, "host apply");
  if (e2 != cudaSuccess) return cuda_fail(e2, "host apply synchronize");
  return PI_OK;
}

extern "C" {

int pi_apply_host_f64(pi_plan* plan, double* y_host, const double* x_host, int ncols) {
  return apply_host<double>(plan, y_host, x_host, ncols, PI_COORDS_REFERENCE);
}

int pi_apply_host_f32(pi_plan* plan, float* y_host, const float* x_host, int ncols, int coords) {
  return apply_host<float>(plan, y_host, x_host, ncols, coords);
}

int pi_dot_f64(pi_plan* plan, const double* a_dev, const double* b_dev, double* out_host2) {
  if (!plan || !a_dev || !b_dev || !out_host2) return fail(PI_ERR_INVALID_ARGUMENT, "null argument");
  BusyGuard guard(plan);
  if (!guard.ok) return fail(PI_ERR_BUSY, "a pi_plan cannot be used concurrently");
  cudaStream_t s = plan->stream;
  cudaError_t e = mdot_f64((const double2*)a_dev, plan->host.dim, 1, (const double2*)b_dev, plan->host.dim,
                           plan->rs, plan->rs.result, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(plan->host_pinned, plan->rs.result, sizeof(double2), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "dot");
  out_host2[0] = plan->host_pinned[0];
  out_host2[1] = plan->host_pinned[1];
  return PI_OK;
}

}  // extern "C"
