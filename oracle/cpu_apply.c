/*
 * CPU restatement of the reference's threaded matrix-free apply (TEST INFRASTRUCTURE ONLY;
 * used as the checker's CPU baseline, never by the product).
 *
 * Follows src/threaded_apply.jl:58-84 (LPT sector schedule, cost n^3 + n, deterministic
 * tie break) and :506-609 (output-sector-owned workers), applying per output sector the
 * fused static kernel of src/liouvillian.jl:3070-3105:
 *   Y  = -i (H X - X H)                       sparse Hamiltonian block
 *   Y += rate_g K_g X K_g^H                    collective gains
 *   Y -= (Q X + X Q) / 2                       fused loss block
 *   Y += r s_b C_b X_nu C_b^H                  one-body gain branches, support path
 *                                              (liouvillian.jl:2486-2537)
 * Sparse blocks arrive as per-sector COO ranges built by oracle/pi_oracle.py.
 * Complex numbers are interleaved (re, im) doubles.
 */
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int nsec;
  const long long* off;
  const int* dim;
  /* Hamiltonian and loss: COO per sector, ranges ptr[s]..ptr[s+1] */
  const long long* h_ptr; const int* h_row; const int* h_col; const double* h_val;
  const long long* q_ptr; const int* q_row; const int* q_col; const double* q_val;
  /* collective gains: ncg blocks sets, ranges k_ptr[g*nsec + s] */
  int ncg; const double* cg_rate;
  const long long* k_ptr; const int* k_row; const int* k_col; const double* k_val;
  /* one-body branches sorted by output sector: br_ptr[s]..br_ptr[s+1] */
  const long long* br_ptr; const int* br_in; const double* br_scale;
  const long long* c_ptr; const int* c_row; const int* c_col; const double* c_val;
} oracle_plan;

static void sparse_left(const long long* p, const int* row, const int* col, const double* val, long long b0,
                        long long b1, const double* X, int n, double* out, double sr, double si) {
  /* out += (sr + i si) * (A X), A in COO */
  for (long long e = b0; e < b1; ++e) {
    const int a = row[e], c = col[e];
    const double vr = val[2 * e] * sr - val[2 * e + 1] * si;
    const double vi = val[2 * e] * si + val[2 * e + 1] * sr;
    for (int b = 0; b < n; ++b) {
      const double xr = X[2 * (c + (long long)b * n)], xi = X[2 * (c + (long long)b * n) + 1];
      out[2 * (a + (long long)b * n)] += vr * xr - vi * xi;
      out[2 * (a + (long long)b * n) + 1] += vr * xi + vi * xr;
    }
  }
  (void)p;
}

static void sparse_right(const int* row, const int* col, const double* val, long long b0, long long b1,
                         const double* X, int n, double* out, double sr, double si) {
  /* out += (sr + i si) * (X A), A in COO: (X A)[a, cc] += X[a, r] A[r, cc] */
  for (long long e = b0; e < b1; ++e) {
    const int r = row[e], cc = col[e];
    const double vr = val[2 * e] * sr - val[2 * e + 1] * si;
    const double vi = val[2 * e] * si + val[2 * e + 1] * sr;
    for (int a = 0; a < n; ++a) {
      const double xr = X[2 * (a + (long long)r * n)], xi = X[2 * (a + (long long)r * n) + 1];
      out[2 * (a + (long long)cc * n)] += vr * xr - vi * xi;
      out[2 * (a + (long long)cc * n) + 1] += vr * xi + vi * xr;
    }
  }
}

static void sandwich(const int* row, const int* col, const double* val, long long b0, long long b1,
                     const double* X, int nin, double* out, int nout, double scale) {
  /* out[rows[l], rows[r]] += scale * val_l * conj(val_r) * X[cols[l], cols[r]] */
  for (long long r = b0; r < b1; ++r) {
    const int oc = row[r], ic = col[r];
    const double rr = val[2 * r], ri = -val[2 * r + 1];
    for (long long l = b0; l < b1; ++l) {
      const int orow = row[l], irow = col[l];
      const double lr = val[2 * l] * rr - val[2 * l + 1] * ri;
      const double li = val[2 * l] * ri + val[2 * l + 1] * rr;
      const double xr = X[2 * (irow + (long long)ic * nin)], xi = X[2 * (irow + (long long)ic * nin) + 1];
      out[2 * (orow + (long long)oc * nout)] += scale * (lr * xr - li * xi);
      out[2 * (orow + (long long)oc * nout) + 1] += scale * (lr * xi + li * xr);
    }
  }
}

static void apply_sector(const oracle_plan* P, int s, const double* x, double* y, double* scratch) {
  const int n = P->dim[s];
  const double* X = x + 2 * P->off[s];
  double* out = y + 2 * P->off[s];
  memset(out, 0, sizeof(double) * 2 * (size_t)n * n);
  /* -i (H X - X H) */
  sparse_left(P->h_ptr, P->h_row, P->h_col, P->h_val, P->h_ptr[s], P->h_ptr[s + 1], X, n, out, 0.0, -1.0);
  sparse_right(P->h_row, P->h_col, P->h_val, P->h_ptr[s], P->h_ptr[s + 1], X, n, out, 0.0, 1.0);
  /* collective gains rate K X K^H: scratch = K X, out += rate * scratch K^H */
  for (int g = 0; g < P->ncg; ++g) {
    const long long b0 = P->k_ptr[g * P->nsec + s], b1 = P->k_ptr[g * P->nsec + s + 1];
    memset(scratch, 0, sizeof(double) * 2 * (size_t)n * n);
    sparse_left(P->k_ptr, P->k_row, P->k_col, P->k_val, b0, b1, X, n, scratch, 1.0, 0.0);
    /* (scratch K^H)[a, c] = sum_r scratch[a, r] conj(K[c, r]) */
    for (long long e = b0; e < b1; ++e) {
      const int c = P->k_row[e], r = P->k_col[e];
      const double vr = P->cg_rate[g] * P->k_val[2 * e], vi = -P->cg_rate[g] * P->k_val[2 * e + 1];
      for (int a = 0; a < n; ++a) {
        const double xr = scratch[2 * (a + (long long)r * n)], xi = scratch[2 * (a + (long long)r * n) + 1];
        out[2 * (a + (long long)c * n)] += vr * xr - vi * xi;
        out[2 * (a + (long long)c * n) + 1] += vr * xi + vi * xr;
      }
    }
  }
  /* - (Q X + X Q) / 2 */
  sparse_left(P->q_ptr, P->q_row, P->q_col, P->q_val, P->q_ptr[s], P->q_ptr[s + 1], X, n, out, -0.5, 0.0);
  sparse_right(P->q_row, P->q_col, P->q_val, P->q_ptr[s], P->q_ptr[s + 1], X, n, out, -0.5, 0.0);
  /* one-body gain branches into this output sector */
  for (long long b = P->br_ptr[s]; b < P->br_ptr[s + 1]; ++b) {
    const int ni = P->br_in[b];
    sandwich(P->c_row, P->c_col, P->c_val, P->c_ptr[b], P->c_ptr[b + 1], x + 2 * P->off[ni], P->dim[ni], out, n,
             P->br_scale[b]);
  }
}

/* LPT assignment (threaded_apply.jl:69-84): returns worker of each sector in `owner`. */
static void lpt(const oracle_plan* P, int workers, int* owner) {
  int ns = P->nsec;
  int* order = (int*)malloc(sizeof(int) * ns);
  double* load = (double*)calloc((size_t)workers, sizeof(double));
  for (int s = 0; s < ns; ++s) order[s] = s;
  for (int i = 1; i < ns; ++i) { /* insertion sort by (-cost, index) */
    int v = order[i], j = i - 1;
    double cv = (double)P->dim[v] * P->dim[v] * P->dim[v] + P->dim[v];
    while (j >= 0) {
      double cj = (double)P->dim[order[j]] * P->dim[order[j]] * P->dim[order[j]] + P->dim[order[j]];
      if (cj < cv || (cj == cv && order[j] > v)) {
        order[j + 1] = order[j];
        --j;
      } else {
        break;
      }
    }
    order[j + 1] = v;
  }
  for (int i = 0; i < ns; ++i) {
    int s = order[i], w = 0;
    for (int k = 1; k < workers; ++k)
      if (load[k] < load[w]) w = k;
    owner[s] = w;
    load[w] += (double)P->dim[s] * P->dim[s] * P->dim[s] + P->dim[s];
  }
  free(order);
  free(load);
}

int oracle_apply(const oracle_plan* P, const double* x, double* y, int nthreads) {
  int maxn = 1;
  for (int s = 0; s < P->nsec; ++s)
    if (P->dim[s] > maxn) maxn = P->dim[s];
  if (nthreads < 1) nthreads = 1;
  int workers = nthreads < P->nsec ? nthreads : P->nsec;
  if (workers < 1) workers = 1;
  int* owner = (int*)malloc(sizeof(int) * (P->nsec > 0 ? P->nsec : 1));
  lpt(P, workers, owner);
#ifdef _OPENMP
#pragma omp parallel num_threads(workers)
#endif
  {
    int w = 0;
#ifdef _OPENMP
    w = omp_get_thread_num();
#endif
    double* scratch = (double*)malloc(sizeof(double) * 2 * (size_t)maxn * maxn);
    for (int s = 0; s < P->nsec; ++s)
      if (owner[s] == w) apply_sector(P, s, x, y, scratch);
    free(scratch);
  }
  free(owner);
  return 0;
}
