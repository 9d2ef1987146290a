// Host-side lowering of a qubit PI model into separable stencil terms.
// See pi_plan.hpp for the stencil form.  Every routine cites the reference routine whose
// arithmetic it restates.
#include "pi_plan.hpp"

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <stdexcept>
#include <utility>

namespace picuda {
namespace {

// ---------------------------------------------------------------------------------------
// Exact rationals with 64-bit numerator/denominator (all qubit CG and branch-weight
// factors are ratios of integers <= N + 2, so a handful of products stays far inside
// this range; every step is checked).
// ---------------------------------------------------------------------------------------
struct Rational {
  long long num = 0, den = 1;
};

Rational make_rat(__int128 n, __int128 d) {
  if (d == 0) throw std::invalid_argument("singular CG product");
  if (d < 0) {
    n = -n;
    d = -d;
  }
  __int128 a = n < 0 ? -n : n, b = d;
  while (b) {
    __int128 t = a % b;
    a = b;
    b = t;
  }
  if (a > 1) {
    n /= a;
    d /= a;
  }
  const __int128 lim = (__int128)1 << 62;
  if (n > lim || n < -lim || d > lim) throw std::overflow_error("rational overflow in plan setup");
  return Rational{(long long)n, (long long)d};
}

Rational mul(Rational x, Rational y) { return make_rat((__int128)x.num * y.num, (__int128)x.den * y.den); }
Rational divr(Rational x, Rational y) { return make_rat((__int128)x.num * y.den, (__int128)x.den * y.num); }

// sqrt of the correctly rounded double of an exact ratio (partitions.jl:130-160).
// Numerator and denominator are below 2^53 here, so the IEEE quotient is correctly
// rounded.
double sqrt_ratio(Rational r) {
  if (r.num < 0) throw std::invalid_argument("negative squared coefficient");
  if (r.num > (1LL << 53) || r.den > (1LL << 53)) {
    long double v = (long double)r.num / (long double)r.den;
    return std::sqrt((double)v);
  }
  return std::sqrt((double)r.num / (double)r.den);
}

// ---------------------------------------------------------------------------------------
// Minimal unsigned big integer for exact f^lambda (hook-length values reach ~1e87 at
// N = 300) with a correctly rounded conversion to double.
// ---------------------------------------------------------------------------------------
struct BigUInt {
  std::vector<uint32_t> limb;  // little endian
  explicit BigUInt(uint64_t v = 0) {
    while (v) {
      limb.push_back((uint32_t)v);
      v >>= 32;
    }
  }
  bool zero() const { return limb.empty(); }
  void mul_small(uint32_t m) {
    uint64_t carry = 0;
    for (auto& w : limb) {
      uint64_t t = (uint64_t)w * m + carry;
      w = (uint32_t)t;
      carry = t >> 32;
    }
    if (carry) limb.push_back((uint32_t)carry);
    if (m == 0) limb.clear();
  }
  // exact division by a small integer (asserts divisibility)
  void div_small(uint32_t d) {
    uint64_t rem = 0;
    for (size_t i = limb.size(); i-- > 0;) {
      uint64_t cur = (rem << 32) | limb[i];
      limb[i] = (uint32_t)(cur / d);
      rem = cur % d;
    }
    if (rem) throw std::logic_error("inexact big-integer division");
    while (!limb.empty() && limb.back() == 0) limb.pop_back();
  }
  int bits() const {
    if (limb.empty()) return 0;
    int b = 32 * (int)(limb.size() - 1);
    uint32_t top = limb.back();
    while (top) {
      ++b;
      top >>= 1;
    }
    return b;
  }
  bool bit(int i) const {
    size_t w = (size_t)i / 32;
    return w < limb.size() && ((limb[w] >> (i % 32)) & 1u);
  }
  // round-to-nearest-even conversion
  double to_double() const {
    int nb = bits();
    if (nb == 0) return 0.0;
    if (nb <= 53) {
      double v = 0.0;
      for (size_t i = limb.size(); i-- > 0;) v = v * 4294967296.0 + (double)limb[i];
      return v;
    }
    uint64_t mant = 0;
    for (int i = nb - 1; i >= nb - 53; --i) mant = (mant << 1) | (bit(i) ? 1u : 0u);
    int shift = nb - 53;
    bool half = bit(shift - 1);
    bool sticky = false;
    for (int i = shift - 2; i >= 0 && !sticky; --i) sticky = bit(i);
    if (half && (sticky || (mant & 1))) mant += 1;
    return std::ldexp((double)mant, shift);
  }
  std::string decimal() const {
    if (limb.empty()) return "0";
    BigUInt t = *this;
    std::string s;
    while (!t.limb.empty()) {
      uint64_t rem = 0;
      for (size_t i = t.limb.size(); i-- > 0;) {
        uint64_t cur = (rem << 32) | t.limb[i];
        t.limb[i] = (uint32_t)(cur / 10);
        rem = cur % 10;
      }
      while (!t.limb.empty() && t.limb.back() == 0) t.limb.pop_back();
      s.push_back((char)('0' + rem));
    }
    std::reverse(s.begin(), s.end());
    return s;
  }
};

// f^(N-k,k) = C(N,k) (N-2k+1)/(N-k+1): hook-length value of a two-row diagram
// (partitions.jl:119-127 evaluates the same integer by the hook-length product).
BigUInt two_row_dimension(int N, int k) {
  BigUInt v(1);
  for (int i = 1; i <= k; ++i) {
    v.mul_small((uint32_t)(N - k + i));
    v.div_small((uint32_t)i);
  }
  v.mul_small((uint32_t)(N - 2 * k + 1));
  v.div_small((uint32_t)(N - k + 1));
  return v;
}

// ---------------------------------------------------------------------------------------
// GT patterns for d = 2 are stored row by row as {m, lam1, lam2} (gtpatterns.jl:2-22);
// ascending entry order inside sector (lam1, lam2) is ascending m in [lam2, lam1], so the
// in-block index is a = m - lam2 (gtpatterns.jl:92-106).
// ---------------------------------------------------------------------------------------
inline int gt_entry(const int g[3], int i, int k) { return g[k * (k - 1) / 2 + i - 1]; }
inline int gt_p(const int g[3], int i, int k) { return gt_entry(g, i, k) + k - i; }

// triangular_shift for D = 2 (gtpatterns.jl:109-122).
bool triangular_shift2(const int mu[3], const int lam[3], int j, int tau[2], int* ntau) {
  const int D = 2;
  if (j < 0 || j >= D) return false;
  *ntau = 0;
  for (int k = 1; k <= D; ++k) {
    int dif[2];
    for (int i = 1; i <= k; ++i) dif[i - 1] = gt_entry(lam, i, k) - gt_entry(mu, i, k);
    if (k <= j) {
      for (int i = 0; i < k; ++i)
        if (dif[i] != 0) return false;
    } else {
      int ones = 0, pos = 0;
      for (int i = 0; i < k; ++i) {
        if (dif[i] == 1) {
          ++ones;
          if (ones == 1) pos = i + 1;
        } else if (dif[i] != 0) {
          return false;
        }
      }
      if (ones != 1) return false;
      tau[(*ntau)++] = pos;
    }
  }
  return true;
}

}  // namespace

// Exact one-box CG coefficient (cgc.jl:6-39) specialised to D = 2.
bool cgc_qubit_exact(const int mu[3], int j, const int lam[3], int* sign_out, long long* num,
                     long long* den) {
  const int D = 2;
  if (lam[1] + lam[2] != mu[1] + mu[2] + 1) return false;
  int tau[2], ntau = 0;
  if (!triangular_shift2(mu, lam, j, tau, &ntau)) return false;
  int tj = tau[0];
  Rational q{1, 1};
  for (int k = 1; k <= j; ++k) q = mul(q, Rational{gt_p(mu, tj, j + 1) - gt_p(mu, k, j), 1});
  for (int k = 1; k <= j + 1; ++k) {
    if (k == tj) continue;
    q = divr(q, Rational{gt_p(mu, tj, j + 1) - gt_p(mu, k, j + 1), 1});
  }
  int sign = 1;
  for (int l = j + 2; l <= D; ++l) {
    int tprev = tau[l - j - 2], tl = tau[l - j - 1];
    sign *= tprev < tl ? -1 : 1;
    for (int k = 1; k <= l; ++k) {
      if (k == tl) continue;
      q = mul(q, make_rat(gt_p(mu, tprev, l - 1) - gt_p(mu, k, l) + 1, gt_p(mu, tl, l) - gt_p(mu, k, l)));
    }
    for (int k = 1; k <= l - 1; ++k) {
      if (k == tprev) continue;
      q = mul(q, make_rat(gt_p(mu, tl, l) - gt_p(mu, k, l - 1), gt_p(mu, tprev, l - 1) - gt_p(mu, k, l - 1) + 1));
    }
  }
  if (q.num < 0) throw std::invalid_argument("negative squared CG coefficient");
  if (q.num == 0) return false;
  *sign_out = sign;
  *num = q.num;
  *den = q.den;
  return true;
}

std::string symmetric_group_dimension_decimal(int N, int k) { return two_row_dimension(N, k).decimal(); }

double sector_multiplicity_double(int N, int k) { return two_row_dimension(N, k).to_double(); }

namespace {

// Exact |lam| f^mu / f^lam (partitions.jl:519-543) for two-row diagrams; row is the
// one-based row from which the box is removed.
Rational branch_weight(int lam1, int lam2, int row) {
  const int D = 2;
  int shifted[2] = {lam1 + D - 1, lam2 + D - 2};
  int r = row - 1;
  int pivot = shifted[r];
  Rational result{pivot, 1};
  for (int index = 0; index < r; ++index) {
    int diff = shifted[index] - pivot;
    result = mul(result, make_rat(diff + 1, diff));
  }
  for (int index = r + 1; index < D; ++index) {
    int diff = pivot - shifted[index];
    result = mul(result, make_rat(diff - 1, diff));
  }
  return result;
}

struct Transition {
  int parent;  // parent pattern index
  int label;   // 0 = |g>, 1 = |e>
  double value;
};

// Child of sector (N-k, k) obtained by removing the box of `row`.
struct Child {
  int row;
  int mu1, mu2;
};

std::vector<Child> children_of(int N, int k) {
  std::vector<Child> out;
  int l1 = N - k, l2 = k;
  if (l1 > l2) out.push_back({1, l1 - 1, l2});  // removable_corners: row 1 first
  if (l2 > 0) out.push_back({2, l1, l2 - 1});
  return out;
}

// One-body transitions parent sector -> child (geometry.jl:465-490).
std::vector<std::vector<Transition>> transitions_for(int N, int k, const Child& c) {
  int l1 = N - k, l2 = k;
  int nchild = c.mu1 - c.mu2 + 1;
  std::vector<std::vector<Transition>> t(nchild);
  for (int ci = 0; ci < nchild; ++ci) {
    int mc = c.mu2 + ci;
    int child[3] = {mc, c.mu1, c.mu2};
    for (int label = 0; label < 2; ++label) {
      // content(child) + e_label; content[0] = m, so label 0 raises m by one.
      int mp = mc + (label == 0 ? 1 : 0);
      if (mp < l2 || mp > l1) continue;
      int parent[3] = {mp, l1, l2};
      int sign;
      long long num, den;
      if (!cgc_qubit_exact(child, label, parent, &sign, &num, &den)) continue;
      double v = (double)sign * sqrt_ratio(Rational{num, den});
      if (v != 0.0) t[ci].push_back({mp - l2, label, v});
    }
  }
  return t;
}

struct Cell {
  int a, c;
  std::vector<std::pair<int, double>> terms;  // (i*2 + j, value)
};

// Packed contraction cells for (lambda, mu, nu) (geometry.jl:405-439); the term order
// inside a cell is child, then left transition, then right transition.
std::vector<Cell> pack_cells(const std::vector<std::vector<Transition>>& left,
                             const std::vector<std::vector<Transition>>& right) {
  std::vector<Cell> cells;
  std::map<std::pair<int, int>, size_t> where;
  for (size_t ci = 0; ci < left.size(); ++ci) {
    for (const auto& L : left[ci]) {
      for (const auto& R : right[ci]) {
        double value = L.value * R.value;
        if (value == 0.0) continue;
        auto key = std::make_pair(L.parent, R.parent);
        auto it = where.find(key);
        size_t idx;
        if (it == where.end()) {
          idx = cells.size();
          where.emplace(key, idx);
          cells.push_back(Cell{L.parent, R.parent, {}});
        } else {
          idx = it->second;
        }
        cells[idx].terms.push_back({L.label * 2 + R.label, value});
      }
    }
  }
  return cells;
}

// Banded rectangular matrix between an output sector (rows, n_r) and a source sector
// (columns, n_c); entry [a, c] with c = a + e + p is stored as diag[p + 2][a].
struct Band {
  int nr = 0, nc = 0, e = 0;
  std::vector<cd> diag[5];
  Band() = default;
  Band(int nr_, int nc_, int e_) : nr(nr_), nc(nc_), e(e_) {
    for (auto& d : diag) d.assign(nr, cd(0, 0));
  }
  void add(int a, int c, cd v) {
    int p = c - a - e;
    if (p < -2 || p > 2) throw std::logic_error("entry outside the stencil band");
    diag[p + 2][a] += v;
  }
  cd get(int a, int c) const {
    int p = c - a - e;
    if (p < -2 || p > 2 || a < 0 || a >= nr || c < 0 || c >= nc) return cd(0, 0);
    return diag[p + 2][a];
  }
  bool has(int p) const {
    for (const auto& v : diag[p + 2])
      if (v != cd(0, 0)) return true;
    return false;
  }
};

inline cd contract(const Cell& cell, const cd X[2][2]) {
  // _contract: sum(conj(z) * X[i,j]) from zero (geometry.jl:867-870); z is real.
  cd v(0, 0);
  for (const auto& t : cell.terms) v += t.second * X[t.first / 2][t.first % 2];
  return v;
}

int classify(const std::vector<cd>& v) {
  bool re = true, im = true;
  for (const auto& z : v) {
    if (z.imag() != 0.0) re = false;
    if (z.real() != 0.0) im = false;
  }
  if (re) return CC_REAL;
  if (im) return CC_IMAG;
  return CC_CPLX;
}

}  // namespace

std::vector<cd> collective_block_dense(int N, int k, const cd X[2][2]) {
  int n = N - 2 * k + 1;
  std::vector<cd> out((size_t)n * n, cd(0, 0));
  for (const Child& c : children_of(N, k)) {
    auto t = transitions_for(N, k, c);
    auto cells = pack_cells(t, t);
    Rational w = branch_weight(N - k, k, c.row);
    double scale = sqrt_ratio(mul(w, w));
    for (const auto& cell : cells) out[(size_t)cell.a + (size_t)cell.c * n] += scale * contract(cell, X);
  }
  return out;
}

QubitPlan build_qubit_plan(int N, std::vector<int> ks, const std::vector<TermSpec>& terms) {
  if (N < 1) throw std::invalid_argument("N must be positive");
  if (N > 20000) throw std::invalid_argument("N is outside the supported range");
  if (ks.empty()) {
    for (int k = 0; 2 * k <= N; ++k) ks.push_back(k);
  }
  std::sort(ks.begin(), ks.end());  // descending partitions == ascending k (basis.jl:27)
  for (size_t i = 0; i < ks.size(); ++i) {
    if (ks[i] < 0 || 2 * ks[i] > N) throw std::invalid_argument("sector is not a two-row partition of N");
    if (i && ks[i] == ks[i - 1]) throw std::invalid_argument("duplicate sector");
  }
  QubitPlan plan;
  plan.N = N;
  const int S = (int)ks.size();
  std::map<int, int> index_of;
  long long off = 0;
  for (int s = 0; s < S; ++s) {
    Sector sec;
    sec.k = ks[s];
    sec.n = N - 2 * ks[s] + 1;
    sec.offset = off;
    BigUInt f = two_row_dimension(N, ks[s]);
    sec.f = f.to_double();
    sec.sqrt_f = std::sqrt(sec.f);
    off += (long long)sec.n * sec.n;
    plan.max_n = std::max(plan.max_n, sec.n);
    index_of[ks[s]] = s;
    plan.sectors.push_back(std::move(sec));
  }
  plan.dim = off;
  for (const auto& sec : plan.sectors) plan.trace_norm2 += (double)sec.n * (sec.sqrt_f * sec.sqrt_f);

  // Geometry: transitions per (sector, child) and branch weights (geometry.jl:519-562).
  std::vector<std::vector<Child>> kids(S);
  std::vector<std::vector<std::vector<std::vector<Transition>>>> trans(S);
  for (int s = 0; s < S; ++s) {
    kids[s] = children_of(N, ks[s]);
    for (const auto& c : kids[s]) trans[s].push_back(transitions_for(N, ks[s], c));
  }
  auto child_index = [&](int s, int mu1, int mu2) -> int {
    for (size_t i = 0; i < kids[s].size(); ++i)
      if (kids[s][i].mu1 == mu1 && kids[s][i].mu2 == mu2) return (int)i;
    return -1;
  };

  // Collective block of X in sector s as a band (geometry.jl:840-865).
  auto collective_band = [&](int s, const cd X[2][2]) {
    const Sector& sec = plan.sectors[s];
    Band b(sec.n, sec.n, 0);
    std::map<std::pair<int, int>, cd> acc;
    std::vector<std::pair<int, int>> order;
    for (size_t ci = 0; ci < kids[s].size(); ++ci) {
      Rational w = branch_weight(N - sec.k, sec.k, kids[s][ci].row);
      double scale = sqrt_ratio(mul(w, w));
      for (const auto& cell : pack_cells(trans[s][ci], trans[s][ci])) {
        auto key = std::make_pair(cell.a, cell.c);
        auto it = acc.find(key);
        if (it == acc.end()) {
          acc.emplace(key, scale * contract(cell, X));
          order.push_back(key);
        } else {
          it->second += scale * contract(cell, X);
        }
      }
    }
    for (const auto& key : order) {
      cd v = acc[key];
      if (v != cd(0, 0)) b.add(key.first, key.second, v);
    }
    return b;
  };

  // Fused Hamiltonian and loss blocks (liouvillian.jl:1543-1640), collective gains
  // (liouvillian.jl:1318-1333) and one-body gain branches (liouvillian.jl:1354-1371).
  std::vector<Band> H(S), Q(S);
  for (int s = 0; s < S; ++s) {
    H[s] = Band(plan.sectors[s].n, plan.sectors[s].n, 0);
    Q[s] = Band(plan.sectors[s].n, plan.sectors[s].n, 0);
  }
  struct CollGain {
    std::vector<Band> K;
    double rate;
  };
  std::vector<CollGain> cgains;
  std::vector<const TermSpec*> local_jumps;
  for (const auto& t : terms) {
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        if (!std::isfinite(t.op[i][j].real()) || !std::isfinite(t.op[i][j].imag()))
          throw std::invalid_argument("fixed operator prototypes must contain only finite coefficients");
    if (!std::isfinite(t.rate)) throw std::invalid_argument("rates must be finite");
    if (t.kind == TERM_HAMILTONIAN) {
      if (!std::isfinite(t.hbar) || t.hbar == 0.0) throw std::invalid_argument("Hamiltonian hbar must be finite and nonzero");
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
          if (std::abs(t.op[i][j] - std::conj(t.op[j][i])) > 0.0)
            throw std::invalid_argument("Hamiltonian prototype must be Hermitian");
      double scale = t.rate / t.hbar;
      for (int s = 0; s < S; ++s) {
        Band b = collective_band(s, t.op);
        for (int p = -2; p <= 2; ++p)
          for (int a = 0; a < b.nr; ++a) H[s].diag[p + 2][a] += scale * b.diag[p + 2][a];
      }
    } else if (t.kind == TERM_COLLECTIVE_JUMP) {
      CollGain g;
      g.rate = t.rate;
      for (int s = 0; s < S; ++s) {
        Band K = collective_band(s, t.op);
        const int n = K.nr;
        // Q = K^H K (sparse Gram product in liouvillian.jl:1318-1333)
        for (int a = 0; a < n; ++a) {
          for (int c = std::max(0, a - 2); c <= std::min(n - 1, a + 2); ++c) {
            cd v(0, 0);
            for (int r = std::max(0, std::min(a, c) - 1); r <= std::min(n - 1, std::max(a, c) + 1); ++r)
              v += std::conj(K.get(r, a)) * K.get(r, c);
            if (v != cd(0, 0)) Q[s].add(a, c, t.rate * v);
          }
        }
        g.K.push_back(std::move(K));
      }
      cgains.push_back(std::move(g));
    } else if (t.kind == TERM_LOCAL_JUMP) {
      cd LL[2][2];
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
          LL[i][j] = cd(0, 0);
          for (int r = 0; r < 2; ++r) LL[i][j] += std::conj(t.op[r][i]) * t.op[r][j];
        }
      for (int s = 0; s < S; ++s) {
        Band b = collective_band(s, LL);
        for (int p = -2; p <= 2; ++p)
          for (int a = 0; a < b.nr; ++a) Q[s].diag[p + 2][a] += t.rate * b.diag[p + 2][a];
      }
      local_jumps.push_back(&t);
    } else {
      throw std::invalid_argument("unsupported term kind for the CUDA backend");
    }
  }

  // Stencil terms per output sector.
  for (int s = 0; s < S; ++s) {
    Sector& sec = plan.sectors[s];
    const int n = sec.n;
    // A = -iH - Q/2 acts from the left, B = iH - Q/2 from the right.
    {
      StencilTerm add;
      add.src = s;
      add.kind = ST_ADD;
      add.alpha.resize(n);
      add.beta.resize(n);
      for (int a = 0; a < n; ++a) {
        cd h = H[s].diag[2][a], qd = Q[s].diag[2][a];
        add.alpha[a] = cd(0, -1) * h - 0.5 * qd;
        add.beta[a] = cd(0, 1) * h - 0.5 * qd;
      }
      std::vector<cd> both(add.alpha);
      both.insert(both.end(), add.beta.begin(), add.beta.end());
      add.cls = classify(both);
      bool nonzero = false;
      for (const auto& z : both) nonzero |= (z != cd(0, 0));
      if (nonzero) sec.terms.push_back(std::move(add));
    }
    for (int p = -2; p <= 2; ++p) {
      if (p == 0) continue;
      if (!H[s].has(p) && !Q[s].has(p)) continue;
      StencilTerm left;
      left.src = s;
      left.kind = ST_LEFT;
      left.p = p;
      left.alpha.resize(n);
      for (int a = 0; a < n; ++a) left.alpha[a] = cd(0, -1) * H[s].get(a, a + p) - 0.5 * Q[s].get(a, a + p);
      left.cls = classify(left.alpha);
      sec.terms.push_back(std::move(left));
      StencilTerm right;
      right.src = s;
      right.kind = ST_RIGHT;
      right.q = p;
      right.beta.resize(n);
      for (int b = 0; b < n; ++b) right.beta[b] = cd(0, 1) * H[s].get(b + p, b) - 0.5 * Q[s].get(b + p, b);
      right.cls = classify(right.beta);
      sec.terms.push_back(std::move(right));
    }
    auto add_sandwich = [&](int src, const Band& M, double scale) {
      for (int p = -2; p <= 2; ++p) {
        if (!M.has(p)) continue;
        for (int q = -2; q <= 2; ++q) {
          if (!M.has(q)) continue;
          StencilTerm t;
          t.src = src;
          t.kind = ST_SAND;
          t.e = M.e;
          t.p = p;
          t.q = q;
          t.alpha.resize(n);
          t.beta.resize(n);
          for (int a = 0; a < n; ++a) t.alpha[a] = scale * M.diag[p + 2][a];
          for (int b = 0; b < n; ++b) t.beta[b] = std::conj(M.diag[q + 2][b]);
          int ca = classify(t.alpha), cb = classify(t.beta);
          t.cls = (ca == CC_REAL && cb == CC_REAL) ? CC_REAL : CC_CPLX;
          sec.terms.push_back(std::move(t));
        }
      }
    };
    for (const auto& g : cgains) add_sandwich(s, g.K[s], g.rate);
    // One-body gains: branches (lambda = s, mu, nu) with a common child
    // (liouvillian.jl:316-326, 2370-2383, 2486-2537).
    for (const TermSpec* lj : local_jumps) {
      for (int ni = 0; ni < S; ++ni) {
        for (size_t cs = 0; cs < kids[s].size(); ++cs) {
          const Child& mu = kids[s][cs];
          int cn = child_index(ni, mu.mu1, mu.mu2);
          if (cn < 0) continue;
          const Sector& nu = plan.sectors[ni];
          Band C(n, nu.n, (nu.n - n) / 2);
          for (const auto& cell : pack_cells(trans[s][cs], trans[ni][cn])) {
            cd v = contract(cell, lj->op);
            if (v != cd(0, 0)) C.add(cell.a, cell.c, v);
          }
          Rational wl = branch_weight(N - sec.k, sec.k, mu.row);
          Rational wn = branch_weight(N - nu.k, nu.k, kids[ni][cn].row);
          double bscale = sqrt_ratio(mul(wl, wn));
          add_sandwich(ni, C, lj->rate * bscale);
        }
      }
    }
    plan.max_terms = std::max(plan.max_terms, (int)sec.terms.size());
  }
  return plan;
}

}  // namespace picuda
