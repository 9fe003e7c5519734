// Synthetic sparse logistic-regression data (host, multi-threaded).
//
// Every row is generated from its own counter-based random stream
// (SplitMix64 keyed by seed, row and a stream id), so any row range can be
// produced independently and the output does not depend on the thread count.
// Distributions are sampled by inverse-CDF tables built once per call.
//
//   row length : 1 + Poisson(lam)                      (len_kind 0)
//                Zipf(s) on [1, cap], rescaled so the
//                matrix has exactly total_nnz entries  (len_kind 1)
//   columns    : distinct per row, sorted; Zipf(s) over [0, n) (col_kind 0)
//                or uniform (col_kind 1)
//   values     : |N(0,1)| (0), N(0,1) (1), lognormal(0, sigma) (2)
//   labels     : ±1 ~ Bernoulli(sigmoid(x·w*)), w*_c ~ N(0, wstar_sd^2)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

extern "C" {
typedef struct {
  int64_t m, n;
  uint64_t seed;
  int32_t len_kind;
  double lam;
  double s_len;
  int64_t len_cap;
  int64_t total_nnz;
  int32_t col_kind;
  double s_col;
  int32_t val_kind;
  double val_sigma;
  double wstar_sd;
  int32_t nthreads;
} syn_cfg;
}

namespace {

inline uint64_t mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Rng {
  uint64_t s;
  Rng(uint64_t seed, uint64_t row, uint64_t stream) : s(mix(seed ^ mix(row * 0x100000001B3ull + stream))) {}
  uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  double normal() {
    double u1 = uniform(), u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

// inverse-CDF table over values offset..offset+K-1 with weights w(k)
struct Table {
  std::vector<double> cdf;
  int64_t offset = 0;
  int64_t sample(double u) const {
    auto it = std::upper_bound(cdf.begin(), cdf.end(), u * cdf.back());
    int64_t k = it - cdf.begin();
    if (k >= (int64_t)cdf.size()) k = (int64_t)cdf.size() - 1;
    return offset + k;
  }
};

Table zipf_table(int64_t K, double s, int64_t offset) {
  Table t;
  t.offset = offset;
  t.cdf.resize(K);
  double acc = 0;
  for (int64_t k = 0; k < K; k++) {
    acc += std::pow((double)(k + 1), -s);
    t.cdf[k] = acc;
  }
  return t;
}

Table poisson_table(double lam) {
  Table t;
  t.offset = 0;
  double p = std::exp(-lam), acc = 0;
  int64_t kmax = (int64_t)(lam + 20 * std::sqrt(lam) + 50);
  for (int64_t k = 0; k <= kmax; k++) {
    acc += p;
    t.cdf.push_back(acc);
    p *= lam / (double)(k + 1);
  }
  return t;
}

template <class F> void parallel_rows(int64_t m, int nt, F fn) {
  if (nt <= 1 || m < 4096) {
    fn(0, m);
    return;
  }
  std::vector<std::thread> th;
  int64_t per = (m + nt - 1) / nt;
  for (int t = 0; t < nt; t++) {
    int64_t a = t * per, b = std::min(m, a + per);
    if (a >= b) break;
    th.emplace_back([=]() { fn(a, b); });
  }
  for (auto& x : th) x.join();
}

int nthreads(const syn_cfg* c) {
  int nt = c->nthreads;
  if (nt <= 0) nt = (int)std::thread::hardware_concurrency();
  return std::max(1, nt);
}

}  // namespace

extern "C" {

// Row lengths of all rows; returns nnz (or -1 on bad config).
int64_t syn_lengths(const syn_cfg* c, int32_t* lens) {
  const int64_t m = c->m, n = c->n;
  if (m < 0 || n <= 0) return -1;
  const int nt = nthreads(c);
  if (c->len_kind == 0) {
    Table pt = poisson_table(c->lam);
    parallel_rows(m, nt, [&](int64_t a, int64_t b) {
      for (int64_t r = a; r < b; r++) {
        Rng g(c->seed, (uint64_t)r, 1);
        int64_t l = 1 + pt.sample(g.uniform());
        if (l > n) l = n;
        if (c->len_cap > 0 && l > c->len_cap) l = c->len_cap;
        lens[r] = (int32_t)l;
      }
    });
  } else {
    const int64_t cap = std::min<int64_t>(c->len_cap > 0 ? c->len_cap : n, n);
    Table zt = zipf_table(cap, c->s_len, 1);
    std::vector<double> raw(m);
    parallel_rows(m, nt, [&](int64_t a, int64_t b) {
      for (int64_t r = a; r < b; r++) {
        Rng g(c->seed, (uint64_t)r, 1);
        raw[r] = (double)zt.sample(g.uniform());
      }
    });
    double tot = 0;
    for (double v : raw) tot += v;
    const double f = (double)c->total_nnz / tot;
    int64_t sum = 0;
    for (int64_t r = 0; r < m; r++) {  // stochastic rounding of the rescaled length
      Rng g(c->seed, (uint64_t)r, 2);
      double x = raw[r] * f;
      int64_t l = (int64_t)std::floor(x + g.uniform());
      l = std::min(l, cap);
      lens[r] = (int32_t)l;
      sum += l;
    }
    // fix the total exactly: walk rows adding / removing one entry
    int64_t r = 0, guard = 0;
    while (sum != c->total_nnz && guard < 64 * m + 64) {
      if (sum < c->total_nnz && lens[r] < cap) { lens[r]++; sum++; }
      else if (sum > c->total_nnz && lens[r] > 0) { lens[r]--; sum--; }
      r = (r + 7919) % m;
      guard++;
    }
  }
  int64_t z = 0;
  for (int64_t r = 0; r < m; r++) z += lens[r];
  return z;
}

// Fills off[m+1], idx[nnz], val[nnz] (FP64) and label[m] (±1, may be NULL)
// for the lengths produced by syn_lengths.
int syn_fill(const syn_cfg* c, const int32_t* lens, int32_t* off, int32_t* idx, double* val, double* label) {
  const int64_t m = c->m, n = c->n;
  const int nt = nthreads(c);
  int64_t acc = 0;
  off[0] = 0;
  for (int64_t r = 0; r < m; r++) {
    acc += lens[r];
    if (acc > 2147483647ll) return -1;
    off[r + 1] = (int32_t)acc;
  }
  Table zc;
  if (c->col_kind == 0) zc = zipf_table(n, c->s_col, 0);
  std::vector<double> wstar;
  if (label) {
    wstar.resize(n);
    parallel_rows(n, nt, [&](int64_t a, int64_t b) {
      for (int64_t k = a; k < b; k++) {
        Rng g(c->seed, (uint64_t)k, 7);
        wstar[k] = c->wstar_sd * g.normal();
      }
    });
  }
  parallel_rows(m, nt, [&](int64_t a, int64_t b) {
    std::vector<int64_t> cols;
    std::vector<std::pair<double, int64_t>> keyed;
    for (int64_t r = a; r < b; r++) {
      const int64_t l = lens[r], base = off[r];
      Rng g(c->seed, (uint64_t)r, 3);
      cols.clear();
      if (l > 0 && 4 * l > n) {
        // dense-ish row: weighted sampling without replacement by keys u^(1/w)
        keyed.clear();
        for (int64_t k = 0; k < n; k++) {
          double w = (c->col_kind == 0) ? std::pow((double)(k + 1), -c->s_col) : 1.0;
          double u = g.uniform();
          if (u < 1e-300) u = 1e-300;
          keyed.push_back({std::log(u) / w, k});
        }
        std::partial_sort(keyed.begin(), keyed.begin() + l, keyed.end(),
                          [](const std::pair<double, int64_t>& x, const std::pair<double, int64_t>& y) {
                            return x.first > y.first;
                          });
        for (int64_t q = 0; q < l; q++) cols.push_back(keyed[q].second);
      } else {
        // draw the missing count, then sort + dedupe, until l distinct columns
        while ((int64_t)cols.size() < l) {
          int64_t need = l - (int64_t)cols.size();
          for (int64_t q = 0; q < need; q++) {
            int64_t cnd = (c->col_kind == 0) ? zc.sample(g.uniform()) : (int64_t)(g.uniform() * (double)n);
            cols.push_back(cnd >= n ? n - 1 : cnd);
          }
          std::sort(cols.begin(), cols.end());
          cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        }
      }
      std::sort(cols.begin(), cols.end());
      Rng gv(c->seed, (uint64_t)r, 4);
      double dotw = 0;
      for (int64_t q = 0; q < l; q++) {
        double v;
        if (c->val_kind == 0) v = std::fabs(gv.normal());
        else if (c->val_kind == 1) v = gv.normal();
        else v = std::exp(c->val_sigma * gv.normal());
        idx[base + q] = (int32_t)cols[q];
        val[base + q] = v;
        if (label) dotw += v * wstar[cols[q]];
      }
      if (label) {
        Rng gl(c->seed, (uint64_t)r, 5);
        double p = 1.0 / (1.0 + std::exp(-dotw));
        label[r] = (gl.uniform() < p) ? 1.0 : -1.0;
      }
    }
  });
  return 0;
}

}  // extern "C"
