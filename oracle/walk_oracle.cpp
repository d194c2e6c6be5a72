// walk_oracle.cpp -- CPU restatement of DistGER's information-oriented random walk
// (InCoM: include/walk.hpp:260-387 for the entropy/length correlation, :818-1042 for the
// walker loop, R = 0.999 at :24, minLength = 20 at :404) and of the per-edge
// common-neighbour counts that walker reads (candidate->data, walk.hpp:920, loaded from a
// file by graph.hpp:826 in the reference).
//
// TEST INFRASTRUCTURE ONLY: the checker of the CUDA walk generator (dsgl_walk.cu).  Only
// tests/, __graft_entry__.smoke() and bench.py's CPU legs load it; the product library
// never links or calls it.
//
// The reference draws from std::mt19937 seeded by std::random_device and from rand(), so
// no run of it can be reproduced.  This restatement keeps its rule and replaces the random
// source by a counter-based stream, which the GPU kernel draws identically:
//   walker w's k-th draw  r_k = mix64(base_w + k * G),  base_w = mix64(seed ^ (w * G)),
//   G = 0x9E3779B97F4A7C15 (a SplitMix64 stream per walker; mix64 is the SplitMix64
//   finaliser of Steele, Lea and Flood 2014, which adds G before mixing);
//   a neighbour index  (r_k >> 32) * deg >> 32   (Lemire's multiply-shift),
//   a uniform double   (r_k >> 11) * 2^-53.
// Walker w in [0, walker_num) starts at vertex w % V (walk.hpp:503-506, the -w option of
// huge_walk); the corpus lists the walks in walker order, -1 after each (path.hpp:96,110).
//
// One move from the current vertex c of degree ds (walk.hpp:889-1036):
//   * ds == 0: the walk ends;
//   * candidate u = adj[c][index(draw)];
//   * ds == 2 and adj[c][0] == c: the walk ends;
//   * no move made yet and u == c: draw again (the reference redraws without limit and
//     spins forever on a vertex whose only neighbour is itself; here the walk ends after
//     64 redraws in a row);
//   * p = uniform(draw); pa = ((1 / (ds - cn)) * max(ds, du)) / min(ds, du) with cn the
//     edge's common-neighbour count; trace = tanh(pa) <= p;
//   * append u (stop test), then, on a trace, append c again (stop test); the walk moves
//     to u only without a trace.  With trace steps off (trace = 0) there is no p draw and
//     every move goes on to u.
// Each appended vertex updates the correlation state with f = the vertex's earlier visits
// in this walk (Correlation::iterate, step 1), and the walk stops once it has made more
// than min_length moves and R * R < r_threshold or R < 0 (walk.hpp:868-874), or once it
// holds max_length vertices (the cap the reference has not; the trainer reads at most
// 1000 tokens per walk, dsgl.hpp:23).
//
// Arithmetic (identical on the GPU; IEEE double, no contraction):
//   * entropy update H' = (S * H - t) / (S + 1) with
//     t = ((xl[S] - xl[S+1]) + xl[f+1]) - xl[f], xl[x] = x * log2(x) from a table, which is
//     the reference's log2((S/(S+1))^S (1/(S+1)) ((f+1)/f)^f (f+1)) (iterateHn, with the
//     f = 0 case) written without pow;
//   * log2 of an integer x = e + ln(m) * log2(e) for x = 2^e m, m in [1, 2), ln(m) =
//     2 atanh(s), s = (m - 1) / (m + 1), by its odd series to s^39;
//   * tanh(x) = (E - 1) / (E + 1), E = exp(2x) = 2^k exp(r) (Cody-Waite reduction with
//     ln 2 split into a 24-bit head and its remainder, exp(r) by Taylor's series to r^13 in
//     Horner form); tanh(x) = 1 for x >= 20 (and for an infinite pa);
//   * moments E' = E + (X - E) / N', R = (EHS - EH ES) / sqrt((EHH - EH^2)(ESS - ES^2)),
//     R = 0 when the numerator is 0.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ULL;
constexpr int kMaxRedraws = 64;

inline uint64_t mix64(uint64_t z) {
  z += kGolden;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

inline double pow2i(int k) {  // 2^k for |k| < 1023, exact
  uint64_t b = (uint64_t)(1023 + k) << 52;
  double d;
  std::memcpy(&d, &b, 8);
  return d;
}

// log2 of an integer x >= 1 (see the header)
double log2_int(int64_t x) {
  int e = 0;
  while ((x >> (e + 1)) != 0) e++;
  const double m = (double)x / pow2i(e);  // exact, in [1, 2)
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double sum = 0.0;
  for (int k = 39; k >= 1; k -= 2) sum = sum * s2 + 1.0 / (double)k;
  const double ln_m = 2.0 * (s * sum);
  return (double)e + ln_m * 1.4426950408889634;
}

double tanh_pos(double x) {  // x >= 0 or +inf (see the header)
  if (!(x < 20.0)) return 1.0;
  const double y = 2.0 * x;
  const double ln2_hi = (double)(float)0.6931471805599453;
  const double ln2_lo = 0.6931471805599453 - ln2_hi;
  const int k = (int)(y * 1.4426950408889634 + 0.5);
  const double r = (y - (double)k * ln2_hi) - (double)k * ln2_lo;
  static const double inv_fact[14] = {1.0,
                                      1.0,
                                      1.0 / 2.0,
                                      1.0 / 6.0,
                                      1.0 / 24.0,
                                      1.0 / 120.0,
                                      1.0 / 720.0,
                                      1.0 / 5040.0,
                                      1.0 / 40320.0,
                                      1.0 / 362880.0,
                                      1.0 / 3628800.0,
                                      1.0 / 39916800.0,
                                      1.0 / 479001600.0,
                                      1.0 / 6227020800.0};
  double p = inv_fact[13];
  for (int i = 12; i >= 0; i--) p = p * r + inv_fact[i];
  const double E = p * pow2i(k);
  return (E - 1.0) / (E + 1.0);
}

struct Corr {
  double H, S, EH, ES, EHS, EHH, ESS, N, R;
};

inline void corr_start(Corr& c) {  // walk.hpp:849-853
  c.H = 0.0;
  c.S = 1.0;
  c.EH = 0.0;
  c.ES = 1.0;
  c.EHS = 0.0;
  c.EHH = 0.0;
  c.ESS = 1.0;
  c.R = 1.0;
  c.N = 1.0;
}

// Correlation::iterate (walk.hpp:330-365) with step 1; S is the walk's vertex count
inline void corr_iterate(Corr& c, const double* xl, int S, int f) {
  const double t = ((xl[S] - xl[S + 1]) + xl[f + 1]) - xl[f];
  const double S1 = (double)(S + 1);
  const double H1 = ((double)S * c.H - t) / S1;
  const double N1 = c.N + 1.0;
  c.EH = c.EH + (H1 - c.EH) / N1;
  c.ES = c.ES + (S1 - c.ES) / N1;
  c.EHS = c.EHS + (H1 * S1 - c.EHS) / N1;
  c.EHH = c.EHH + (H1 * H1 - c.EHH) / N1;
  c.ESS = c.ESS + (S1 * S1 - c.ESS) / N1;
  const double DH = c.EHH - c.EH * c.EH;
  const double DS = c.ESS - c.ES * c.ES;
  const double ex = c.EHS - c.EH * c.ES;
  c.R = ex == 0.0 ? 0.0 : ex / std::sqrt(DH * DS);
  c.H = H1;
  c.S = S1;
  c.N = N1;
}

struct WalkParams {
  const int64_t* indptr;
  const int32_t* indices;
  const int32_t* cn;
  int64_t V;
  int32_t min_length, max_length;
  double r_threshold;
  uint64_t seed;
  const double* xl;
  int32_t trace;  // 1: the trace step; 0: moves only (no p draw)
};

// One walk; writes its vertices to out (capacity max_length) and returns the count.
int walk_one(const WalkParams& P, int64_t w, int32_t* out) {
  const int64_t start = w % P.V;
  uint64_t ctr = mix64(P.seed ^ ((uint64_t)w * kGolden));
  auto draw = [&]() {
    const uint64_t r = mix64(ctr);
    ctr += kGolden;
    return r;
  };
  int len = 0;
  auto count_of = [&](int32_t v) {
    int f = 0;
    for (int i = 0; i < len; i++) f += out[i] == v;
    return f;
  };
  out[len++] = (int32_t)start;
  Corr c;
  corr_start(c);
  if (len >= P.max_length) return len;
  int steps = 0, redraws = 0;
  int64_t cur = start;
  auto append = [&](int32_t v) -> bool {  // true: the walk stops here
    const int f = count_of(v);
    corr_iterate(c, P.xl, len, f);
    out[len++] = v;
    steps++;
    if (steps > P.min_length && (c.R * c.R < P.r_threshold || c.R < 0.0)) return true;
    return len >= P.max_length;
  };
  while (true) {
    const int64_t b = P.indptr[cur];
    const int64_t ds = P.indptr[cur + 1] - b;
    if (ds == 0) break;
    const uint64_t r = draw();
    const int64_t e = b + (int64_t)(((r >> 32) * (uint64_t)ds) >> 32);
    const int32_t u = P.indices[e];
    if (ds == 2 && P.indices[b] == cur) break;
    if (steps == 0 && u == cur) {
      if (++redraws >= kMaxRedraws) break;
      continue;
    }
    bool trace = false;
    if (P.trace) {
      const double p = (double)(draw() >> 11) * (1.0 / 9007199254740992.0);
      const int64_t du = P.indptr[(int64_t)u + 1] - P.indptr[u];
      const int64_t mx = ds > du ? ds : du, mn = ds < du ? ds : du;
      const double pa = ((1.0 / (double)(ds - P.cn[e])) * (double)mx) / (double)mn;
      trace = tanh_pos(pa) <= p;
    }
    if (append(u)) break;
    if (trace) {
      if (append((int32_t)cur)) break;
    } else {
      cur = u;
    }
  }
  return len;
}

}  // namespace

extern "C" {

// x * log2(x) for x = 0..n-1 (the entropy table of the walker)
void oracle_xlog2x_table(int32_t n, double* t) {
  for (int32_t x = 0; x < n; x++) t[x] = x == 0 ? 0.0 : (double)x * log2_int(x);
}

double oracle_tanh_pos(double x) { return tanh_pos(x); }

// cn[e] = |N(u) & N(v)| for the CSR edge e = (u, v); adjacency lists strictly increasing.
void oracle_edge_common_neighbors(const int64_t* indptr, const int32_t* indices, int64_t V, int32_t* cn) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t u = 0; u < V; u++) {
    for (int64_t e = indptr[u]; e < indptr[u + 1]; e++) {
      const int64_t v = indices[e];
      int64_t i = indptr[u], j = indptr[v], c = 0;
      while (i < indptr[u + 1] && j < indptr[v + 1]) {
        if (indices[i] < indices[j]) i++;
        else if (indices[i] > indices[j]) j++;
        else {
          c++;
          i++;
          j++;
        }
      }
      cn[e] = (int32_t)c;
    }
  }
}

// Information-oriented walks (see the header).  corpus: capacity cap; *n_tokens = entries
// the walks yield (also when cap is too small: then nothing is written and 1 returned).
int32_t oracle_info_walks(const int64_t* indptr, const int32_t* indices, const int32_t* cn, int64_t V,
                          int64_t walker_num, int32_t min_length, int32_t max_length, double r_threshold,
                          uint64_t seed, int32_t trace, int32_t* corpus, int64_t cap, int64_t* n_tokens,
                          int32_t* lengths) {
  std::vector<double> xl((size_t)max_length + 2);
  oracle_xlog2x_table(max_length + 2, xl.data());
  WalkParams P{indptr, indices, cn, V, min_length, max_length, r_threshold, seed, xl.data(), trace};
  const int64_t n = walker_num;
  std::vector<int32_t> len((size_t)n);
#pragma omp parallel
  {
    std::vector<int32_t> buf((size_t)max_length);
#pragma omp for schedule(dynamic, 1024)
    for (int64_t w = 0; w < n; w++) len[w] = walk_one(P, w, buf.data());
  }
  std::vector<int64_t> off((size_t)n + 1, 0);
  for (int64_t w = 0; w < n; w++) off[w + 1] = off[w] + len[w] + 1;
  *n_tokens = off[n];
  if (lengths)
    for (int64_t w = 0; w < n; w++) lengths[w] = len[w];
  if (off[n] > cap || !corpus) return 1;
#pragma omp parallel
  {
    std::vector<int32_t> buf((size_t)max_length);
#pragma omp for schedule(dynamic, 1024)
    for (int64_t w = 0; w < n; w++) {
      const int L = walk_one(P, w, buf.data());
      std::memcpy(corpus + off[w], buf.data(), sizeof(int32_t) * L);
      corpus[off[w] + L] = -1;
    }
  }
  return 0;
}

}  // extern "C"
