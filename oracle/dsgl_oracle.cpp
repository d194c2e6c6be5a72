// dsgl_oracle.cpp -- CPU restatement of DistGER's DSGL skip-gram negative-sampling
// trainer (include/dsgl.hpp in trsenli/GDistGER-re).
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA trainer: only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  Nothing
// in the product library links or calls it.
//
// Parity is pinned against the reference itself: oracle/build_ref.sh compiles the
// unmodified include/dsgl.hpp (header shims for MPI/MKL only) and
// tests/golden/make_golden.py records its output; tests/test_oracle_golden.py checks
// this restatement bit for bit against those vectors.
//
// Arithmetic contract (shared with the CUDA kernels):
//   * the three small GEMMs of a step use the sequential-k order of the reference's
//     plain loops (dsgl.hpp:1226-1229, 1282-1285, 1301-1304), each multiply-add
//     fused (fmaf) -- the contract of the reference's MKL build (-mavx512f);
//   * every other float expression is evaluated exactly as written in dsgl.hpp
//     (compile with -ffp-contract=off so no other contraction happens).
//
// Two memory policies are restated:
//   POLICY_REF    -- the reference's per-walk input buffers (snapshot at walk load,
//                    overwrite at walk end, dsgl.hpp:940-962, 1377-1398) and the
//                    per-pool negative buffer (snapshot at pool build, overwrite after
//                    two walk completions, dsgl.hpp:1054-1088, 1399-1407).
//   POLICY_WINDOW -- the GPU-resident policy of the fast engine: a walk's context
//                    rows are held on chip while any of their positions lies in the
//                    sliding window [pos-w, pos+w] (one copy per walk, exactly as the
//                    reference dedupes them) and written back when they leave it;
//                    negative rows are read from and added to Woh at each step; each
//                    forward dot product is eight sequential partial sums (even and odd
//                    k of each quarter of [0, d)) combined pairwise.
// Storage: FP32, BF16 with stochastic rounding on every write-back, or FP64.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

constexpr int kMaxExp = 6;                 // dsgl.hpp:22
constexpr int kExpTableSize = 1000;        // dsgl.hpp:21
constexpr int kMaxSentence = 1000;         // dsgl.hpp:23
constexpr int kTableScale = kExpTableSize / kMaxExp / 2;  // integer 83 (dsgl.hpp:1257)

enum { POLICY_REF = 0, POLICY_WINDOW = 1 };
enum { STORE_F32 = 0, STORE_BF16 = 1, STORE_F64 = 2 };
// write-event kinds for the stochastic-rounding stream
enum { EV_TARGET1 = 0, EV_TARGET2 = 1, EV_WALK0 = 2, EV_WALK1 = 3, EV_NEG = 4, EV_POOL = 5 };

inline uint64_t lcg_next(uint64_t r) { return r * 25214903917ULL + 11ULL; }

// SplitMix64 finaliser (Steele, Lea, Flood 2014) -- the stochastic-rounding hash.
inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
inline uint64_t sr_event_key(uint64_t seed, int kind, uint32_t worker, uint64_t step) {
  return mix64(seed ^ ((uint64_t)kind << 56) ^ ((uint64_t)worker << 34) ^ step);
}
// 16 random bits for one column: columns 4q, 4q+1 take the low and high halves of
// h = fmix32(lo32(ev) ^ (row * 0x9E3779B1 + q * 0x85EBCA77)) (murmur3's 32-bit finaliser
// with Wellons' low-bias constants), columns 4q+2, 4q+3 those of h2 = t ^ (t >> 16),
// t = (h ^ hi32(ev)) * 0x9E3779B1 mod 2^32
inline uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  return h ^ (h >> 16);
}
inline uint32_t sr_bits16(uint64_t ev, uint32_t row, int col) {
  const uint32_t q = (uint32_t)(col >> 2);
  const uint32_t h = fmix32((uint32_t)ev ^ (row * 0x9E3779B1u + q * 0x85EBCA77u));
  const uint32_t t = (h ^ (uint32_t)(ev >> 32)) * 0x9E3779B1u;
  const uint64_t bits = ((uint64_t)(t ^ (t >> 16)) << 32) | h;
  return (uint32_t)(bits >> ((col & 3) * 16)) & 0xFFFFu;
}
inline float bf16_to_f32(uint16_t b) {
  uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
// Stochastic rounding to bfloat16: add 16 uniform bits below the kept mantissa, truncate
// (infinities stay infinite, finite values near the top may round up to infinity); NaN
// becomes the canonical 0x7FFF, as the GPU's stochastic-rounding conversion does.
inline uint16_t f32_to_bf16_sr(float x, uint32_t r16) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7FFFFFFFu) > 0x7F800000u) return 0x7FFFu;
  return (uint16_t)((u + r16) >> 16);
}

// ---- storage traits -------------------------------------------------------------
template <int S> struct Store;
template <> struct Store<STORE_F32> {
  typedef float T;
  typedef float A;
  static A load(const T* p) { return *p; }
  static void store(T* p, A v, uint64_t, uint32_t, int) { *p = v; }
};
template <> struct Store<STORE_BF16> {
  typedef uint16_t T;
  typedef float A;
  static A load(const T* p) { return bf16_to_f32(*p); }
  static void store(T* p, A v, uint64_t ev, uint32_t row, int col) {
    *p = f32_to_bf16_sr(v, sr_bits16(ev, row, col));
  }
};
template <> struct Store<STORE_F64> {
  typedef double T;
  typedef double A;
  static A load(const T* p) { return *p; }
  static void store(T* p, A v, uint64_t, uint32_t, int) { *p = v; }
};

inline float fma_acc(float a, float b, float c) { return fmaf(a, b, c); }
inline double fma_acc(double a, double b, double c) { return fma(a, b, c); }

// ---- vocabulary / tables (dsgl.hpp:121-147, 246-252, 314-382, 433-457, 1557-1562) --
struct VocabVertex {
  int cn;
  uint32_t id;
};

void build_vocab(const int32_t* counts, int64_t V, uint32_t* order, int32_t* row_of,
                 int32_t* cn_sorted, uint64_t* train_words) {
  std::vector<VocabVertex> v(V);
  uint64_t tw = 0;
  for (int64_t i = 0; i < V; i++) {
    v[i].cn = counts[i];
    v[i].id = (uint32_t)i;
    tw += counts[i];
  }
  // dsgl.hpp:249-250: std::sort (unstable) on count, descending.
  std::sort(v.begin(), v.end(), [](VocabVertex a, VocabVertex b) { return a.cn > b.cn; });
  for (int64_t r = 0; r < V; r++) {
    order[r] = v[r].id;
    row_of[v[r].id] = (int32_t)r;
    cn_sorted[r] = v[r].cn;
  }
  *train_words = tw;
}

// dsgl.hpp:121-147.  train_words_pow is an OpenMP `reduction(+)` over a static
// schedule with `threads` threads: contiguous per-thread partial sums, combined here
// in thread order (for <= 2 threads this is the only possible result).
void build_unigram_table(const int32_t* cn_sorted, int64_t V, int64_t table_size, int threads,
                         int32_t* table) {
  const float power = 0.75f;
  if (threads < 1) threads = 1;
  double twp = 0.;
  const int64_t q = V / threads, rem = V % threads;
  for (int t = 0; t < threads; t++) {
    int64_t lo = t * q + std::min<int64_t>(t, rem);
    int64_t hi = lo + q + (t < rem ? 1 : 0);
    double p = 0.;
    for (int64_t i = lo; i < hi; i++) p += std::pow((double)cn_sorted[i], (double)power);
    twp += p;
  }
  int64_t i = 0;
  float d1 = (float)(std::pow((double)cn_sorted[i], (double)power) / twp);
  for (int64_t a = 0; a < table_size; a++) {
    table[a] = (int32_t)i;
    if ((float)(int)a / (float)table_size > d1) {
      i++;
      if (i >= V) i = V - 1;
      d1 = (float)((double)d1 + std::pow((double)cn_sorted[i], (double)power) / twp);
    }
  }
}

void build_exp_table(float* t) {
  for (int i = 0; i < kExpTableSize + 1; i++) {
    float e = expf(((float)i / (float)kExpTableSize * 2 - 1) * kMaxExp);
    t[i] = e / (e + 1);
  }
}

// Subsampling keep-threshold per sorted row (dsgl.hpp:923-924).  The reference
// indexes the vertex-indexed count array with the sorted row number; so does this.
void build_keep_threshold(const int32_t* counts, int64_t V, float sample, uint64_t train_words,
                          float* ran) {
  const float st = sample * (float)train_words;
  for (int64_t w = 0; w < V; w++) {
    float ratio = st / (float)counts[w];
    ran[w] = sqrtf(ratio) + ratio;
  }
}

// ---- the trainer -----------------------------------------------------------------
struct Shared {
  const int32_t* corpus;
  int64_t words_num;
  const int32_t* row_of;
  const float* ran;
  const int32_t* table;
  int64_t table_size;
  int64_t V;
  const float* exp_table;
  int d, window, negative, iter, workers, policy;
  int windows;  // 2: two walks per step (dsgl.hpp:1100-1132); 1: one walk, target 2 a
                // placeholder copy of target 1 with multiplicity 0, never written
  float sample, start_alpha;
  uint64_t train_words;
  uint64_t sr_seed;
  std::atomic<uint64_t> wca;
  std::atomic<float> alpha;
  std::atomic<uint64_t> steps, pairs;
};

template <int S>
struct Worker {
  typedef typename Store<S>::T T;
  typedef typename Store<S>::A A;
  typedef Store<S> ST;

  Shared& sh;
  T* Wih;
  T* Woh;
  const int d, window, K;
  const uint32_t wid;

  uint64_t rng, word_count = 0, last_word_count = 0, step_id = 0;
  int64_t start = 0, n_slice = 0, cur = 0;
  int local_iter;
  int len[2] = {0, 0}, pos[2] = {0, 0};
  std::vector<int32_t> sen[2];
  int train_sen_num = 0;
  bool change_neg = true;
  int neg_count = 0, neg_batch_num = 1;
  std::vector<int32_t> neg_words;

  // POLICY_REF walk buffers: unique vertices of the walk, their rows, position->slot
  std::vector<int32_t> uniq[2], slot_of_pos[2];
  std::vector<A> buf[2];
  // POLICY_REF negative pool
  std::vector<int32_t> neg_buffer;
  std::vector<A> negbuf;
  // POLICY_WINDOW resident rows: per walk, slots with (vertex, refcount, row)
  struct Resident {
    std::vector<int32_t> vert, ref;
    std::vector<A> rows;
    std::vector<int32_t> pos_slot;  // slot of each position while resident
  } res[2];

  // per-step scratch
  std::vector<int32_t> in_walk, in_slot, out_id, out_meta;
  std::vector<A> inputM, outputM, outputMd, corrM;

  Worker(Shared& s, T* wih, T* woh, uint32_t id)
      : sh(s), Wih(wih), Woh(woh), d(s.d), window(s.window), K(s.negative), wid(id) {
    rng = id;  // dsgl.hpp:791 with one process: thread id - 1
    local_iter = s.iter;
    // dsgl.hpp:811-826 corpus slice
    uint64_t words_num = (uint64_t)s.words_num;
    uint64_t parts = (uint64_t)s.workers;
    uint64_t tw = words_num / parts;
    start = (int64_t)(tw * id);
    if (words_num % parts > 0 && id == parts - 1) tw = words_num - (parts - 1) * tw;
    n_slice = (int64_t)tw;
    cur = start;
    sen[0].resize(kMaxSentence);
    sen[1].resize(kMaxSentence);
    int imax = 2 * (2 * window + 1);
    in_walk.resize(imax);
    in_slot.resize(imax);
    out_id.resize(K + 2);
    out_meta.resize(K + 2);
    inputM.resize((size_t)imax * d);
    outputM.resize((size_t)(K + 2) * d);
    outputMd.resize((size_t)(K + 2) * d);
    corrM.resize((size_t)(K + 2) * imax);
  }

  bool slice_done() const { return cur >= start + n_slice || cur >= sh.words_num; }

  // dsgl.hpp:909-933
  void fill_walk(int w) {
    int L = 0;
    const int64_t end = start + n_slice;
    while (true) {
      int32_t origin = sh.corpus[cur];
      word_count++;
      cur++;
      if (origin == -1 || cur >= end) break;
      int32_t r = sh.row_of[origin];
      if (sh.sample > 0) {
        rng = lcg_next(rng);
        if (sh.ran[r] < (float)(rng & 0xFFFF) / 65536.f) continue;
      }
      sen[w][L++] = r;
      if (L >= kMaxSentence) break;
    }
    len[w] = L;
    pos[w] = 0;
  }

  void load_row(A* dst, const T* src) {
    for (int c = 0; c < d; c++) dst[c] = ST::load(src + c);
  }
  void store_row(T* dst, const A* src, uint64_t ev, int32_t row) {
    for (int c = 0; c < d; c++) ST::store(dst + c, src[c], ev, (uint32_t)row, c);
  }

  // ---- POLICY_REF walk buffer (dsgl.hpp:940-962) ----
  void ref_load_walk(int w) {
    uniq[w].clear();
    slot_of_pos[w].assign(len[w], 0);
    for (int i = 0; i < len[w]; i++) {
      int32_t v = sen[w][i];
      auto p = std::find(uniq[w].begin(), uniq[w].end(), v);
      if (p == uniq[w].end()) {
        slot_of_pos[w][i] = (int32_t)uniq[w].size();
        uniq[w].push_back(v);
      } else {
        slot_of_pos[w][i] = (int32_t)(p - uniq[w].begin());
      }
    }
    buf[w].resize(uniq[w].size() * (size_t)d);
    for (size_t s = 0; s < uniq[w].size(); s++)
      load_row(&buf[w][s * d], Wih + (size_t)uniq[w][s] * d);
  }
  void ref_flush_walk(int w) {  // dsgl.hpp:1380-1384, 1391-1395
    uint64_t ev = sr_event_key(sh.sr_seed, EV_WALK0 + w, wid, step_id);
    for (size_t s = 0; s < uniq[w].size(); s++)
      store_row(Wih + (size_t)uniq[w][s] * d, &buf[w][s * d], ev, uniq[w][s]);
  }

  // ---- POLICY_WINDOW resident rows ----
  void win_enter(int w, int p) {
    Resident& R = res[w];
    int32_t v = sen[w][p];
    int found = -1;
    for (size_t s = 0; s < R.vert.size(); s++)
      if (R.ref[s] > 0 && R.vert[s] == v) { found = (int)s; break; }
    if (found < 0) {
      for (size_t s = 0; s < R.vert.size(); s++)
        if (R.ref[s] == 0) { found = (int)s; break; }
      if (found < 0) {
        found = (int)R.vert.size();
        R.vert.push_back(0);
        R.ref.push_back(0);
        R.rows.resize(R.vert.size() * (size_t)d);
      }
      R.vert[found] = v;
      R.ref[found] = 0;
      load_row(&R.rows[(size_t)found * d], Wih + (size_t)v * d);
    }
    R.ref[found]++;
    R.pos_slot[p] = found;
  }
  void win_leave(int w, int p, uint64_t ev) {
    Resident& R = res[w];
    int s = R.pos_slot[p];
    if (--R.ref[s] == 0) store_row(Wih + (size_t)R.vert[s] * d, &R.rows[(size_t)s * d], ev, R.vert[s]);
  }
  void win_load_walk(int w) {
    Resident& R = res[w];
    R.vert.clear();
    R.ref.clear();
    R.rows.clear();
    R.pos_slot.assign(len[w], -1);
    int hi = std::min(len[w] - 1, window);
    for (int p = 0; p <= hi; p++) win_enter(w, p);
  }
  void win_flush_all(int w, uint64_t ev) {
    Resident& R = res[w];
    for (size_t s = 0; s < R.vert.size(); s++)
      if (R.ref[s] > 0) {
        store_row(Wih + (size_t)R.vert[s] * d, &R.rows[s * d], ev, R.vert[s]);
        R.ref[s] = 0;
      }
  }
  void win_drop(int w) {
    res[w].vert.clear();
    res[w].ref.clear();
  }

  void on_walk_loaded(int w) {
    if (sh.policy == POLICY_REF) ref_load_walk(w);
    else win_load_walk(w);
  }

  // dsgl.hpp:1054-1088
  void build_pool() {
    neg_words.clear();
    neg_buffer.clear();
    neg_batch_num = sh.windows == 2 ? std::max(len[0], len[1]) : len[0];
    for (int i = 0; i < neg_batch_num; i++) {
      for (int k = 0; k < K; k++) {
        rng = lcg_next(rng);
        int32_t s = sh.table[(rng >> 16) % (uint64_t)sh.table_size];
        if (!s) s = (int32_t)(rng % (uint64_t)(sh.V - 1) + 1);
        neg_words.push_back(s);
        if (sh.policy == POLICY_REF &&
            std::find(neg_buffer.begin(), neg_buffer.end(), s) == neg_buffer.end())
          neg_buffer.push_back(s);
      }
    }
    if (sh.policy == POLICY_REF) {
      negbuf.resize(neg_buffer.size() * (size_t)d);
      for (size_t p = 0; p < neg_buffer.size(); p++)
        load_row(&negbuf[p * d], Woh + (size_t)neg_buffer[p] * d);
    }
    change_neg = false;
  }

  A* input_row(int j) {
    int w = in_walk[j];
    if (sh.policy == POLICY_REF) return &buf[w][(size_t)in_slot[j] * d];
    return &res[w].rows[(size_t)in_slot[j] * d];
  }

  // dsgl.hpp:1089-1407
  void step() {
    const int w = window;
    const uint64_t ev_step = step_id;
    const bool two = sh.windows == 2;
    const int t1 = sen[0][pos[0]], t2 = two ? sen[1][pos[1]] : t1;
    rng = lcg_next(rng);
    const int b = (int)(rng % (uint64_t)w);
    int I = 0, first = 0;
    for (int walk = 0; walk < (two ? 2 : 1); walk++) {
      for (int i = b; i < 2 * w + 1 - b; i++) {
        if (i == w) continue;
        int c = pos[walk] - w + i;
        if (c < 0) continue;
        if (c >= len[walk]) break;
        in_walk[I] = walk;
        in_slot[I] = sh.policy == POLICY_REF ? slot_of_pos[walk][c] : res[walk].pos_slot[c];
        I++;
      }
      if (walk == 0) first = I;
    }
    neg_count++;
    const int start_g = neg_count % neg_batch_num;
    int off = 1;
    out_id[0] = t1;
    out_meta[0] = 1;
    for (int k = 0; k < K; k++) {
      int32_t s = neg_words[(size_t)start_g * K + k];
      int found = -1;
      for (int q = 0; q < off; q++)
        if (out_id[q] == s) { found = q; break; }
      if (found < 0) {
        out_id[off] = s;
        out_meta[off] = 1;
        off++;
      } else {
        out_meta[found]++;
      }
    }
    out_id[0] = t1;
    out_meta[0] = 1;
    out_id[off] = t2;
    out_meta[off] = two ? 1 : 0;
    const int O = off + 1;

    // gather (dsgl.hpp:1173-1211)
    for (int j = 0; j < I; j++) std::memcpy(&inputM[(size_t)j * d], input_row(j), sizeof(A) * d);
    load_row(&outputM[0], Woh + (size_t)t1 * d);
    load_row(&outputM[(size_t)(O - 1) * d], Woh + (size_t)t2 * d);
    std::vector<int> neg_slot(O, -1);
    for (int i = 1; i < O - 1; i++) {
      if (sh.policy == POLICY_REF) {
        int p = (int)(std::find(neg_buffer.begin(), neg_buffer.end(), out_id[i]) - neg_buffer.begin());
        neg_slot[i] = p;
        std::memcpy(&outputM[(size_t)i * d], &negbuf[(size_t)p * d], sizeof(A) * d);
      } else {
        load_row(&outputM[(size_t)i * d], Woh + (size_t)out_id[i] * d);
      }
    }

    // forward + gradient (dsgl.hpp:1241-1272, MKL branch labels)
    const A alpha = (A)sh.alpha.load(std::memory_order_relaxed);
    // The window policy's engine sums each dot product as eight sequential partial sums:
    // the even and the odd k of each quarter of [0, d), s_m = even_m + odd_m, combined as
    // (s0 + s1) + (s2 + s3); when d % 16 != 0, [0, d) is one range and f = even + odd.
    const bool window_order = sh.policy == POLICY_WINDOW;
    const int nq = d % 16 == 0 ? 4 : 1;
    for (int i = 0; i < O; i++) {
      const A c = (A)out_meta[i];
      for (int j = 0; j < I; j++) {
        A f = 0;
        const A* o = &outputM[(size_t)i * d];
        const A* x = &inputM[(size_t)j * d];
        if (window_order) {
          const int qd = d / nq;
          A s4[4] = {0, 0, 0, 0};
          for (int m = 0; m < nq; m++) {
            A ev = 0, od = 0;
            for (int k = m * qd; k < (m + 1) * qd; k += 2) {
              ev = fma_acc(o[k], x[k], ev);
              od = fma_acc(o[k + 1], x[k + 1], od);
            }
            s4[m] = ev + od;
          }
          f = nq == 4 ? (s4[0] + s4[1]) + (s4[2] + s4[3]) : s4[0];
        } else {
          for (int k = 0; k < d; k++) f = fma_acc(o[k], x[k], f);
        }
        int label = j < first ? (i == 0 ? 1 : 0) : (i == O - 1 ? 1 : 0);
        A g;
        if (f > kMaxExp) g = (A)(label - 1) * alpha;
        else if (f < -kMaxExp) g = (A)label * alpha;
        else g = ((A)label - (A)sh.exp_table[(int)((f + (A)kMaxExp) * (A)kTableScale)]) * alpha;
        corrM[(size_t)i * I + j] = g * c;
      }
    }
    // outputMd = corrM . inputM  (dsgl.hpp:1290-1291)
    for (int i = 0; i < O; i++)
      for (int c = 0; c < d; c++) {
        A f = 0;
        for (int j = 0; j < I; j++) f = fma_acc(corrM[(size_t)i * I + j], inputM[(size_t)j * d + c], f);
        outputMd[(size_t)i * d + c] = f;
      }
    // inputM = corrM^T . outputM  (dsgl.hpp:1309-1310)
    for (int j = 0; j < I; j++)
      for (int c = 0; c < d; c++) {
        A f = 0;
        for (int i = 0; i < O; i++) f = fma_acc(corrM[(size_t)i * I + j], outputM[(size_t)i * d + c], f);
        inputM[(size_t)j * d + c] = f;
      }
    // scatter (dsgl.hpp:1314-1368)
    for (int j = 0; j < I; j++) {
      A* dst = input_row(j);
      for (int c = 0; c < d; c++) dst[c] += inputM[(size_t)j * d + c];
    }
    {
      uint64_t e1 = sr_event_key(sh.sr_seed, EV_TARGET1, wid, ev_step);
      uint64_t e2 = sr_event_key(sh.sr_seed, EV_TARGET2, wid, ev_step);
      T* r1 = Woh + (size_t)t1 * d;
      T* r2 = Woh + (size_t)t2 * d;
      const A* m1 = &outputMd[0];
      const A* m2 = &outputMd[(size_t)(O - 1) * d];
      for (int c = 0; c < d; c++) {
        ST::store(r1 + c, ST::load(r1 + c) + m1[c], e1, (uint32_t)t1, c);
        if (two) ST::store(r2 + c, ST::load(r2 + c) + m2[c], e2, (uint32_t)t2, c);
      }
    }
    if (sh.policy == POLICY_REF) {
      for (int i = 1; i < O - 1; i++) {
        A* dst = &negbuf[(size_t)neg_slot[i] * d];
        for (int c = 0; c < d; c++) dst[c] += outputMd[(size_t)i * d + c];
      }
    } else {
      uint64_t en = sr_event_key(sh.sr_seed, EV_NEG, wid, ev_step);
      for (int i = 1; i < O - 1; i++) {
        T* r = Woh + (size_t)out_id[i] * d;
        for (int c = 0; c < d; c++)
          ST::store(r + c, ST::load(r + c) + outputMd[(size_t)i * d + c], en, (uint32_t)out_id[i], c);
      }
    }
    sh.pairs.fetch_add((uint64_t)I, std::memory_order_relaxed);
    sh.steps.fetch_add(1, std::memory_order_relaxed);

    // positions, flushes (dsgl.hpp:1372-1407)
    pos[0]++;
    pos[1]++;
    for (int walk = 0; walk < (two ? 2 : 1); walk++) {
      uint64_t ev = sr_event_key(sh.sr_seed, EV_WALK0 + walk, wid, ev_step);
      if (pos[walk] >= len[walk]) {
        if (sh.policy == POLICY_REF) ref_flush_walk(walk);
        else win_flush_all(walk, ev);
        len[walk] = 0;
        train_sen_num++;
      } else if (sh.policy == POLICY_WINDOW) {
        int P = pos[walk];
        if (P + w < len[walk]) win_enter(walk, P + w);
        if (P - w - 1 >= 0) win_leave(walk, P - w - 1, ev);
      }
    }
    if (train_sen_num >= 2) {
      if (sh.policy == POLICY_REF) {
        uint64_t ev = sr_event_key(sh.sr_seed, EV_POOL, wid, ev_step);
        for (size_t p = 0; p < neg_buffer.size(); p++)
          store_row(Woh + (size_t)neg_buffer[p] * d, &negbuf[p * d], ev, neg_buffer[p]);
      }
      change_neg = true;
      train_sen_num = 0;
    }
    step_id++;
  }

  // one pass of the reference's compute loop body (dsgl.hpp:876-1407); false = done
  bool iterate() {
    if (word_count - last_word_count > 10000) {  // dsgl.hpp:886-897
      uint64_t diff = word_count - last_word_count;
      uint64_t wca_now = sh.wca.fetch_add(diff) + diff;
      last_word_count = word_count;
      float a = sh.start_alpha *
                (1 - (float)(wca_now * 1ULL) / (float)((uint64_t)sh.iter * sh.train_words + 1));
      if (a < sh.start_alpha * 0.0001f) a = sh.start_alpha * 0.0001f;
      sh.alpha.store(a, std::memory_order_relaxed);
    }
    for (int w = 0; w < sh.windows; w++) {
      while (len[w] == 0) {
        if (slice_done()) break;
        fill_walk(w);
        if (len[w] == 1 || len[w] == 0) {
          len[w] = 0;
          continue;
        }
        on_walk_loaded(w);
      }
    }
    if (slice_done()) {  // dsgl.hpp:1031-1050
      sh.wca.fetch_add(word_count - last_word_count);
      local_iter--;
      if (local_iter == 0) return false;
      word_count = 0;
      cur = start;
      last_word_count = 0;
      len[0] = len[1] = 0;
      if (sh.policy == POLICY_WINDOW) {
        win_drop(0);
        win_drop(1);
      }
      return true;
    }
    if (change_neg) build_pool();
    step();
    return true;
  }
};

template <int S>
void run_workers(Shared& sh, typename Store<S>::T* Wih, typename Store<S>::T* Woh, int threads, int schedule) {
  if (schedule == 1) {
    // every worker in flight: thread t owns workers t, t + threads, ... and gives each of
    // them one step in turn until all have finished their slices
#pragma omp parallel num_threads(threads < 1 ? 1 : threads)
    {
      const int nt = omp_get_num_threads(), t = omp_get_thread_num();
      std::vector<Worker<S>*> mine;
      for (int id = t; id < sh.workers; id += nt) mine.push_back(new Worker<S>(sh, Wih, Woh, (uint32_t)id));
      size_t live = mine.size();
      while (live)
        for (auto& w : mine)
          if (w && !w->iterate()) {
            delete w;
            w = nullptr;
            live--;
          }
    }
    return;
  }
  if (sh.workers == 1 || threads <= 1) {
    // deterministic: workers run one after another, each to completion
    for (int id = 0; id < sh.workers; id++) {
      Worker<S> wk(sh, Wih, Woh, (uint32_t)id);
      while (wk.iterate()) {
      }
    }
    return;
  }
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
  for (int id = 0; id < sh.workers; id++) {
    Worker<S> wk(sh, Wih, Woh, (uint32_t)id);
    while (wk.iterate()) {
    }
  }
}

}  // namespace

extern "C" {

struct oracle_config {
  int32_t d, window, negative, iter;
  int32_t workers;        // corpus slices = reference compute threads
  int32_t threads;        // host threads running the workers (1 = deterministic)
  int32_t table_threads;  // -threads of the reference: partition of the table reduction
  int32_t policy;         // 0 = reference buffers, 1 = GPU window/direct policy
  int32_t storage;        // 0 = f32, 1 = bf16 + stochastic rounding, 2 = f64
  int32_t schedule;       // 0 = each worker runs to completion (at most `threads` in
                          // flight, as the reference's compute threads); 1 = every worker in
                          // flight at once, each thread stepping its workers round-robin
                          // (how a GPU runs them; used to study concurrency, not for parity)
  int64_t table_size;
  float sample, alpha;
  uint64_t sr_seed;
  int32_t windows;        // windows per step: 2 (the reference's two walks) or 1
  int32_t pad_;
};

struct oracle_stats {
  uint64_t steps, pairs, word_count_actual;
  float final_alpha;
  float pad_;
  double train_seconds;  // the worker loop alone, as the reference's "Train SGNS MPI TIME"
                         // (dsgl.hpp:1571-1573) excludes preparatory_work
};

void oracle_build_vocab(const int32_t* counts, int64_t V, uint32_t* order, int32_t* row_of,
                        int32_t* cn_sorted, uint64_t* train_words) {
  build_vocab(counts, V, order, row_of, cn_sorted, train_words);
}
void oracle_build_unigram_table(const int32_t* cn_sorted, int64_t V, int64_t table_size,
                                int32_t threads, int32_t* table) {
  build_unigram_table(cn_sorted, V, table_size, threads, table);
}
void oracle_build_exp_table(float* t) { build_exp_table(t); }
void oracle_init_wih(int64_t V, int32_t d, float* Wih) {  // dsgl.hpp:451-456
  uint64_t r = 1;
  for (int64_t i = 0; i < V * d; i++) {
    r = lcg_next(r);
    Wih[i] = (((float)(r & 0xFFFF) / 65536.f) - 0.5f) / (float)(size_t)d;
  }
}
uint64_t oracle_lcg_next(uint64_t r) { return lcg_next(r); }
uint16_t oracle_bf16_sr(float x, uint64_t seed, int32_t kind, uint32_t worker, uint64_t step,
                        uint32_t row, int32_t col) {
  return f32_to_bf16_sr(x, sr_bits16(sr_event_key(seed, kind, worker, step), row, col));
}

// Full training run.  counts: per-vertex occurrence counts (V).  corpus: vertex ids
// with -1 walk separators.  Wih/Woh: V*d elements of the storage type, in sorted-row
// order; Wih must hold the initial values (oracle_init_wih) and Woh zeros.
int oracle_train(const oracle_config* cfg, const int32_t* counts, int64_t V, const int32_t* corpus,
                 int64_t n_tokens, void* Wih, void* Woh, oracle_stats* stats) {
  if (V < 2 || cfg->d < 1 || cfg->window < 1 || cfg->negative < 0 || cfg->workers < 1) return -1;
  std::vector<uint32_t> order(V);
  std::vector<int32_t> row_of(V), cn_sorted(V);
  uint64_t train_words = 0;
  build_vocab(counts, V, order.data(), row_of.data(), cn_sorted.data(), &train_words);
  std::vector<int32_t> table(cfg->table_size);
  build_unigram_table(cn_sorted.data(), V, cfg->table_size, cfg->table_threads, table.data());
  std::vector<float> exp_table(kExpTableSize + 1);
  build_exp_table(exp_table.data());
  std::vector<float> ran(V);
  build_keep_threshold(counts, V, cfg->sample, train_words, ran.data());

  Shared sh;
  sh.corpus = corpus;
  sh.words_num = n_tokens;
  sh.row_of = row_of.data();
  sh.ran = ran.data();
  sh.table = table.data();
  sh.table_size = cfg->table_size;
  sh.V = V;
  sh.exp_table = exp_table.data();
  sh.d = cfg->d;
  sh.window = cfg->window;
  sh.negative = cfg->negative;
  sh.iter = cfg->iter;
  sh.workers = cfg->workers;
  sh.policy = cfg->policy;
  sh.windows = cfg->windows == 1 ? 1 : 2;
  sh.sample = cfg->sample;
  sh.start_alpha = cfg->alpha;
  sh.train_words = train_words;
  sh.sr_seed = cfg->sr_seed;
  sh.wca = 0;
  sh.alpha = cfg->alpha;
  sh.steps = 0;
  sh.pairs = 0;
  const double t0 = omp_get_wtime();
  if (cfg->storage == STORE_F32)
    run_workers<STORE_F32>(sh, (float*)Wih, (float*)Woh, cfg->threads, cfg->schedule);
  else if (cfg->storage == STORE_BF16)
    run_workers<STORE_BF16>(sh, (uint16_t*)Wih, (uint16_t*)Woh, cfg->threads, cfg->schedule);
  else if (cfg->storage == STORE_F64)
    run_workers<STORE_F64>(sh, (double*)Wih, (double*)Woh, cfg->threads, cfg->schedule);
  else
    return -1;
  if (stats) {
    stats->steps = sh.steps.load();
    stats->pairs = sh.pairs.load();
    stats->word_count_actual = sh.wca.load();
    stats->final_alpha = sh.alpha.load();
    stats->train_seconds = omp_get_wtime() - t0;
  }
  return 0;
}

// One minibatch update, given explicit rows (the per-minibatch check of the GPU step).
// inputM: I rows, outputM: O rows (row 0 = target of walk 1, row O-1 = target of walk
// 2), first = number of inputs from walk 1, meta: multiplicity of each output row.
// Writes dIn (I x d, the reference's updated inputM) and dOut (O x d, outputMd).
// acc: 0 = float (fused sequential order), 1 = double.
int oracle_minibatch(int32_t acc, int32_t d, int32_t I, int32_t first, int32_t O,
                     const int32_t* meta, float alpha, const double* inputM,
                     const double* outputM, double* dIn, double* dOut) {
  std::vector<float> et(kExpTableSize + 1);
  build_exp_table(et.data());
  auto run = [&](auto zero) {
    typedef decltype(zero) A;
    std::vector<A> x((size_t)I * d), o((size_t)O * d), corr((size_t)O * I);
    for (size_t q = 0; q < x.size(); q++) x[q] = (A)inputM[q];
    for (size_t q = 0; q < o.size(); q++) o[q] = (A)outputM[q];
    const A al = (A)alpha;
    for (int i = 0; i < O; i++)
      for (int j = 0; j < I; j++) {
        A f = 0;
        for (int k = 0; k < d; k++) f = fma_acc(o[(size_t)i * d + k], x[(size_t)j * d + k], f);
        int label = j < first ? (i == 0 ? 1 : 0) : (i == O - 1 ? 1 : 0);
        A g;
        if (f > kMaxExp) g = (A)(label - 1) * al;
        else if (f < -kMaxExp) g = (A)label * al;
        else g = ((A)label - (A)et[(int)((f + (A)kMaxExp) * (A)kTableScale)]) * al;
        corr[(size_t)i * I + j] = g * (A)meta[i];
      }
    for (int i = 0; i < O; i++)
      for (int c = 0; c < d; c++) {
        A f = 0;
        for (int j = 0; j < I; j++) f = fma_acc(corr[(size_t)i * I + j], x[(size_t)j * d + c], f);
        dOut[(size_t)i * d + c] = (double)f;
      }
    for (int j = 0; j < I; j++)
      for (int c = 0; c < d; c++) {
        A f = 0;
        for (int i = 0; i < O; i++) f = fma_acc(corr[(size_t)i * I + j], o[(size_t)i * d + c], f);
        dIn[(size_t)j * d + c] = (double)f;
      }
    return 0;
  };
  if (acc == 0) return run(0.0f);
  return run(0.0);
}

// Walk text -> corpus tokens.  The reference writes " %u" per vertex and "\n" after each
// walk (include/path.hpp:92,108) and its reader splits lines on " \n\r\t"
// (src/word2vec.cu:1002-1041); this restatement reads ids as integers of at most 10 digits
// (leading zeros included) no larger than 2^31 - 1, emits -1 after every line that holds an
// id, and treats the end of the buffer as a final newline.  Returns 0, 1 (a byte other than
// a digit or separator: *err_pos = its smallest offset; checked before ids), 2 (an id too
// long or too large: *err_pos = offset of its last digit) or 3 (more than cap tokens;
// *n_out still says how many).
int32_t oracle_parse_walks(const uint8_t* b, int64_t n, int32_t* out, int64_t cap, int64_t* n_out,
                           int64_t* max_id, int64_t* err_pos) {
  *n_out = 0;
  *max_id = -1;
  *err_pos = -1;
  for (int64_t i = 0; i < n; i++) {
    const uint8_t c = b[i];
    if (!((c >= '0' && c <= '9') || c == ' ' || c == '\t' || c == '\r' || c == '\n')) {
      *err_pos = i;
      return 1;
    }
  }
  int64_t cnt = 0, val = 0;
  int nd = 0;
  bool line_has_ids = false;
  int32_t code = 0;
  for (int64_t i = 0; i <= n; i++) {
    const uint8_t c = i < n ? b[i] : (uint8_t)'\n';
    if (c >= '0' && c <= '9') {
      val = val * 10 + (c - '0');
      nd++;
      if (nd > 11) val = 0;  // already too long; keep val bounded
      continue;
    }
    if (nd > 0) {
      if (nd > 10 || val > 2147483647LL) {
        if (code == 0) {
          code = 2;
          *err_pos = i - 1;
        }
        val = 0;
      }
      if (cnt < cap) out[cnt] = (int32_t)val;
      cnt++;
      if (val > *max_id) *max_id = val;
      line_has_ids = true;
      nd = 0;
      val = 0;
    }
    if (c == '\n') {
      if (line_has_ids) {
        if (cnt < cap) out[cnt] = -1;
        cnt++;
      }
      line_has_ids = false;
    }
  }
  *n_out = cnt;
  if (code) return code;
  return cnt > cap ? 3 : 0;
}

// Link-prediction score of pair (u, v): <table[u], table[v]> in fp32, in the GPU kernel's
// fixed order -- lane l (0..31) sums columns 4l..4l+3 of each 128-column chunk with fused
// multiply-adds, then the lane sums are combined by an xor butterfly (16, 8, 4, 2, 1).
// dtype 0: fp32 table; 1: bf16 table (raw bits).  Returns 1 if a pair is outside [0, V)
// (its score is 0), else 0.
int32_t oracle_link_scores(int32_t dtype, int32_t d, const void* table, int64_t V, const int32_t* pairs, int64_t n,
                           float* scores) {
  int32_t bad = 0;
  auto at = [&](int64_t row, int c) -> float {
    if (dtype == 1) return bf16_to_f32(static_cast<const uint16_t*>(table)[row * d + c]);
    return static_cast<const float*>(table)[row * d + c];
  };
  for (int64_t i = 0; i < n; i++) {
    const int32_t u = pairs[2 * i], v = pairs[2 * i + 1];
    if (u < 0 || v < 0 || u >= V || v >= V) {
      scores[i] = 0.f;
      bad = 1;
      continue;
    }
    float lane[32];
    for (int l = 0; l < 32; l++) {
      float acc = 0.f;
      for (int q = l; q < d / 4; q += 32)
        for (int k = 0; k < 4; k++) acc = fmaf(at(u, 4 * q + k), at(v, 4 * q + k), acc);
      lane[l] = acc;
    }
    for (int o = 16; o > 0; o >>= 1) {
      float next[32];
      for (int l = 0; l < 32; l++) next[l] = lane[l] + lane[l ^ o];
      for (int l = 0; l < 32; l++) lane[l] = next[l];
    }
    scores[i] = lane[0];
  }
  return bad;
}

}  // extern "C"
