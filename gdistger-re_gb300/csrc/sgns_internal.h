// sgns_internal.h -- structures shared by the host library and the CUDA kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#if defined(__CUDACC__)
#define SGNS_HD __host__ __device__ __forceinline__
#else
#define SGNS_HD inline
#endif

namespace sgns {

constexpr int kMaxExp = 6;                                 // dsgl.hpp:22
constexpr int kExpTableSize = 1000;                        // dsgl.hpp:21
constexpr int kMaxSentence = 1000;                         // dsgl.hpp:23
constexpr int kTableScale = kExpTableSize / kMaxExp / 2;   // integer 83, dsgl.hpp:1257
constexpr int kWMax = 16;                                  // window limit of the kernels
constexpr int kKMax = 10;                                  // negative limit of the kernels
constexpr int kOMax = kKMax + 2;                           // outputs per step
constexpr int kIMax = 4 * kWMax;                           // inputs per step (two windows)
constexpr int kDMax = 256;                                 // hidden size limit

// write-event kinds of the stochastic-rounding stream (same numbering as the oracle)
enum { EV_TARGET1 = 0, EV_TARGET2 = 1, EV_WALK0 = 2, EV_WALK1 = 3, EV_NEG = 4, EV_POOL = 5 };
enum { STORE_F32 = 0, STORE_BF16 = 1 };

// ---- 64-bit division by an invariant divisor --------------------------------------
// Granlund & Montgomery, "Division by invariant integers using multiplication" (PLDI
// 1994), Fig. 4.1 with N = 64: q = (t + ((n - t) >> 1)) >> (l - 1), t = mulhi(m, n),
// l = ceil(log2 d), m = floor(2^64 (2^l - d) / d) + 1.  Exact for every 64-bit n.
struct FastDiv64 {
  uint64_t d;
  uint64_t m;
  int32_t shift;  // l - 1
  int32_t one;    // d == 1
};

inline FastDiv64 make_fastdiv(uint64_t d) {
  FastDiv64 f{};
  f.d = d;
  if (d <= 1) {
    f.one = 1;
    return f;
  }
  int l = 0;
  while (l < 64 && ((unsigned __int128)1 << l) < d) l++;
  unsigned __int128 two64 = (unsigned __int128)1 << 64;
  unsigned __int128 num = two64 * ((((unsigned __int128)1) << l) - d);
  f.m = (uint64_t)(num / d + 1);
  f.shift = l - 1;
  return f;
}

SGNS_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
SGNS_HD uint64_t fast_div(uint64_t n, const FastDiv64& f) {
  if (f.one) return n;
  uint64_t t = mulhi64(f.m, n);
  return (t + ((n - t) >> 1)) >> f.shift;
}
SGNS_HD uint64_t fast_mod(uint64_t n, const FastDiv64& f) { return n - fast_div(n, f) * f.d; }

// ---- the reference's LCG (dsgl.hpp:925) and jump-ahead -----------------------------
constexpr uint64_t kLcgA = 25214903917ULL;
constexpr uint64_t kLcgC = 11ULL;
SGNS_HD uint64_t lcg_next(uint64_t r) { return r * kLcgA + kLcgC; }

// r_{n+k} = mul[k] * r_n + add[k]; small[] covers k = 0..32, pow2[] covers k = 2^i.
struct LcgJumps {
  uint64_t small_mul[33], small_add[33];
  uint64_t pow2_mul[64], pow2_add[64];
};
inline void make_lcg_jumps(LcgJumps* j) {
  uint64_t m = 1, a = 0;
  for (int k = 0; k <= 32; k++) {
    j->small_mul[k] = m;
    j->small_add[k] = a;
    a = a * kLcgA + kLcgC;
    m = m * kLcgA;
  }
  uint64_t pm = kLcgA, pa = kLcgC;
  for (int i = 0; i < 64; i++) {
    j->pow2_mul[i] = pm;
    j->pow2_add[i] = pa;
    pa = pm * pa + pa;  // compose the step with itself
    pm = pm * pm;
  }
}

// ---- stochastic rounding (identical stream in the oracle) --------------------------
SGNS_HD uint64_t mix64(uint64_t z) {  // SplitMix64 finaliser (Steele, Lea, Flood 2014)
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
SGNS_HD uint64_t sr_event_key(uint64_t seed, int kind, uint32_t worker, uint64_t step) {
  return mix64(seed ^ ((uint64_t)kind << 56) ^ ((uint64_t)worker << 34) ^ step);
}
// 64 random bits for the 4 consecutive columns 4*col4 .. 4*col4+3 of one row, from the
// event key ev (one SplitMix64 output per write event):
//   h  = fmix32(lo32(ev) ^ (row * 0x9E3779B1 + col4 * 0x85EBCA77))   (murmur3's 32-bit
//        finaliser, Appleby 2011; constants of Wellons' low-bias variant),
//   t  = (h ^ hi32(ev)) * 0x9E3779B1 (mod 2^32),  h2 = t ^ (t >> 16),
//   bits = h2 << 32 | h  (columns 4q, 4q+1 take h; 4q+2, 4q+3 take h2).
// Both words are bijections of uniform words, so every 16-bit field is uniform and the
// rounding unbiased (the high word of a product by a 32-bit constant would not be: its
// range ends at the constant).  About half the instructions of a 64-bit finaliser per
// chunk, on the write-back path of every output row of every step.
SGNS_HD uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  return h ^ (h >> 16);
}
SGNS_HD uint64_t sr_bits4(uint64_t ev, uint32_t row, uint32_t col4) {
  const uint32_t h = fmix32((uint32_t)ev ^ (row * 0x9E3779B1u + col4 * 0x85EBCA77u));
  const uint32_t t = (h ^ (uint32_t)(ev >> 32)) * 0x9E3779B1u;
  return ((uint64_t)(t ^ (t >> 16)) << 32) | h;
}
SGNS_HD float bf16_bits_to_f32(uint16_t b) {
  uint32_t u = (uint32_t)b << 16;
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  __builtin_memcpy(&f, &u, 4);
  return f;
#endif
}

// ---- kernel parameters -------------------------------------------------------------
struct DeviceCounters {            // one per handle, in device memory
  unsigned long long wca;          // word_count_actual (dsgl.hpp:536)
  unsigned long long steps;
  unsigned long long pairs;        // sum of I (input rows) over steps
  unsigned long long outputs;      // sum of O (output rows) over steps
  unsigned long long row_loads;    // table rows read into on-chip/HBM buffers
  unsigned long long row_stores;   // table rows written back from buffers
  double loss;
  float alpha;                     // the shared learning rate (dsgl.hpp:894)
  int32_t active;                  // workers still running
  int32_t status;                  // 0 or an sgns_status set by a kernel
  int32_t pad;
};

struct TrainParams {
  const int32_t* corpus;           // sorted rows, -1 separators
  int64_t words_num;
  const float* ran;                // subsampling keep threshold per row
  const int32_t* table;            // unigram^0.75 table (rows)
  const float* exp_table;          // 1001 sigmoid values
  const LcgJumps* jumps;           // device copy of the LCG jump tables
  void* wih;
  void* woh;
  FastDiv64 div_table, div_vm1, div_window;
  int64_t V;
  int32_t d, window, K, iter, workers, sample_on;
  float start_alpha, alpha_denom;
  uint64_t sr_seed;
  int32_t compute_loss, lmax, storage;
  int32_t fwd_tile;                // lanes per input in the forward (1, or 2 where supported)
  int32_t windows;                 // windows per step: 2 (two walks, dsgl.hpp:1100-1132) or 1
  int32_t pad2;
  DeviceCounters* ctr;
  // plain-engine state (HBM)
  void* plain_state;
  int64_t plain_stride;            // bytes of scratch per worker
};

// host-side launchers (CUDA translation units)
cudaError_t launch_init_wih(void* wih, int storage, int64_t V, int32_t d, const LcgJumps* jumps,
                            cudaStream_t s);
cudaError_t launch_map_corpus(const int32_t* ids, const int32_t* row_of, int32_t* rows, int64_t n,
                              int64_t V, int32_t* bad, cudaStream_t s);
// longest run of non-separator tokens, capped at kMaxSentence (atomicMax into *out)
// hotness-block sync: rows of a table (fp32 or bf16) to fp32 rows of buf and back
// (table row = buf row / divisor, bf16 rounded to nearest even)
cudaError_t launch_gather_rows(const void* tab, int storage, int d, const int32_t* rows, int64_t n, float* buf,
                               cudaStream_t s);
cudaError_t launch_scatter_rows(void* tab, int storage, int d, const int32_t* rows, int64_t n, const float* buf,
                                float divisor, cudaStream_t s);
// bf16 bits -> fp32 for n elements (n % 4 == 0)
cudaError_t launch_widen_bf16(const void* src, float* dst, int64_t n, cudaStream_t s);
cudaError_t launch_max_walk(const int32_t* rows, int64_t n, int32_t* out, cudaStream_t s);
size_t window_smem_bytes(int d, int window, int K, int lmax, int warps_per_cta);
cudaError_t window_engine_occupancy(int storage, int d, int window, int K, int lmax, int wpc, int tile,
                                    int* ctas_per_sm);
// whether a problem shape has the two-lanes-per-input forward (d <= 128, K <= 5)
inline bool window_engine_has_tile2(int d, int K) { return d <= 128 && K <= 5; }
cudaError_t launch_window_engine(const TrainParams& p, int warps_per_cta, cudaStream_t s);
size_t plain_worker_bytes(int d, int window, int K, int lmax);
cudaError_t launch_plain_init(const TrainParams& p, cudaStream_t s);
cudaError_t launch_plain_step(const TrainParams& p, cudaStream_t s);
// offsets: device scratch of 2*n int64; *status set to 1 for a minibatch over the limits
cudaError_t launch_minibatch(int d, int n, int imax, int omax, const int32_t* in_count,
                             const int32_t* in_first, const int32_t* out_count, const int32_t* out_meta,
                             const float* alpha, const float* in_rows, const float* out_rows, float* d_in,
                             float* d_out, const float* exp_table, int64_t* offsets, int32_t* status,
                             cudaStream_t s);
// the same update, each updated row written as bf16 bits with the trainers' stochastic
// rounding (event keys from sr_seed and the minibatch index)
cudaError_t launch_minibatch_bf16(int d, int n, int imax, const int32_t* in_count, const int32_t* in_first,
                                  const int32_t* out_count, const int32_t* out_meta, const float* alpha,
                                  const float* in_rows, const float* out_rows, uint16_t* new_in, uint16_t* new_out,
                                  uint64_t sr_seed, const float* exp_table, int64_t* offsets, int32_t* status,
                                  cudaStream_t s);
// host helpers shared by the translation units (sgns_host.cpp)
// walk-file text -> corpus (dsgl_ingest.cu); scratch of ingest_scratch_bytes(n) bytes
size_t ingest_scratch_bytes(int64_t n);
cudaError_t launch_ingest_count(const uint8_t* bytes, int64_t n, void* scratch, unsigned long long* n_out,
                                long long* err_pos, cudaStream_t s);
cudaError_t launch_ingest_emit(const uint8_t* bytes, int64_t n, void* scratch, int32_t* tokens, long long* err_pos,
                               long long* max_id, cudaStream_t s);
cudaError_t launch_vertex_count(const int32_t* tokens, int64_t n, int32_t* counts, int64_t V, int num_sms,
                                cudaStream_t s);

// link-prediction scores (dsgl_eval.cu); *bad set to 1 for a pair outside [0, V)
cudaError_t launch_link_scores(int storage, const void* table, int d, int64_t V, const int32_t* pairs, int64_t n,
                               float* scores, int32_t* bad, int num_sms, cudaStream_t s);

// information-oriented walks and common-neighbour counts (dsgl_walk.cu)
constexpr int kWalkMaxLength = 1000;  // vertices per walk (the trainer's limit, dsgl.hpp:23)
cudaError_t launch_validate_csr(const int64_t* indptr, const int32_t* indices, int64_t V, int64_t E,
                                int32_t* status, int num_sms, cudaStream_t s);
cudaError_t launch_edge_common_neighbors(const int64_t* indptr, const int32_t* indices, int64_t V, int64_t E,
                                         int32_t* cn, int32_t* status, int num_sms, cudaStream_t s);
int walk_block_threads(int max_length);
size_t walk_scratch_bytes(int64_t walker_num);
cudaError_t launch_info_walks_count(const int64_t* indptr, const int32_t* indices, const int32_t* cn,
                                    const double* xl, int64_t V, int64_t walker_num, int min_length,
                                    int max_length, double r_threshold, uint64_t seed, int trace, void* scratch,
                                    int num_sms, int64_t** offsets_out, cudaStream_t s);
cudaError_t launch_info_walks_emit(const int64_t* indptr, const int32_t* indices, const int32_t* cn,
                                   const double* xl, int64_t V, int64_t walker_num, int min_length, int max_length,
                                   double r_threshold, uint64_t seed, int trace, const int64_t* offsets,
                                   int32_t* corpus, int num_sms, cudaStream_t s);

void host_exp_table(float* t /* kExpTableSize + 1 */);
int report_error(int status, const char* fmt, ...);  // sets sgns_last_error(NULL); returns status

size_t adjoint_scratch_bytes(int64_t V);
// phase 1 of the adjoint: marks, checks, slots, ids, zeroed gradient rows; info (device, 5
// ints): distinct input rows, distinct output rows, status bits (1 bad id, 2 bad size),
// largest input count, largest output count
cudaError_t launch_adjoint_prepare(int dtype, int d, int n, int64_t V, const int32_t* in_ptr, const int32_t* in_ids,
                                   const int32_t* in_first, const int32_t* out_ptr, const int32_t* out_ids,
                                   double* loss, int32_t* grad_in_ids, void* grad_in, int32_t* grad_out_ids,
                                   void* grad_out, int32_t* info, void* scratch, cudaStream_t s);
// phase 2: loss and row gradients (imax / omax from phase 1)
cudaError_t launch_adjoint(int dtype, int d, int n, int64_t V, int imax, int omax, const int32_t* in_ptr,
                           const int32_t* in_ids, const int32_t* in_first, const int32_t* out_ptr,
                           const int32_t* out_ids, const int32_t* out_meta, const void* wih, const void* woh,
                           double* loss, void* grad_in, void* grad_out, void* scratch, cudaStream_t s);

}  // namespace sgns

// Host set-up of sgns_set_vocab (sorted rows, unigram table, subsampling thresholds, sigmoid
// table) without a device, exported for the CPU tests; not part of include/sgns.h.  Any
// output pointer may be null.  Returns SGNS_EINVAL for V or table_size outside
// [1, 2^31 - 1] or a negative count.
extern "C" int32_t sgns_internal_host_vocab(const int32_t* counts, int64_t V, float sample, int64_t table_size,
                                            int32_t threads, uint32_t* order, int32_t* table, float* ran,
                                            float* exp_table, uint64_t* train_words);
// The writer of sgns_save_text (my_saveModel's format) on host arrays: order (V row ids),
// w (V x d floats, sorted-row order); exported for the CPU tests.
extern "C" int32_t sgns_internal_write_embedding(const uint32_t* order, const float* w, int64_t V, int32_t d,
                                                 int32_t binary, const char* path);
// The walker's x * log2(x) table (n entries) exactly as sgns_info_walks builds it; exported
// for the CPU tests.
extern "C" void sgns_internal_xlog2x_table(int32_t n, double* t);
// The stochastic-rounding bits of n (event key, row, column chunk) triples, computed by the
// host copy of sr_bits4 (the kernels' function); exported for the CPU tests.
extern "C" void sgns_internal_sr_bits4(int64_t n, const uint64_t* ev, const uint32_t* row, const uint32_t* col4,
                                       uint64_t* bits);
// The row draw of sgns_sync_rows from count-sorted counts (no device); exported for the CPU
// tests.  Returns SGNS_EINVAL (with *n_rows set) when cap is too small.
extern "C" int32_t sgns_internal_sync_rows(const int32_t* cn_sorted, int64_t V, uint64_t seed, uint64_t round,
                                           int32_t full, int32_t* rows, int64_t cap, int64_t* n_rows);
