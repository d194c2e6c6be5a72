// sgns_host.cpp -- the C ABI of include/sgns.h: options, vocabulary and tables, corpus
// staging, engine dispatch, CUDA-graph capture of the persistent launch, the autotuner,
// and the reference's text embedding output.
//
// Host-side set-up follows the reference's preparatory_work (include/dsgl.hpp:511-519):
// vocabulary sort, unigram table, sigmoid table and subsampling thresholds are built
// here once per vocabulary (the reference also builds them on the host); all training
// work runs in the CUDA kernels.  There is no CPU training path.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>  // header-only; ranges are free unless a profiler is attached

#include "sgns.h"
#include "sgns_internal.h"

using namespace sgns;

// NVTX range for the duration of a scope (library phases in a profiler timeline)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

struct sgns_handle {
  sgns_options opt{};
  std::string err;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // vocabulary (host)
  int64_t V = 0;
  uint64_t train_words = 0;
  std::vector<uint32_t> order;
  std::vector<int32_t> row_of, cn_sorted;
  // device state
  void* wih = nullptr;
  void* woh = nullptr;
  int32_t* d_row_of = nullptr;
  float* d_ran = nullptr;
  int32_t* d_table = nullptr;
  float* d_exp = nullptr;
  LcgJumps* d_jumps = nullptr;
  DeviceCounters* d_ctr = nullptr;
  DeviceCounters* h_ctr = nullptr;  // pinned
  int32_t* d_flags = nullptr;       // [0] bad id, [1] longest walk
  int32_t* h_flags = nullptr;       // pinned
  int32_t* d_ids = nullptr;
  int32_t* d_corpus = nullptr;
  int64_t n_tokens = 0, corpus_cap = 0;
  int lmax = 0;
  void* plain_scratch = nullptr;
  size_t plain_bytes = 0;
  // persistent engine launch shape and its captured graph
  int workers = 0, wpc = 0, tile = 1;
  bool tuned = false;
  cudaGraphExec_t graph = nullptr;
  std::string graph_key;
  sgns_stats stats{};
};

namespace {

// message of the calling thread's last failed call without a handle (sgns_create, the
// kernel-level entry points); per thread, so the pointer sgns_last_error(NULL) returns
// stays valid until that thread's next failure
thread_local std::string g_create_err;

sgns_status fail(sgns_handle* h, sgns_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  else {
    g_create_err = buf;
  }
  // a failed allocation or copy also sets the runtime's per-thread last error, which the
  // launchers read back after their next launch: clear it so it is reported only here
  if (st == SGNS_ECUDA || st == SGNS_ENOMEM) cudaGetLastError();
  return st;
}

#define CU(h, call)                                                                          \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return fail((h), SGNS_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),   \
                  __FILE__, __LINE__);                                                       \
  } while (0)

template <class T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

size_t elem_bytes(const sgns_options& o) { return o.storage == SGNS_STORE_BF16_SR ? 2 : 4; }

// Back to the state before any vocabulary: every buffer sized by V or by the corpus is
// freed together, so no later call sees some of them and not the others.
void drop_vocab(sgns_handle* h) {
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  h->graph_key.clear();
  h->tuned = false;
  dfree(h->wih);
  dfree(h->woh);
  dfree(h->d_row_of);
  dfree(h->d_ran);
  dfree(h->d_table);
  dfree(h->d_corpus);
  dfree(h->d_ids);
  h->V = 0;
  h->train_words = 0;
  h->n_tokens = h->corpus_cap = 0;
  h->lmax = 2;  // an empty corpus: the shortest walk the engines stage
}

// ---- the reference's host set-up, restated (dsgl.hpp:121-147, 246-252, 314-382) ----
struct VocabVertex {
  int cn;
  uint32_t id;
};

void build_unigram_table(const std::vector<int32_t>& cn, int64_t table_size, int threads,
                         std::vector<int32_t>& table) {
  const int64_t V = (int64_t)cn.size();
  const float power = 0.75f;
  if (threads < 1) threads = 1;
  // OpenMP static-schedule reduction of dsgl.hpp:127-132: per-thread contiguous
  // partial sums, combined in thread order.
  double twp = 0.;
  const int64_t q = V / threads, rem = V % threads;
  for (int t = 0; t < threads; t++) {
    const int64_t lo = t * q + std::min<int64_t>(t, rem);
    const int64_t hi = lo + q + (t < rem ? 1 : 0);
    double part = 0.;
    for (int64_t i = lo; i < hi; i++) part += std::pow((double)cn[i], (double)power);
    twp += part;
  }
  table.resize(table_size);
  int64_t i = 0;
  float d1 = (float)(std::pow((double)cn[0], (double)power) / twp);
  for (int64_t a = 0; a < table_size; a++) {
    table[a] = (int32_t)i;
    if ((float)(int)a / (float)table_size > d1) {
      i++;
      if (i >= V) i = V - 1;
      d1 = (float)((double)d1 + std::pow((double)cn[i], (double)power) / twp);
    }
  }
}

// The reference's host set-up of a vocabulary: rows sorted by count, descending, with
// std::sort (dsgl.hpp:246-252, 314-382), the unigram table (dsgl.hpp:121-147) and the
// subsampling keep thresholds sqrt(r) + r, r = sample * train_words / count (dsgl.hpp:
// 923-924), indexed by sorted row as the reference indexes its vertex-indexed count array.
struct HostVocab {
  std::vector<uint32_t> order;
  std::vector<int32_t> row_of, cn_sorted, table;
  std::vector<float> ran;
  uint64_t train_words = 0;
};

void build_host_vocab(const int32_t* counts, int64_t V, float sample, int64_t table_size, int threads,
                      HostVocab& hv) {
  std::vector<VocabVertex> v(V);
  uint64_t tw = 0;
  for (int64_t i = 0; i < V; i++) {
    v[i].cn = counts[i];
    v[i].id = (uint32_t)i;
    tw += (uint64_t)counts[i];
  }
  std::sort(v.begin(), v.end(), [](VocabVertex a, VocabVertex b) { return a.cn > b.cn; });
  hv.order.resize(V);
  hv.row_of.resize(V);
  hv.cn_sorted.resize(V);
  for (int64_t r = 0; r < V; r++) {
    hv.order[r] = v[r].id;
    hv.row_of[v[r].id] = (int32_t)r;
    hv.cn_sorted[r] = v[r].cn;
  }
  build_unigram_table(hv.cn_sorted, table_size, threads, hv.table);
  hv.ran.resize(V);
  const float st = sample * (float)tw;
  for (int64_t w = 0; w < V; w++) {
    const float ratio = st / (float)counts[w];
    hv.ran[w] = sqrtf(ratio) + ratio;
  }
  hv.train_words = tw;
}

// my_saveModel (dsgl.hpp:1443-1461): "V d\n", then per row "<id> " and d x "%f " (or d raw
// floats with binary) and "\n", rows in sorted order.  Rows are formatted in parallel
// chunks and written in order.  Returns SGNS_EIO when the file cannot be written.
sgns_status write_embedding(const uint32_t* order, const float* w, int64_t V, int d, bool binary, const char* path) {
  FILE* f = fopen(path, "wb");
  if (!f) return SGNS_EIO;
  fprintf(f, "%lld %lld\n", (long long)V, (long long)d);  // dsgl.hpp:1448
  const int nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  const int64_t chunk = 4096;
  bool ok = true;
  for (int64_t r0 = 0; r0 < V && ok; r0 += chunk * nth) {
    std::vector<std::string> parts(nth);
    std::vector<std::thread> th;
    for (int t = 0; t < nth; t++)
      th.emplace_back([&, t] {
        const int64_t lo = r0 + t * chunk, hi = std::min<int64_t>(V, lo + chunk);
        std::string& s = parts[t];
        char buf[64];
        for (int64_t r = lo; r < hi; r++) {
          int n = snprintf(buf, sizeof buf, "%u ", order[r]);
          s.append(buf, n);
          if (binary) {
            s.append(reinterpret_cast<const char*>(&w[(size_t)r * d]), sizeof(float) * d);
          } else {
            for (int c = 0; c < d; c++) {
              n = snprintf(buf, sizeof buf, "%f ", w[(size_t)r * d + c]);
              s.append(buf, n);
            }
          }
          s.push_back('\n');
        }
      });
    for (auto& t : th) t.join();
    for (auto& s : parts)
      if (!s.empty() && fwrite(s.data(), 1, s.size(), f) != s.size()) ok = false;
  }
  if (fclose(f) != 0) ok = false;
  return ok ? SGNS_OK : SGNS_EIO;
}

// x * log2(x) for integers 0..n-1 from basic IEEE operations only (the same bits on every
// host): log2 x = e + ln(m) log2(e) for x = 2^e m, m in [1, 2), ln(m) = 2 atanh(s) with
// s = (m - 1) / (m + 1) by its odd series to s^39.
void xlog2x_table(int n, double* t) {
  for (int x = 0; x < n; x++) {
    if (x == 0) {
      t[x] = 0.0;
      continue;
    }
    int e = 0;
    while ((x >> (e + 1)) != 0) e++;
    uint64_t bits = (uint64_t)(1023 + e) << 52;
    double p2;
    memcpy(&p2, &bits, 8);
    const double m = (double)x / p2;
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double sum = 0.0;
    for (int k = 39; k >= 1; k -= 2) sum = sum * s2 + 1.0 / (double)k;
    const double ln_m = 2.0 * (s * sum);
    t[x] = (double)x * ((double)e + ln_m * 1.4426950408889634);
  }
}

void build_exp_table(float* t) {  // dsgl.hpp:1557-1562
  for (int i = 0; i < kExpTableSize + 1; i++) {
    const float e = expf(((float)i / (float)kExpTableSize * 2 - 1) * kMaxExp);
    t[i] = e / (e + 1);
  }
}

sgns_status validate(sgns_handle* h, const sgns_options& o) {
  if (o.size < 4 || o.size > kDMax || o.size % 4)
    return fail(h, SGNS_EINVAL, "-size %d: must be a multiple of 4 in [4, %d]", o.size, kDMax);
  if (o.window < 1 || o.window > kWMax - 1)
    return fail(h, SGNS_EINVAL, "-window %d: must be in [1, %d]", o.window, kWMax - 1);
  if (o.negative < 0 || o.negative > kKMax)
    return fail(h, SGNS_EINVAL, "-negative %d: must be in [0, %d]", o.negative, kKMax);
  if (o.iter < 1) return fail(h, SGNS_EINVAL, "-iter %d: must be >= 1", o.iter);
  if (!(o.alpha >= 0.f) || !std::isfinite(o.alpha)) return fail(h, SGNS_EINVAL, "-alpha must be finite and >= 0");
  if (!std::isfinite(o.sample)) return fail(h, SGNS_EINVAL, "-sample must be finite");
  if (o.table_size < 1 || o.table_size > (int64_t)INT32_MAX)
    return fail(h, SGNS_EINVAL, "table size %lld out of range", (long long)o.table_size);
  if (o.storage != SGNS_STORE_FP32 && o.storage != SGNS_STORE_BF16_SR)
    return fail(h, SGNS_EINVAL, "unknown storage %d", o.storage);
  if (o.engine != SGNS_ENGINE_PLAIN && o.engine != SGNS_ENGINE_PERSISTENT)
    return fail(h, SGNS_EINVAL, "unknown engine %d", o.engine);
  if (o.workers < 0 || o.warps_per_cta < 0 || o.warps_per_cta > 8)
    return fail(h, SGNS_EINVAL, "workers/warps_per_cta out of range");
  if (o.mode != SGNS_MODE_HOGWILD && o.mode != SGNS_MODE_REPLAY_EXACT)
    return fail(h, SGNS_EINVAL, "unknown mode %d", o.mode);
  if (o.windows_per_step < 0 || o.windows_per_step > 2)
    return fail(h, SGNS_EINVAL, "windows_per_step %d: 1 or 2 (0 = 2)", o.windows_per_step);
  if (o.forward_tile < 0 || o.forward_tile > 2)
    return fail(h, SGNS_EINVAL, "forward_tile %d: 0 (tuned), 1 or 2", o.forward_tile);
  if (o.forward_tile == 2 && !window_engine_has_tile2(o.size, o.negative))
    return fail(h, SGNS_EINVAL, "forward_tile 2 needs d <= 128 and K <= 5");
  if (o.mode == SGNS_MODE_REPLAY_EXACT && o.workers > 1)
    return fail(h, SGNS_EINVAL, "-mode exact replays one worker; -workers %d asks for more", o.workers);
  return SGNS_OK;
}

TrainParams make_params(sgns_handle* h, int workers) {
  TrainParams p{};
  const sgns_options& o = h->opt;
  p.corpus = h->d_corpus;
  p.words_num = h->n_tokens;
  p.ran = h->d_ran;
  p.table = h->d_table;
  p.exp_table = h->d_exp;
  p.jumps = h->d_jumps;
  p.wih = h->wih;
  p.woh = h->woh;
  p.div_table = make_fastdiv((uint64_t)o.table_size);
  p.div_vm1 = make_fastdiv((uint64_t)(h->V - 1));
  p.div_window = make_fastdiv((uint64_t)o.window);
  p.V = h->V;
  p.d = o.size;
  p.window = o.window;
  p.K = o.negative;
  p.iter = o.iter;
  p.workers = workers;
  p.sample_on = o.sample > 0 ? 1 : 0;
  p.start_alpha = o.alpha;
  p.alpha_denom = (float)((uint64_t)o.iter * h->train_words + 1);  // dsgl.hpp:894
  p.sr_seed = o.seed;
  p.compute_loss = o.compute_loss;
  p.lmax = h->lmax;
  p.storage = o.storage == SGNS_STORE_BF16_SR ? STORE_BF16 : STORE_F32;
  p.fwd_tile = h->tile;
  p.windows = o.windows_per_step == 1 ? 1 : 2;
  p.ctr = h->d_ctr;
  return p;
}

sgns_status reset_counters(sgns_handle* h, int workers) {
  DeviceCounters c{};
  c.alpha = h->opt.alpha;
  c.active = workers;
  *h->h_ctr = c;
  CU(h, cudaMemcpyAsync(h->d_ctr, h->h_ctr, sizeof c, cudaMemcpyHostToDevice, h->stream));
  return SGNS_OK;
}

sgns_status finish_stats(sgns_handle* h, int workers, float ms) {
  CU(h, cudaMemcpyAsync(h->h_ctr, h->d_ctr, sizeof(DeviceCounters), cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  const DeviceCounters& c = *h->h_ctr;
  if (c.status == 1) return fail(h, SGNS_EINVAL, "kernel reported a walk longer than the staged capacity");
  if (c.status != 0) return fail(h, SGNS_EINVAL, "kernel reported an internal inconsistency (code %d)", c.status);
  sgns_stats& s = h->stats;
  s.steps = c.steps;
  s.pairs = c.pairs;
  s.word_count_actual = c.wca;
  s.row_bytes = 2ULL * (c.pairs + c.outputs) * (uint64_t)h->opt.size * elem_bytes(h->opt);
  s.loss = c.loss;
  s.final_alpha = c.alpha;
  s.train_ms = ms;
  s.workers = workers;
  s.warps_per_cta = h->opt.engine == SGNS_ENGINE_PERSISTENT ? h->wpc : 4;
  // single-window steps run the one-lane kernel
  s.forward_tile = h->opt.engine != SGNS_ENGINE_PERSISTENT ? 0 : h->opt.windows_per_step == 1 ? 1 : h->tile;
  s.warps_per_worker = 1;
  s.row_loads = c.row_loads;
  s.row_stores = c.row_stores;
  s.output_rows = c.outputs;
  return SGNS_OK;
}

// largest worker count the persistent engine keeps resident in one wave
sgns_status persistent_shape(sgns_handle* h, int wpc, int* workers) {
  int ctas = 0;
  const sgns_options& o = h->opt;
  CU(h, window_engine_occupancy(o.storage == SGNS_STORE_BF16_SR ? STORE_BF16 : STORE_F32, o.size,
                                o.window, o.negative, h->lmax, wpc, h->tile, &ctas));
  if (ctas < 1)
    return fail(h, SGNS_EINVAL, "a %d-warp CTA does not fit in shared memory (d=%d, walks up to %d)", wpc,
                o.size, h->lmax);
  *workers = ctas * wpc * h->num_sms;
  // At most V/400 workers: with many workers per vertex in flight, hot rows are updated
  // from many stale window copies at once, which costs link-prediction quality (4-block
  // SBM, 100k vertices, every worker in flight: AUC 0.7865 with 266 workers, 0.7842 with
  // 532, 0.7804 with 1064, against the reference trainer's 0.7886).  Large vocabularies
  // keep the full resident count (2.24M vertices: 5596 > 1064).
  const int64_t cap = std::max<int64_t>(1, h->V / 400);
  if (*workers > cap) *workers = (int)cap;
  return SGNS_OK;
}

sgns_status run_persistent(sgns_handle* h, int workers, int wpc, bool use_graph, float* ms_out) {
  TrainParams p = make_params(h, workers);
  if (use_graph) {
    char key[256];
    snprintf(key, sizeof key, "%p/%lld/%d/%d/%p/%p/%d/%d/%d", (void*)h->d_corpus, (long long)h->n_tokens,
             workers, wpc, h->wih, h->woh, h->lmax, h->opt.iter, h->tile);
    if (!h->graph || h->graph_key != key) {
      if (h->graph) cudaGraphExecDestroy(h->graph);
      h->graph = nullptr;
      DeviceCounters c{};
      c.alpha = h->opt.alpha;
      c.active = workers;
      *h->h_ctr = c;
      cudaGraph_t g;
      CU(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e1 = cudaMemcpyAsync(h->d_ctr, h->h_ctr, sizeof c, cudaMemcpyHostToDevice, h->stream);
      cudaError_t e2 = launch_window_engine(p, wpc, h->stream);
      cudaError_t e3 = cudaStreamEndCapture(h->stream, &g);
      if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
        return fail(h, SGNS_ECUDA, "graph capture of the persistent launch failed: %s",
                    cudaGetErrorString(e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3));
      cudaError_t e4 = cudaGraphInstantiate(&h->graph, g, 0);
      cudaGraphDestroy(g);
      if (e4 != cudaSuccess) return fail(h, SGNS_ECUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e4));
      h->graph_key = key;
    }
    // the captured host->device copy reads h_ctr at replay time: refresh it
    DeviceCounters c{};
    c.alpha = h->opt.alpha;
    c.active = workers;
    *h->h_ctr = c;
    CU(h, cudaEventRecord(h->ev0, h->stream));
    CU(h, cudaGraphLaunch(h->graph, h->stream));
    CU(h, cudaEventRecord(h->ev1, h->stream));
  } else {
    sgns_status st = reset_counters(h, workers);
    if (st) return st;
    CU(h, cudaEventRecord(h->ev0, h->stream));
    CU(h, launch_window_engine(p, wpc, h->stream));
    CU(h, cudaEventRecord(h->ev1, h->stream));
  }
  CU(h, cudaEventSynchronize(h->ev1));
  CU(h, cudaEventElapsedTime(ms_out, h->ev0, h->ev1));
  return SGNS_OK;
}

sgns_status run_plain(sgns_handle* h, int workers, float* ms_out) {
  const sgns_options& o = h->opt;
  const size_t stride = plain_worker_bytes(o.size, o.window, o.negative, h->lmax);
  const size_t need = stride * (size_t)workers;
  if (need > h->plain_bytes) {
    dfree(h->plain_scratch);
    h->plain_bytes = 0;
    CU(h, cudaMalloc(&h->plain_scratch, need));
    h->plain_bytes = need;
  }
  TrainParams p = make_params(h, workers);
  p.plain_state = h->plain_scratch;
  p.plain_stride = (int64_t)stride;
  sgns_status st = reset_counters(h, workers);
  if (st) return st;
  CU(h, cudaEventRecord(h->ev0, h->stream));
  CU(h, launch_plain_init(p, h->stream));
  for (int64_t it = 0;; it++) {
    CU(h, launch_plain_step(p, h->stream));
    if (it % 64 == 63) {
      CU(h, cudaMemcpyAsync(&h->h_ctr->active, &h->d_ctr->active, sizeof(int32_t), cudaMemcpyDeviceToHost,
                            h->stream));
      CU(h, cudaStreamSynchronize(h->stream));
      if (h->h_ctr->active <= 0) break;
    }
  }
  CU(h, cudaEventRecord(h->ev1, h->stream));
  CU(h, cudaEventSynchronize(h->ev1));
  CU(h, cudaEventElapsedTime(ms_out, h->ev0, h->ev1));
  return SGNS_OK;
}

// Autotuner: times each CTA shape of the persistent engine on a prefix of the corpus,
// on scratch copies of the tables, and keeps the fastest (pairs per second).
// Autotuner cache: with SGNS_TUNE_CACHE naming a file, the chosen CTA shape is kept per
// device model and problem shape ("key<TAB>warps_per_cta" lines) and reused by later runs.
// The file is only an optimisation: any error reading or writing it is ignored.
std::string tune_key(const sgns_handle* h) {
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, h->opt.device) != cudaSuccess) prop.name[0] = 0;
  char key[384];
  // V enters the key because the default worker count is capped at V/400
  snprintf(key, sizeof key, "%s|sms=%d|d=%d|w=%d|K=%d|storage=%d|lmax=%d|workers=%d|V=%lld", prop.name, h->num_sms,
           h->opt.size, h->opt.window, h->opt.negative, h->opt.storage, h->lmax, h->opt.workers, (long long)h->V);
  for (char* c = key; *c; c++)
    if (*c == '\t' || *c == '\n') *c = ' ';
  return key;
}
// "key<TAB>warps_per_cta<TAB>forward_tile" lines; the last entry for a key wins
bool tune_cache_lookup(const std::string& key, int* wpc, int* tile) {
  const char* path = getenv("SGNS_TUNE_CACHE");
  if (!path || !*path) return false;
  FILE* f = fopen(path, "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (fgets(line, sizeof line, f)) {
    char* tab = strchr(line, '\t');
    if (!tab) continue;
    *tab = 0;
    if (key != line) continue;
    int a = 0, b = 1;
    if (sscanf(tab + 1, "%d\t%d", &a, &b) >= 1 && a >= 1 && a <= 8 && (b == 1 || b == 2)) {
      *wpc = a;
      *tile = b;
      found = true;
    }
  }
  fclose(f);
  return found;
}
void tune_cache_store(const std::string& key, int wpc, int tile) {
  const char* path = getenv("SGNS_TUNE_CACHE");
  if (!path || !*path) return;
  if (FILE* f = fopen(path, "a")) {
    fprintf(f, "%s\t%d\t%d\n", key.c_str(), wpc, tile);
    fclose(f);
  }
}

// The forward tile used when none is given and nothing is tuned: two lanes per input for
// fp32 tables (measured faster there), one for bf16.
int default_tile(const sgns_handle* h) {
  if (!window_engine_has_tile2(h->opt.size, h->opt.negative)) return 1;
  if (h->opt.forward_tile > 0) return h->opt.forward_tile;
  return h->opt.storage == SGNS_STORE_FP32 ? 2 : 1;
}

// Autotuner: times each launch shape of the persistent engine -- warps per CTA (1..8) and,
// where the shape has it, the forward tile (1 or 2 lanes per input) -- on a prefix of the
// corpus, on scratch copies of the tables, and keeps the fastest (pairs per second).
// Autotuner cache: with SGNS_TUNE_CACHE naming a file, the choice is kept per device model
// and problem shape and reused by later runs.  The file is only an optimisation: any error
// reading or writing it is ignored.
sgns_status autotune(sgns_handle* h) {
  const sgns_options& o = h->opt;
  const std::string key = tune_key(h);
  const bool tile2 = window_engine_has_tile2(o.size, o.negative);
  if (o.warps_per_cta <= 0) {
    int cached = 0, ctile = 1;
    if (tune_cache_lookup(key, &cached, &ctile)) {
      if (!tile2) ctile = 1;
      if (o.forward_tile > 0) ctile = o.forward_tile;
      h->tile = ctile;
      int workers = o.workers;
      if (!workers && persistent_shape(h, cached, &workers) != SGNS_OK) workers = 0;
      if (workers > 0) {
        h->wpc = cached;
        h->workers = workers;
        h->tuned = true;
        if (o.debug > 0)
          fprintf(stderr, "sgns: persistent engine shape from the tuning cache: %d warps/CTA, tile %d\n", cached,
                  ctile);
        return SGNS_OK;
      }
    }
  }
  if (o.warps_per_cta > 0) {  // a given CTA shape: only the tile may be left to choose
    h->wpc = o.warps_per_cta;
    h->tile = default_tile(h);
    h->workers = o.workers;
    if (!h->workers) {
      sgns_status st = persistent_shape(h, h->wpc, &h->workers);
      if (st) return st;
    }
    h->tuned = true;
    return SGNS_OK;
  }
  // the trial launches train scratch copies of the tables; the handle's own pointers,
  // corpus length and pass count are put back on every path out of the search
  const size_t tbytes = (size_t)h->V * o.size * elem_bytes(o);
  void *wih_s = nullptr, *woh_s = nullptr;
  void *wih0 = h->wih, *woh0 = h->woh;
  const int64_t n0 = h->n_tokens;
  const int iter0 = h->opt.iter;
  auto restore = [&]() {
    cudaStreamSynchronize(h->stream);
    h->wih = wih0;
    h->woh = woh0;
    h->n_tokens = n0;
    h->opt.iter = iter0;
    dfree(wih_s);
    dfree(woh_s);
  };
  double best = -1.0;
  int best_wpc = 1, best_workers = 0, best_tile = default_tile(h);
  sgns_status st = SGNS_OK;
  cudaError_t e;
  if ((e = cudaMalloc(&wih_s, tbytes)) != cudaSuccess || (e = cudaMalloc(&woh_s, tbytes)) != cudaSuccess) {
    // no room for scratch tables: take, untimed, the shape with the most resident
    // workers (warps per SM bound this latency-bound kernel); ties go to the wider CTA
    restore();
    cudaGetLastError();
    h->tile = best_tile;
    for (int wpc = 1; wpc <= 8; wpc++) {
      int workers = 0;
      if (persistent_shape(h, wpc, &workers) != SGNS_OK) continue;
      if (workers >= best_workers) {
        best_wpc = wpc;
        best_workers = workers;
      }
    }
    if (best_workers == 0) return fail(h, SGNS_EINVAL, "no persistent-engine shape fits this configuration");
    if (o.workers > 0) best_workers = o.workers;
    h->wpc = best_wpc;
    h->workers = best_workers;
    h->tuned = true;
    if (o.debug > 0)
      fprintf(stderr, "sgns: no memory for autotuning; persistent engine at %d warps/CTA\n", best_wpc);
    return SGNS_OK;
  }
  if ((e = cudaMemcpyAsync(wih_s, h->wih, tbytes, cudaMemcpyDeviceToDevice, h->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(woh_s, h->woh, tbytes, cudaMemcpyDeviceToDevice, h->stream)) != cudaSuccess) {
    restore();
    return fail(h, SGNS_ECUDA, "autotuner table copies: %s", cudaGetErrorString(e));
  }
  h->wih = wih_s;
  h->woh = woh_s;
  h->opt.iter = 1;
  const int tile_lo = o.forward_tile > 0 ? o.forward_tile : 1;
  const int tile_hi = o.forward_tile > 0 ? o.forward_tile : (tile2 ? 2 : 1);
  for (int tile = tile_lo; tile <= tile_hi && !st; tile++) {
    h->tile = tile;
    for (int wpc = 1; wpc <= 8; wpc++) {
      int workers = 0;
      st = persistent_shape(h, wpc, &workers);
      if (st) {
        st = SGNS_OK;
        continue;
      }
      if (o.workers > 0) workers = o.workers;
      // a prefix long enough to give every worker a few hundred steps
      h->n_tokens = std::min<int64_t>(n0, (int64_t)workers * 2000);
      float ms = 0.f;
      st = run_persistent(h, workers, wpc, false, &ms);
      if (st) break;
      if ((e = cudaMemcpy(h->h_ctr, h->d_ctr, sizeof(DeviceCounters), cudaMemcpyDeviceToHost)) != cudaSuccess) {
        st = fail(h, SGNS_ECUDA, "autotuner counters: %s", cudaGetErrorString(e));
        break;
      }
      const double rate = ms > 0 ? (double)h->h_ctr->pairs / ms : 0.0;
      if (rate > best) {
        best = rate;
        best_wpc = wpc;
        best_workers = workers;
        best_tile = tile;
      }
    }
  }
  restore();
  if (st) return st;
  if (best_workers == 0) return fail(h, SGNS_EINVAL, "no persistent-engine shape fits this configuration");
  h->wpc = best_wpc;
  h->workers = best_workers;
  h->tile = best_tile;
  h->tuned = true;
  tune_cache_store(key, best_wpc, best_tile);
  if (o.debug > 0)
    fprintf(stderr, "sgns: autotuned persistent engine: %d warps/CTA, tile %d, %d workers\n", h->wpc, h->tile,
            h->workers);
  return SGNS_OK;
}

// Scratch of the kernel-level entry points, one growable buffer per device.
struct DeviceScratch {
  std::mutex mx;
  void* buf = nullptr;
  size_t bytes = 0;
  float* exp = nullptr;
  sgns_status ensure(size_t need) {
    if (!exp) {
      float et[kExpTableSize + 1];
      build_exp_table(et);
      if (cudaMalloc(&exp, sizeof et) != cudaSuccess) return fail(nullptr, SGNS_ENOMEM, "cudaMalloc");
      if (cudaMemcpy(exp, et, sizeof et, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(nullptr, SGNS_ECUDA, "cudaMemcpy");
    }
    if (need <= bytes) return SGNS_OK;
    if (buf) {
      cudaDeviceSynchronize();
      cudaFree(buf);
    }
    buf = nullptr;
    bytes = 0;
    if (cudaMalloc(&buf, need) != cudaSuccess) return fail(nullptr, SGNS_ENOMEM, "scratch of %zu bytes", need);
    bytes = need;
    return SGNS_OK;
  }
};

DeviceScratch* device_scratch() {
  static DeviceScratch table[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  return &table[dev];
}

}  // namespace

namespace sgns {
void host_exp_table(float* t) { build_exp_table(t); }
int report_error(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_create_err = buf;
  // as in fail(): a failed runtime call also left the per-thread last error set, which the
  // next launcher would otherwise read back as its own failure
  if (status == SGNS_ECUDA || status == SGNS_ENOMEM) cudaGetLastError();
  return status;
}
}  // namespace sgns

// ===================================================================================
extern "C" {

// Host set-up of sgns_set_vocab without a device (declared in sgns_internal.h, not in the
// public header): the CPU tests compare it with the oracle.
int32_t sgns_internal_host_vocab(const int32_t* counts, int64_t V, float sample, int64_t table_size, int32_t threads,
                                 uint32_t* order, int32_t* table, float* ran, float* exp_table,
                                 uint64_t* train_words) {
  if (!counts || V < 1 || V > (int64_t)INT32_MAX || table_size < 1 || table_size > (int64_t)INT32_MAX)
    return SGNS_EINVAL;
  for (int64_t i = 0; i < V; i++)
    if (counts[i] < 0) return SGNS_EINVAL;
  HostVocab hv;
  build_host_vocab(counts, V, sample, table_size, threads, hv);
  if (order) std::memcpy(order, hv.order.data(), sizeof(uint32_t) * V);
  if (table) std::memcpy(table, hv.table.data(), sizeof(int32_t) * table_size);
  if (ran) std::memcpy(ran, hv.ran.data(), sizeof(float) * V);
  if (exp_table) build_exp_table(exp_table);
  if (train_words) *train_words = hv.train_words;
  return SGNS_OK;
}

// The embedding writer of sgns_save_text on host arrays (declared in sgns_internal.h, not
// in the public header): the CPU tests compare its bytes with the reference's files.
int32_t sgns_internal_write_embedding(const uint32_t* order, const float* w, int64_t V, int32_t d, int32_t binary,
                                      const char* path) {
  if (!order || !w || !path || V < 0 || d < 1) return SGNS_EINVAL;
  return write_embedding(order, w, V, d, binary != 0, path);
}

// The walker's x * log2(x) table as sgns_info_walks uploads it; exported for the CPU tests.
void sgns_internal_xlog2x_table(int32_t n, double* t) { xlog2x_table(n, t); }

// The stochastic-rounding bits of the kernels' write-backs (host copy of sr_bits4).
void sgns_internal_sr_bits4(int64_t n, const uint64_t* ev, const uint32_t* row, const uint32_t* col4, uint64_t* bits) {
  for (int64_t i = 0; i < n; i++) bits[i] = sr_bits4(ev[i], row[i], col4[i]);
}

void sgns_default_options(sgns_options* o) {
  std::memset(o, 0, sizeof *o);
  o->size = 100;  // dsgl.hpp:70
  o->window = 5;  // dsgl.hpp:69
  o->negative = 5;
  o->batch_size = 11;
  o->sample = 1e-3f;  // dsgl.hpp:75
  o->alpha = 0.1f;
  o->min_count = 5;
  o->iter = 5;
  o->threads = 12;
  o->debug = 2;
  o->binary = 0;
  o->storage = SGNS_STORE_FP32;
  o->engine = SGNS_ENGINE_PERSISTENT;
  o->table_size = 100000000;  // dsgl.hpp:82
  o->seed = 0x5EEDULL;
  o->windows_per_step = 2;
}

sgns_status sgns_options_from_args(sgns_options* o, int argc, const char* const* argv) {
  auto pos = [&](const char* f) {  // ArgPos, dsgl.hpp:1429-1441
    for (int a = 1; a < argc; a++)
      if (!std::strcmp(f, argv[a])) return a;
    return -1;
  };
  struct IntFlag {
    const char* name;
    int32_t* dst;
  } ints[] = {{"-size", &o->size},         {"-debug", &o->debug},         {"-binary", &o->binary},
              {"-window", &o->window},     {"-negative", &o->negative},   {"-threads", &o->threads},
              {"-iter", &o->iter},         {"-min-count", &o->min_count}, {"-batch-size", &o->batch_size},
              {"-workers", &o->workers},   {"-warps-per-cta", &o->warps_per_cta},
              {"-forward-tile", &o->forward_tile}, {"-windows-per-step", &o->windows_per_step},
              {"-device", &o->device},
              {"-loss", &o->compute_loss}};
  for (auto& f : ints) {
    int i = pos(f.name);
    if (i > 0) {
      if (i + 1 >= argc) return fail(nullptr, SGNS_EINVAL, "flag %s needs a value", f.name);
      *f.dst = atoi(argv[i + 1]);
    }
  }
  int i;
  if ((i = pos("-alpha")) > 0) {
    if (i + 1 >= argc) return fail(nullptr, SGNS_EINVAL, "flag -alpha needs a value");
    o->alpha = (float)atof(argv[i + 1]);
  }
  if ((i = pos("-sample")) > 0) {
    if (i + 1 >= argc) return fail(nullptr, SGNS_EINVAL, "flag -sample needs a value");
    o->sample = (float)atof(argv[i + 1]);
  }
  if ((i = pos("-table-size")) > 0) {
    if (i + 1 >= argc) return fail(nullptr, SGNS_EINVAL, "flag -table-size needs a value");
    o->table_size = atoll(argv[i + 1]);
  }
  if ((i = pos("-seed")) > 0) {
    if (i + 1 >= argc) return fail(nullptr, SGNS_EINVAL, "flag -seed needs a value");
    o->seed = strtoull(argv[i + 1], nullptr, 0);
  }
  if ((i = pos("-storage")) > 0) {
    if (i + 1 >= argc) return fail(nullptr, SGNS_EINVAL, "flag -storage needs a value");
    if (!std::strcmp(argv[i + 1], "fp32")) o->storage = SGNS_STORE_FP32;
    else if (!std::strcmp(argv[i + 1], "bf16")) o->storage = SGNS_STORE_BF16_SR;
    else return fail(nullptr, SGNS_EINVAL, "-storage %s: expected fp32 or bf16", argv[i + 1]);
  }
  if ((i = pos("-mode")) > 0) {
    if (i + 1 >= argc) return fail(nullptr, SGNS_EINVAL, "flag -mode needs a value");
    if (!std::strcmp(argv[i + 1], "hogwild")) o->mode = SGNS_MODE_HOGWILD;
    else if (!std::strcmp(argv[i + 1], "exact")) o->mode = SGNS_MODE_REPLAY_EXACT;
    else return fail(nullptr, SGNS_EINVAL, "-mode %s: expected hogwild or exact", argv[i + 1]);
  }
  if ((i = pos("-engine")) > 0) {
    if (i + 1 >= argc) return fail(nullptr, SGNS_EINVAL, "flag -engine needs a value");
    if (!std::strcmp(argv[i + 1], "plain")) o->engine = SGNS_ENGINE_PLAIN;
    else if (!std::strcmp(argv[i + 1], "persistent")) o->engine = SGNS_ENGINE_PERSISTENT;
    else return fail(nullptr, SGNS_EINVAL, "-engine %s: expected plain or persistent", argv[i + 1]);
  }
  return SGNS_OK;
}

sgns_status sgns_create(const sgns_options* opt, sgns_handle** out) {
  if (!opt || !out) return fail(nullptr, SGNS_EINVAL, "null argument");
  *out = nullptr;
  sgns_status st = validate(nullptr, *opt);
  if (st) return st;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    return fail(nullptr, SGNS_ECUDA, "no CUDA device available");
  if (opt->device < 0 || opt->device >= ndev) return fail(nullptr, SGNS_EINVAL, "device %d not present", opt->device);
  if (cudaSetDevice(opt->device) != cudaSuccess) return fail(nullptr, SGNS_ECUDA, "cudaSetDevice failed");
  sgns_handle* h = new (std::nothrow) sgns_handle();
  if (!h) return fail(nullptr, SGNS_ENOMEM, "out of host memory");
  h->opt = *opt;
  auto bail = [&](const char* what, cudaError_t e) {
    fail(nullptr, SGNS_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    sgns_destroy(h);
    return SGNS_ECUDA;
  };
  cudaError_t e;
  if ((e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, opt->device)) != cudaSuccess)
    return bail("cudaDeviceGetAttribute", e);
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail("cudaStreamCreate", e);
  if ((e = cudaEventCreate(&h->ev0)) != cudaSuccess || (e = cudaEventCreate(&h->ev1)) != cudaSuccess)
    return bail("cudaEventCreate", e);
  if ((e = cudaMalloc(&h->d_ctr, sizeof(DeviceCounters))) != cudaSuccess) return bail("cudaMalloc", e);
  if ((e = cudaMallocHost(&h->h_ctr, sizeof(DeviceCounters))) != cudaSuccess) return bail("cudaMallocHost", e);
  if ((e = cudaMalloc(&h->d_flags, 4 * sizeof(int32_t))) != cudaSuccess) return bail("cudaMalloc", e);
  if ((e = cudaMallocHost(&h->h_flags, 4 * sizeof(int32_t))) != cudaSuccess) return bail("cudaMallocHost", e);
  if ((e = cudaMalloc(&h->d_exp, sizeof(float) * (kExpTableSize + 1))) != cudaSuccess) return bail("cudaMalloc", e);
  if ((e = cudaMalloc(&h->d_jumps, sizeof(LcgJumps))) != cudaSuccess) return bail("cudaMalloc", e);
  float et[kExpTableSize + 1];
  build_exp_table(et);
  LcgJumps J;
  make_lcg_jumps(&J);
  if ((e = cudaMemcpy(h->d_exp, et, sizeof et, cudaMemcpyHostToDevice)) != cudaSuccess) return bail("cudaMemcpy", e);
  if ((e = cudaMemcpy(h->d_jumps, &J, sizeof J, cudaMemcpyHostToDevice)) != cudaSuccess) return bail("cudaMemcpy", e);
  *out = h;
  return SGNS_OK;
}

void sgns_destroy(sgns_handle* h) {
  if (!h) return;
  cudaSetDevice(h->opt.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  dfree(h->wih);
  dfree(h->woh);
  dfree(h->d_row_of);
  dfree(h->d_ran);
  dfree(h->d_table);
  dfree(h->d_exp);
  dfree(h->d_jumps);
  dfree(h->d_ctr);
  dfree(h->d_flags);
  dfree(h->d_ids);
  dfree(h->d_corpus);
  dfree(h->plain_scratch);
  if (h->h_ctr) cudaFreeHost(h->h_ctr);
  if (h->h_flags) cudaFreeHost(h->h_flags);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

const char* sgns_last_error(const sgns_handle* h) {
  if (h) return h->err.c_str();
  return g_create_err.c_str();
}

sgns_status sgns_set_vocab(sgns_handle* h, const int32_t* counts, int64_t V) {
  NvtxRange r_("sgns_set_vocab");
  if (!h || !counts) return fail(h, SGNS_EINVAL, "null argument");
  if (V < 2 || V > (int64_t)INT32_MAX) return fail(h, SGNS_EINVAL, "vocabulary size %lld out of range", (long long)V);
  CU(h, cudaSetDevice(h->opt.device));
  for (int64_t i = 0; i < V; i++)
    if (counts[i] < 0) return fail(h, SGNS_EINVAL, "negative count at vertex %lld", (long long)i);
  HostVocab hv;
  build_host_vocab(counts, V, h->opt.sample, h->opt.table_size, h->opt.threads, hv);
  drop_vocab(h);
  h->order = std::move(hv.order);
  h->row_of = std::move(hv.row_of);
  h->cn_sorted = std::move(hv.cn_sorted);
  const std::vector<int32_t>& table = hv.table;
  const std::vector<float>& ran = hv.ran;
  const uint64_t tw = hv.train_words;
  // a failure below leaves the handle without a vocabulary (as before the first call)
  const size_t tbytes = (size_t)V * h->opt.size * elem_bytes(h->opt);
  cudaError_t e;
  if ((e = cudaMalloc(&h->wih, tbytes)) != cudaSuccess || (e = cudaMalloc(&h->woh, tbytes)) != cudaSuccess) {
    drop_vocab(h);
    cudaGetLastError();
    return fail(h, SGNS_ENOMEM, "embedding tables (2 x %zu bytes): %s", tbytes, cudaGetErrorString(e));
  }
  if ((e = cudaMalloc(&h->d_row_of, sizeof(int32_t) * V)) != cudaSuccess ||
      (e = cudaMalloc(&h->d_ran, sizeof(float) * V)) != cudaSuccess ||
      (e = cudaMalloc(&h->d_table, sizeof(int32_t) * table.size())) != cudaSuccess) {
    drop_vocab(h);
    cudaGetLastError();
    return fail(h, SGNS_ENOMEM, "vocabulary tables: %s", cudaGetErrorString(e));
  }
  if ((e = cudaMemcpy(h->d_row_of, h->row_of.data(), sizeof(int32_t) * V, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(h->d_ran, ran.data(), sizeof(float) * V, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(h->d_table, table.data(), sizeof(int32_t) * table.size(), cudaMemcpyHostToDevice)) !=
          cudaSuccess) {
    drop_vocab(h);
    return fail(h, SGNS_ECUDA, "vocabulary upload: %s", cudaGetErrorString(e));
  }
  h->V = V;
  h->train_words = tw;
  const sgns_status rs = sgns_reset_model(h);
  if (rs) drop_vocab(h);
  return rs;
}

sgns_status sgns_reset_model(sgns_handle* h) {
  if (!h) return fail(h, SGNS_EINVAL, "null handle");
  if (!h->wih) return fail(h, SGNS_ESTATE, "sgns_set_vocab has not been called");
  CU(h, cudaSetDevice(h->opt.device));
  const size_t tbytes = (size_t)h->V * h->opt.size * elem_bytes(h->opt);
  CU(h, launch_init_wih(h->wih, h->opt.storage == SGNS_STORE_BF16_SR ? STORE_BF16 : STORE_F32, h->V,
                        h->opt.size, h->d_jumps, h->stream));
  CU(h, cudaMemsetAsync(h->woh, 0, tbytes, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  return SGNS_OK;
}

// Maps n ids (device memory, or pinned host memory mapped for this device) to sorted rows
// (validating them), finds the longest walk.
sgns_status map_uploaded_corpus(sgns_handle* h, const int32_t* ids, int64_t n) {
  h->n_tokens = n;
  CU(h, cudaMemsetAsync(h->d_flags, 0, 4 * sizeof(int32_t), h->stream));
  if (n > 0) {
    CU(h, launch_map_corpus(ids, h->d_row_of, h->d_corpus, n, h->V, h->d_flags, h->stream));
    CU(h, launch_max_walk(h->d_corpus, n, h->d_flags + 1, h->stream));
  }
  CU(h, cudaMemcpyAsync(h->h_flags, h->d_flags, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  if (h->h_flags[0]) {
    h->n_tokens = 0;
    return fail(h, SGNS_EINVAL, "corpus holds a token outside [0, %lld) that is not the -1 separator", (long long)h->V);
  }
  const int lmax = std::max(2, (int)h->h_flags[1]);
  if (lmax != h->lmax) h->tuned = false;
  h->lmax = lmax;
  return SGNS_OK;
}

sgns_status ensure_corpus_capacity(sgns_handle* h, int64_t n) {
  if (n <= h->corpus_cap) return SGNS_OK;
  dfree(h->d_ids);
  dfree(h->d_corpus);
  h->corpus_cap = 0;
  cudaError_t e;
  if ((e = cudaMalloc(&h->d_ids, sizeof(int32_t) * n)) != cudaSuccess ||
      (e = cudaMalloc(&h->d_corpus, sizeof(int32_t) * n)) != cudaSuccess)
    return fail(h, SGNS_ENOMEM, "corpus of %lld tokens: %s", (long long)n, cudaGetErrorString(e));
  h->corpus_cap = n;
  return SGNS_OK;
}

sgns_status sgns_upload_corpus(sgns_handle* h, const int32_t* tokens, int64_t n) {
  NvtxRange r_("sgns_upload_corpus");
  if (!h || (!tokens && n > 0) || n < 0) return fail(h, SGNS_EINVAL, "bad corpus arguments");
  if (!h->wih) return fail(h, SGNS_ESTATE, "sgns_set_vocab has not been called");
  CU(h, cudaSetDevice(h->opt.device));
  sgns_status st = ensure_corpus_capacity(h, n);
  if (st) return st;
  // Pinned host memory mapped into this device's address space is read in place by the
  // mapping kernel (the ids cross the host link once); anything else is copied first.
  cudaPointerAttributes a{};
  const bool mapped = n > 0 && cudaPointerGetAttributes(&a, tokens) == cudaSuccess &&
                      a.type == cudaMemoryTypeHost && a.devicePointer != nullptr && a.device == h->opt.device;
  cudaGetLastError();  // a failed attribute query leaves no error behind
  if (mapped) return map_uploaded_corpus(h, static_cast<const int32_t*>(a.devicePointer), n);
  if (n > 0) CU(h, cudaMemcpyAsync(h->d_ids, tokens, sizeof(int32_t) * n, cudaMemcpyHostToDevice, h->stream));
  return map_uploaded_corpus(h, h->d_ids, n);
}

sgns_status sgns_train(sgns_handle* h) {
  NvtxRange r_("sgns_train");
  if (!h) return fail(h, SGNS_EINVAL, "null handle");
  if (!h->wih) return fail(h, SGNS_ESTATE, "sgns_set_vocab has not been called");
  CU(h, cudaSetDevice(h->opt.device));
  float ms = 0.f;
  int workers = 0;
  sgns_status st;
  const bool exact = h->opt.mode == SGNS_MODE_REPLAY_EXACT;
  if (h->opt.engine == SGNS_ENGINE_PERSISTENT) {
    if (exact) {  // one worker in a one-warp CTA: nothing to tune
      workers = 1;
      h->wpc = h->opt.warps_per_cta > 0 ? h->opt.warps_per_cta : 1;
      h->tile = default_tile(h);
      st = run_persistent(h, 1, h->wpc, true, &ms);
      if (st) return st;
      return finish_stats(h, workers, ms);
    }
    if (!h->tuned) {
      st = autotune(h);
      if (st) return st;
    }
    workers = h->opt.workers > 0 ? h->opt.workers : h->workers;
    st = run_persistent(h, workers, h->wpc, true, &ms);
  } else if (exact) {
    workers = 1;
    st = run_plain(h, 1, &ms);
  } else {
    // Default worker count.  Each worker of the reference policy holds snapshots of about
    // max(len1,len2)*K negative rows and two walks' rows and writes them back over the
    // tables; with many workers in flight those write-backs erase each other's updates.
    // Link-prediction AUC on 4-block SBMs (10% holdout): at 100k vertices 0.795 with 152
    // workers, 0.60 with 304, 0.50 with 608 (GB300); at 1.1M vertices 0.708 with 1571
    // (GB300), and with every worker in flight at once on the host (the same policy run
    // step by step round-robin) 0.717 with 1571 and 0.783 with 785.  V / 1400 workers.
    workers = h->opt.workers > 0 ? h->opt.workers
                                 : (int)std::max<int64_t>(1, std::min<int64_t>(h->num_sms * 16, h->V / 1400));
    const size_t stride = plain_worker_bytes(h->opt.size, h->opt.window, h->opt.negative, h->lmax);
    const size_t budget = (size_t)8 << 30;  // HBM set aside for per-worker buffers
    if (h->opt.workers == 0 && stride * (size_t)workers > budget) workers = std::max<int>(1, (int)(budget / stride));
    st = run_plain(h, workers, &ms);
  }
  if (st) return st;
  return finish_stats(h, workers, ms);
}

sgns_status sgns_train_corpus(sgns_handle* h, const int32_t* tokens, int64_t n) {
  sgns_status st = sgns_upload_corpus(h, tokens, n);
  if (st) return st;
  return sgns_train(h);
}

sgns_status sgns_get_stats(const sgns_handle* h, sgns_stats* out) {
  if (!h || !out) return SGNS_EINVAL;
  *out = h->stats;
  return SGNS_OK;
}

int64_t sgns_vocab_size(const sgns_handle* h) { return h ? h->V : 0; }

sgns_status sgns_get_order(const sgns_handle* h, uint32_t* out) {
  if (!h || !out) return SGNS_EINVAL;
  if (!h->V) return SGNS_ESTATE;
  std::memcpy(out, h->order.data(), sizeof(uint32_t) * h->V);
  return SGNS_OK;
}

sgns_status sgns_get_embeddings(sgns_handle* h, int32_t which, float* out) {
  if (!h || !out || (which != 0 && which != 1)) return fail(h, SGNS_EINVAL, "bad arguments");
  if (!h->wih) return fail(h, SGNS_ESTATE, "sgns_set_vocab has not been called");
  CU(h, cudaSetDevice(h->opt.device));
  const size_t n = (size_t)h->V * h->opt.size;
  const void* src = which ? h->woh : h->wih;
  if (h->opt.storage == SGNS_STORE_BF16_SR) {
    // Pinned host memory mapped into this device's address space (16-byte aligned) is
    // written in place by the widening kernel: the fp32 rows cross the host link once,
    // with no staging buffer and no copy.
    cudaPointerAttributes a{};
    const bool mapped = cudaPointerGetAttributes(&a, out) == cudaSuccess && a.type == cudaMemoryTypeHost &&
                        a.devicePointer != nullptr && a.device == h->opt.device &&
                        (reinterpret_cast<uintptr_t>(a.devicePointer) & 15) == 0;
    cudaGetLastError();  // a failed attribute query leaves no error behind
    if (mapped) {
      cudaError_t e = launch_widen_bf16(src, static_cast<float*>(a.devicePointer), (int64_t)n, h->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
      if (e != cudaSuccess) return fail(h, SGNS_ECUDA, "reading embeddings: %s", cudaGetErrorString(e));
      return SGNS_OK;
    }
    // otherwise widened on the device in chunks through a small staging buffer, so the
    // host receives fp32 rows directly (no host-side conversion of V*d elements)
    const size_t chunk = std::min<size_t>(n, (size_t)8 << 20);
    float* stage = nullptr;
    CU(h, cudaMalloc(&stage, chunk * 4));
    cudaError_t e = cudaSuccess;
    for (size_t i = 0; i < n && e == cudaSuccess; i += chunk) {
      const size_t m = std::min(chunk, n - i);
      e = launch_widen_bf16(static_cast<const uint16_t*>(src) + i, stage, (int64_t)m, h->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(out + i, stage, m * 4, cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(stage);
    if (e != cudaSuccess) return fail(h, SGNS_ECUDA, "reading embeddings: %s", cudaGetErrorString(e));
  } else {
    CU(h, cudaMemcpyAsync(out, src, n * 4, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
  }
  return SGNS_OK;
}

sgns_status sgns_set_embeddings(sgns_handle* h, int32_t which, const float* in) {
  if (!h || !in || (which != 0 && which != 1)) return fail(h, SGNS_EINVAL, "bad arguments");
  if (!h->wih) return fail(h, SGNS_ESTATE, "sgns_set_vocab has not been called");
  CU(h, cudaSetDevice(h->opt.device));
  const size_t n = (size_t)h->V * h->opt.size;
  void* dst = which ? h->woh : h->wih;
  if (h->opt.storage == SGNS_STORE_BF16_SR) {
    std::vector<uint16_t> tmp(n);
    for (size_t i = 0; i < n; i++) {  // round to nearest even
      uint32_t u;
      std::memcpy(&u, &in[i], 4);
      if ((u & 0x7F800000u) == 0x7F800000u) tmp[i] = (uint16_t)((u >> 16) | ((u & 0xFFFF) ? 0x40 : 0));
      else tmp[i] = (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
    }
    CU(h, cudaMemcpy(dst, tmp.data(), n * 2, cudaMemcpyHostToDevice));
  } else {
    CU(h, cudaMemcpy(dst, in, n * 4, cudaMemcpyHostToDevice));
  }
  return SGNS_OK;
}

sgns_status sgns_device_tables(sgns_handle* h, void** wih, void** woh) {
  if (!h) return SGNS_EINVAL;
  if (!h->wih) return fail(h, SGNS_ESTATE, "sgns_set_vocab has not been called");
  if (wih) *wih = h->wih;
  if (woh) *woh = h->woh;
  return SGNS_OK;
}

sgns_status sgns_sync_rows(const sgns_handle* h, uint64_t seed, uint64_t round, int32_t full, int32_t* rows,
                           int64_t cap, int64_t* n_rows) {
  if (!h || !n_rows || cap < 0 || (cap > 0 && !rows)) return fail(nullptr, SGNS_EINVAL, "bad sync-row arguments");
  if (h->V == 0) return fail(nullptr, SGNS_ESTATE, "sgns_set_vocab has not been called");
  const int32_t st = sgns_internal_sync_rows(h->cn_sorted.data(), h->V, seed, round, full, rows, cap, n_rows);
  if (st) return fail(nullptr, SGNS_EINVAL, "%lld sync rows, capacity %lld", (long long)*n_rows, (long long)cap);
  return SGNS_OK;
}

// The row draw of sgns_sync_rows from the count-sorted counts; exported for the CPU tests.
int32_t sgns_internal_sync_rows(const int32_t* cn_sorted, int64_t V, uint64_t seed, uint64_t round, int32_t full,
                                int32_t* rows, int64_t cap, int64_t* n_rows) {
  std::vector<int32_t> out;
  if (full) {
    out.resize(V);
    for (int64_t r = 0; r < V; r++) out[r] = (int32_t)r;
  } else {
    // block starts: row 0 and every row whose count differs from the previous row's
    std::vector<int64_t> starts{0};
    for (int64_t r = 1; r < V; r++)
      if (cn_sorted[r] != cn_sorted[r - 1]) starts.push_back(r);
    // one row per block [starts[j-1], starts[j]) for j = 1..: the last block is not drawn
    const uint64_t base = mix64(seed ^ (round * 0x9E3779B97F4A7C15ULL));
    for (size_t j = 1; j < starts.size(); j++) {
      const uint64_t r = mix64(base + (uint64_t)j * 0x9E3779B97F4A7C15ULL);
      const uint64_t len = (uint64_t)(starts[j] - starts[j - 1]);
      out.push_back((int32_t)(starts[j - 1] + (int64_t)(((r >> 32) * len) >> 32)));
    }
  }
  *n_rows = (int64_t)out.size();
  if ((int64_t)out.size() > cap) return SGNS_EINVAL;
  if (!out.empty()) memcpy(rows, out.data(), sizeof(int32_t) * out.size());
  return SGNS_OK;
}

sgns_status sgns_gather_rows(sgns_handle* h, int32_t which, const int32_t* rows, int64_t n, float* buf) {
  if (!h || (which != 0 && which != 1) || n < 0 || (n > 0 && (!rows || !buf)))
    return fail(h, SGNS_EINVAL, "bad gather arguments");
  if (!h->wih) return fail(h, SGNS_ESTATE, "sgns_set_vocab has not been called");
  CU(h, cudaSetDevice(h->opt.device));
  CU(h, launch_gather_rows(which ? h->woh : h->wih, h->opt.storage == SGNS_STORE_BF16_SR ? STORE_BF16 : STORE_F32,
                           h->opt.size, rows, n, buf, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  return SGNS_OK;
}

sgns_status sgns_scatter_rows(sgns_handle* h, int32_t which, const int32_t* rows, int64_t n, const float* buf,
                              float divisor) {
  if (!h || (which != 0 && which != 1) || n < 0 || (n > 0 && (!rows || !buf)) || !(divisor > 0))
    return fail(h, SGNS_EINVAL, "bad scatter arguments");
  if (!h->wih) return fail(h, SGNS_ESTATE, "sgns_set_vocab has not been called");
  CU(h, cudaSetDevice(h->opt.device));
  CU(h, launch_scatter_rows(which ? h->woh : h->wih, h->opt.storage == SGNS_STORE_BF16_SR ? STORE_BF16 : STORE_F32,
                            h->opt.size, rows, n, buf, divisor, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  return SGNS_OK;
}

sgns_status sgns_save_text(sgns_handle* h, const char* path) {
  NvtxRange r_("sgns_save_text");
  if (!h || !path) return fail(h, SGNS_EINVAL, "bad arguments");
  if (!h->wih) return fail(h, SGNS_ESTATE, "sgns_set_vocab has not been called");
  const int64_t V = h->V;
  const int d = h->opt.size;
  std::vector<float> w((size_t)V * d);
  sgns_status st = sgns_get_embeddings(h, 0, w.data());
  if (st) return st;
  st = write_embedding(h->order.data(), w.data(), V, d, h->opt.binary != 0, path);
  if (st == SGNS_EIO) return fail(h, SGNS_EIO, "cannot write %s", path);
  return st;
}

namespace {
// Parses n bytes of walk text in device memory into tokens (capacity cap); see
// sgns_parse_walks.  h may be null (kernel-level call).
sgns_status parse_walks(sgns_handle* h, const uint8_t* bytes, int64_t n, int32_t* tokens, int64_t cap,
                        int64_t* n_tokens, int64_t* max_id, cudaStream_t s) {
  DeviceScratch* ds = device_scratch();
  if (!ds) return fail(h, SGNS_ECUDA, "no current CUDA device");
  std::lock_guard<std::mutex> g(ds->mx);
  sgns_status st = ds->ensure(ingest_scratch_bytes(n));
  if (st) return st;
  unsigned long long cnt = 0;
  long long err = 0, mx = -1;
  cudaError_t e = launch_ingest_count(bytes, n, ds->buf, &cnt, &err, s);
  if (e != cudaSuccess) return fail(h, SGNS_ECUDA, "walk parse: %s", cudaGetErrorString(e));
  if (err != 0x7FFFFFFFFFFFFFFFLL) {
    uint8_t c = 0;
    cudaMemcpy(&c, bytes + err, 1, cudaMemcpyDeviceToHost);
    return fail(h, SGNS_EINVAL, "unexpected byte 0x%02x at offset %lld of the walk text", c, err);
  }
  *n_tokens = (int64_t)cnt;
  *max_id = -1;
  if ((int64_t)cnt > cap)
    return fail(h, SGNS_EINVAL, "walk text yields %llu tokens, capacity %lld", cnt, (long long)cap);
  if (cnt == 0) return SGNS_OK;
  e = launch_ingest_emit(bytes, n, ds->buf, tokens, &err, &mx, s);
  if (e != cudaSuccess) return fail(h, SGNS_ECUDA, "walk parse: %s", cudaGetErrorString(e));
  if (err != 0x7FFFFFFFFFFFFFFFLL)
    return fail(h, SGNS_EINVAL, "vertex id ending at offset %lld of the walk text exceeds 2^31 - 1", err);
  *max_id = mx;
  return SGNS_OK;
}
}  // namespace

sgns_status sgns_parse_walks(const uint8_t* bytes, int64_t n, int32_t* tokens, int64_t cap, int64_t* n_tokens,
                             int64_t* max_id, void* stream) {
  NvtxRange r_("sgns_parse_walks");
  if ((!bytes && n > 0) || n < 0 || cap < 0 || (cap > 0 && !tokens) || !n_tokens || !max_id)
    return fail(nullptr, SGNS_EINVAL, "bad walk-parse arguments");
  return parse_walks(nullptr, bytes, n, tokens, cap, n_tokens, max_id, static_cast<cudaStream_t>(stream));
}

sgns_status sgns_train_walk_files(sgns_handle* h, const char* const* paths, int32_t n_paths, int64_t V) {
  NvtxRange r_("sgns_train_walk_files");
  if (!h || !paths || n_paths <= 0) return fail(h, SGNS_EINVAL, "bad arguments");
  CU(h, cudaSetDevice(h->opt.device));
  // total text: each file followed by a newline, which ends its last walk as the host
  // reader did at end of file
  std::vector<int64_t> sizes(n_paths);
  int64_t total = 0;
  for (int p = 0; p < n_paths; p++) {
    FILE* f = paths[p] ? fopen(paths[p], "rb") : nullptr;
    if (!f) return fail(h, SGNS_EIO, "cannot open walk file %s", paths[p] ? paths[p] : "(null)");
    if (fseek(f, 0, SEEK_END) != 0 || (sizes[p] = (int64_t)ftell(f)) < 0) {
      fclose(f);
      return fail(h, SGNS_EIO, "cannot size walk file %s", paths[p]);
    }
    fclose(f);
    total += sizes[p] + 1;
  }
  uint8_t* d_text = nullptr;
  uint8_t* stage[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  int32_t* d_tok = nullptr;
  int32_t* d_cnt = nullptr;
  auto cleanup = [&]() {
    cudaStreamSynchronize(h->stream);
    dfree(d_text);
    for (int k = 0; k < 2; k++) {
      if (stage[k]) cudaFreeHost(stage[k]);
      if (done[k]) cudaEventDestroy(done[k]);
    }
    dfree(d_tok);
    dfree(d_cnt);
  };
  auto bail = [&](sgns_status st) {
    cleanup();
    return st;
  };
  const size_t kStage = (size_t)64 << 20;
  cudaError_t e;
  if ((e = cudaMalloc(&d_text, (size_t)total)) != cudaSuccess)
    return bail(fail(h, SGNS_ENOMEM, "walk text of %lld bytes: %s", (long long)total, cudaGetErrorString(e)));
  for (int k = 0; k < 2; k++)
    if ((e = cudaHostAlloc(&stage[k], kStage, cudaHostAllocDefault)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming)) != cudaSuccess)
      return bail(fail(h, SGNS_ENOMEM, "staging buffers: %s", cudaGetErrorString(e)));
  // read every file through two pinned staging buffers; the copy of one overlaps the read
  // of the next
  int64_t off = 0;
  int k = 0;
  bool used[2] = {false, false};
  for (int p = 0; p < n_paths; p++) {
    FILE* f = fopen(paths[p], "rb");
    if (!f) return bail(fail(h, SGNS_EIO, "cannot open walk file %s", paths[p]));
    int64_t left = sizes[p] + 1;
    while (left > 0) {
      if (used[k] && (e = cudaEventSynchronize(done[k])) != cudaSuccess) {
        fclose(f);
        return bail(fail(h, SGNS_ECUDA, "staging copy: %s", cudaGetErrorString(e)));
      }
      size_t want = (size_t)std::min<int64_t>(left, (int64_t)kStage), got = 0;
      const bool last = (int64_t)want == left;  // this chunk ends with the file's newline
      const size_t from_file = last ? want - 1 : want;
      if (from_file > 0) got = fread(stage[k], 1, from_file, f);
      if (got != from_file) {
        fclose(f);
        return bail(fail(h, SGNS_EIO, "short read of walk file %s", paths[p]));
      }
      if (last) stage[k][want - 1] = '\n';
      if ((e = cudaMemcpyAsync(d_text + off, stage[k], want, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
          (e = cudaEventRecord(done[k], h->stream)) != cudaSuccess) {
        fclose(f);
        return bail(fail(h, SGNS_ECUDA, "staging copy: %s", cudaGetErrorString(e)));
      }
      used[k] = true;
      off += (int64_t)want;
      left -= (int64_t)want;
      k ^= 1;
    }
    fclose(f);
  }
  int64_t n = 0, max_id = -1;
  sgns_status st = parse_walks(h, d_text, total, nullptr, 0, &n, &max_id, h->stream);
  if (st && n == 0) return bail(st);  // a bad byte (a zero-token text is not an error here)
  if (n > 0) {
    if ((e = cudaMalloc(&d_tok, sizeof(int32_t) * (size_t)n)) != cudaSuccess)
      return bail(fail(h, SGNS_ENOMEM, "corpus of %lld tokens: %s", (long long)n, cudaGetErrorString(e)));
    st = parse_walks(h, d_text, total, d_tok, n, &n, &max_id, h->stream);
    if (st) return bail(st);
  }
  dfree(d_text);
  if (V <= 0) V = max_id + 1;
  if (max_id >= V) return bail(fail(h, SGNS_EINVAL, "walk files name vertex %lld >= V = %lld", (long long)max_id, (long long)V));
  if (V < 2) return bail(fail(h, SGNS_EINVAL, "vocabulary size %lld out of range", (long long)V));
  // vertex_cn (path.hpp:98) on the device, then the host vocabulary sort
  std::vector<int32_t> counts((size_t)V, 0);
  if ((e = cudaMalloc(&d_cnt, sizeof(int32_t) * (size_t)V)) != cudaSuccess ||
      (e = launch_vertex_count(d_tok, n, d_cnt, V, h->num_sms, h->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(counts.data(), d_cnt, sizeof(int32_t) * (size_t)V, cudaMemcpyDeviceToHost, h->stream)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(h->stream)) != cudaSuccess)
    return bail(fail(h, SGNS_ECUDA, "vertex counts: %s", cudaGetErrorString(e)));
  dfree(d_cnt);
  st = sgns_set_vocab(h, counts.data(), V);
  if (st) return bail(st);
  // the parsed ids become the handle's corpus ids (no host round trip)
  dfree(h->d_ids);
  dfree(h->d_corpus);
  h->d_ids = d_tok;
  d_tok = nullptr;
  h->corpus_cap = 0;
  if ((e = cudaMalloc(&h->d_corpus, sizeof(int32_t) * (size_t)std::max<int64_t>(n, 1))) != cudaSuccess)
    return bail(fail(h, SGNS_ENOMEM, "corpus of %lld tokens: %s", (long long)n, cudaGetErrorString(e)));
  h->corpus_cap = n;
  cleanup();
  st = map_uploaded_corpus(h, h->d_ids, n);
  if (st) return st;
  return sgns_train(h);
}

sgns_status sgns_minibatch_update(int32_t d, int32_t n, const int32_t* in_count, const int32_t* in_first,
                                  const int32_t* out_count, const int32_t* out_meta, const float* alpha,
                                  const float* in_rows, const float* out_rows, float* d_in, float* d_out,
                                  void* stream) {
  if (d < 4 || d > kDMax || d % 4 || n < 0) return fail(nullptr, SGNS_EINVAL, "bad minibatch arguments");
  if (n == 0) return SGNS_OK;
  DeviceScratch* ds = device_scratch();
  if (!ds) return fail(nullptr, SGNS_ECUDA, "no current CUDA device");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> g(ds->mx);
  sgns_status st = ds->ensure(sizeof(int64_t) * 2 * n + 16);
  if (st) return st;
  int32_t* status = reinterpret_cast<int32_t*>(static_cast<char*>(ds->buf) + sizeof(int64_t) * 2 * n);
  if (cudaMemsetAsync(status, 0, sizeof(int32_t), s) != cudaSuccess) return fail(nullptr, SGNS_ECUDA, "memset");
  cudaError_t e = launch_minibatch(d, n, kIMax, kOMax, in_count, in_first, out_count, out_meta, alpha, in_rows,
                                   out_rows, d_in, d_out, ds->exp, static_cast<int64_t*>(ds->buf), status, s);
  if (e != cudaSuccess) return fail(nullptr, SGNS_ECUDA, "minibatch kernel: %s", cudaGetErrorString(e));
  int32_t hs = 0;
  if ((e = cudaMemcpyAsync(&hs, status, sizeof hs, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(nullptr, SGNS_ECUDA, "minibatch kernel: %s", cudaGetErrorString(e));
  if (hs) return fail(nullptr, SGNS_EINVAL, "a minibatch exceeds %d inputs / %d outputs or has first > inputs", kIMax, kOMax);
  return SGNS_OK;
}

sgns_status sgns_minibatch_update_bf16(int32_t d, int32_t n, const int32_t* in_count, const int32_t* in_first,
                                       const int32_t* out_count, const int32_t* out_meta, const float* alpha,
                                       const float* in_rows, const float* out_rows, uint16_t* new_in,
                                       uint16_t* new_out, uint64_t sr_seed, void* stream) {
  if (d < 4 || d > kDMax || d % 4 || n < 0) return fail(nullptr, SGNS_EINVAL, "bad minibatch arguments");
  if (n == 0) return SGNS_OK;
  DeviceScratch* ds = device_scratch();
  if (!ds) return fail(nullptr, SGNS_ECUDA, "no current CUDA device");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> g(ds->mx);
  sgns_status st = ds->ensure(sizeof(int64_t) * 2 * n + 16);
  if (st) return st;
  int32_t* status = reinterpret_cast<int32_t*>(static_cast<char*>(ds->buf) + sizeof(int64_t) * 2 * n);
  if (cudaMemsetAsync(status, 0, sizeof(int32_t), s) != cudaSuccess) return fail(nullptr, SGNS_ECUDA, "memset");
  cudaError_t e = launch_minibatch_bf16(d, n, kIMax, in_count, in_first, out_count, out_meta, alpha, in_rows,
                                        out_rows, new_in, new_out, sr_seed, ds->exp,
                                        static_cast<int64_t*>(ds->buf), status, s);
  if (e != cudaSuccess) return fail(nullptr, SGNS_ECUDA, "minibatch kernel: %s", cudaGetErrorString(e));
  int32_t hs = 0;
  if ((e = cudaMemcpyAsync(&hs, status, sizeof hs, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(nullptr, SGNS_ECUDA, "minibatch kernel: %s", cudaGetErrorString(e));
  if (hs) return fail(nullptr, SGNS_EINVAL, "a minibatch exceeds %d inputs / %d outputs or has first > inputs", kIMax, kOMax);
  return SGNS_OK;
}

sgns_status sgns_link_scores(int32_t dtype, int32_t d, const void* table, int64_t V, const int32_t* pairs,
                             int64_t n, float* scores, void* stream) {
  if ((dtype != 0 && dtype != 1) || d < 4 || d > kDMax || d % 4 || V < 1 || n < 0 ||
      (n > 0 && (!table || !pairs || !scores)))
    return fail(nullptr, SGNS_EINVAL, "bad link-score arguments");
  if (n == 0) return SGNS_OK;
  DeviceScratch* ds = device_scratch();
  if (!ds) return fail(nullptr, SGNS_ECUDA, "no current CUDA device");
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return fail(nullptr, SGNS_ECUDA, "device query failed");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> g(ds->mx);
  sgns_status st = ds->ensure(16);
  if (st) return st;
  int32_t* bad = static_cast<int32_t*>(ds->buf);
  int32_t hb = 0;
  cudaError_t e;
  if ((e = cudaMemsetAsync(bad, 0, sizeof(int32_t), s)) != cudaSuccess ||
      (e = launch_link_scores(dtype == 1 ? STORE_BF16 : STORE_F32, table, d, V, pairs, n, scores, bad, sms, s)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(&hb, bad, sizeof hb, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(nullptr, SGNS_ECUDA, "link scores: %s", cudaGetErrorString(e));
  if (hb) return fail(nullptr, SGNS_EINVAL, "a pair names a row outside [0, %lld)", (long long)V);
  return SGNS_OK;
}

namespace {
// Checks a device CSR graph; status word in scratch.  Returns SGNS_OK or the error.
sgns_status check_csr(const char* what, const int64_t* indptr, const int32_t* indices, int64_t V, int64_t E,
                      int32_t* status, int sms, cudaStream_t s) {
  int32_t hs = 0;
  cudaError_t e;
  if ((e = cudaMemsetAsync(status, 0, sizeof(int32_t), s)) != cudaSuccess ||
      (e = launch_validate_csr(indptr, indices, V, E, status, sms, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&hs, status, sizeof hs, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(nullptr, SGNS_ECUDA, "%s: %s", what, cudaGetErrorString(e));
  if (hs & 4) return fail(nullptr, SGNS_EINVAL, "%s: indptr must start at 0, end at n_edges and not decrease", what);
  if (hs & 1) return fail(nullptr, SGNS_EINVAL, "%s: a neighbour id lies outside [0, %lld)", what, (long long)V);
  return SGNS_OK;
}

int device_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  return sms;
}
}  // namespace

sgns_status sgns_edge_common_neighbors(const int64_t* indptr, const int32_t* indices, int64_t V, int64_t n_edges,
                                       int32_t* cn, void* stream) {
  NvtxRange r_("sgns_edge_common_neighbors");
  if (V < 1 || V > INT32_MAX || n_edges < 0 || !indptr || (n_edges > 0 && (!indices || !cn)))
    return fail(nullptr, SGNS_EINVAL, "bad common-neighbour arguments");
  const int sms = device_sms();
  if (!sms) return fail(nullptr, SGNS_ECUDA, "no current CUDA device");
  DeviceScratch* ds = device_scratch();
  if (!ds) return fail(nullptr, SGNS_ECUDA, "no current CUDA device");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> g(ds->mx);
  sgns_status st = ds->ensure(64);
  if (st) return st;
  int32_t* status = static_cast<int32_t*>(ds->buf);
  if ((st = check_csr("common neighbours", indptr, indices, V, n_edges, status, sms, s))) return st;
  int32_t hs = 0;
  cudaError_t e;
  if ((e = launch_edge_common_neighbors(indptr, indices, V, n_edges, cn, status, sms, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&hs, status, sizeof hs, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(nullptr, SGNS_ECUDA, "common neighbours: %s", cudaGetErrorString(e));
  if (hs & 2) return fail(nullptr, SGNS_EINVAL, "common neighbours: an adjacency list is not strictly increasing");
  return SGNS_OK;
}

sgns_status sgns_info_walks(const sgns_walk_options* o, const int64_t* indptr, const int32_t* indices,
                            const int32_t* cn, int64_t V, int64_t n_edges, int32_t* corpus, int64_t cap,
                            int64_t* n_tokens, void* stream) {
  NvtxRange r_("sgns_info_walks");
  if (!o || !n_tokens || V < 1 || V > INT32_MAX || n_edges < 0 || !indptr || (n_edges > 0 && (!indices || !cn)) ||
      cap < 0 || (cap > 0 && !corpus))
    return fail(nullptr, SGNS_EINVAL, "bad walk arguments");
  if (o->walker_num < 0 || o->min_length < 0 || o->max_length < 1 || o->max_length > kWalkMaxLength ||
      !(o->r_threshold == o->r_threshold) || (o->trace_steps != 0 && o->trace_steps != 1))
    return fail(nullptr, SGNS_EINVAL,
                "walk options: walker_num >= 0, min_length >= 0, max_length in [1, %d], trace_steps 0 or 1",
                kWalkMaxLength);
  *n_tokens = 0;
  if (o->walker_num == 0) return SGNS_OK;
  const int sms = device_sms();
  if (!sms) return fail(nullptr, SGNS_ECUDA, "no current CUDA device");
  DeviceScratch* ds = device_scratch();
  if (!ds) return fail(nullptr, SGNS_ECUDA, "no current CUDA device");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> g(ds->mx);
  const size_t xl_bytes = sizeof(double) * (size_t)(kWalkMaxLength + 2);
  sgns_status st = ds->ensure(256 + xl_bytes + walk_scratch_bytes(o->walker_num));
  if (st) return st;
  char* base = static_cast<char*>(ds->buf);
  int32_t* status = reinterpret_cast<int32_t*>(base);
  double* xl = reinterpret_cast<double*>(base + 256);
  void* scratch = base + 256 + xl_bytes;
  if ((st = check_csr("walks", indptr, indices, V, n_edges, status, sms, s))) return st;
  std::vector<double> hxl(kWalkMaxLength + 2);
  xlog2x_table(kWalkMaxLength + 2, hxl.data());
  int64_t* offsets = nullptr;
  int64_t total = 0;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(xl, hxl.data(), xl_bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = launch_info_walks_count(indptr, indices, cn, xl, V, o->walker_num, o->min_length, o->max_length,
                                   o->r_threshold, o->seed, o->trace_steps, scratch, sms, &offsets, s)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(&total, offsets + o->walker_num, sizeof total, cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(nullptr, SGNS_ECUDA, "walks: %s", cudaGetErrorString(e));
  *n_tokens = total;
  if (total > cap) {
    if (cap == 0 && !corpus) return SGNS_OK;
    return fail(nullptr, SGNS_EINVAL, "walks yield %lld tokens, capacity %lld", (long long)total, (long long)cap);
  }
  if ((e = launch_info_walks_emit(indptr, indices, cn, xl, V, o->walker_num, o->min_length, o->max_length,
                                  o->r_threshold, o->seed, o->trace_steps, offsets, corpus, sms, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(nullptr, SGNS_ECUDA, "walks: %s", cudaGetErrorString(e));
  return SGNS_OK;
}

sgns_status sgns_loss_adjoint(int32_t dtype, int32_t d, int64_t V, int32_t n, const int32_t* in_ptr,
                              const int32_t* in_ids, const int32_t* in_first, const int32_t* out_ptr,
                              const int32_t* out_ids, const int32_t* out_meta, const void* wih, const void* woh,
                              double* loss, int32_t* grad_in_ids, void* grad_in, int64_t* n_in,
                              int32_t* grad_out_ids, void* grad_out, int64_t* n_out, void* stream) {
  if (dtype < 0 || dtype > 2 || d < 1 || d > kDMax || V < 1 || V > INT32_MAX || n < 0 || !n_in || !n_out)
    return fail(nullptr, SGNS_EINVAL, "bad adjoint arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DeviceScratch* ds = device_scratch();
  if (!ds) return fail(nullptr, SGNS_ECUDA, "no current CUDA device");
  std::lock_guard<std::mutex> g(ds->mx);
  sgns_status st = ds->ensure(adjoint_scratch_bytes(V) + 64);
  if (st) return st;
  int32_t* info = reinterpret_cast<int32_t*>(static_cast<char*>(ds->buf) + adjoint_scratch_bytes(V));
  // phase 1 finds, on the device, the distinct rows and the largest minibatch; its sizes
  // (five ints) are the one read-back before the gradient kernel
  cudaError_t e = launch_adjoint_prepare(dtype, d, n, V, in_ptr, in_ids, in_first, out_ptr, out_ids, loss,
                                         grad_in_ids, grad_in, grad_out_ids, grad_out, info, ds->buf, s);
  int32_t h[5];
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, info, sizeof h, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(nullptr, SGNS_ECUDA, "adjoint: %s", cudaGetErrorString(e));
  if (h[2] & 2)
    return fail(nullptr, SGNS_EINVAL, "adjoint: a minibatch has descending or negative offsets, more than %d inputs "
                "or %d outputs, or first outside [0, inputs]", kIMax, kOMax);
  if (h[2] & 1) return fail(nullptr, SGNS_EINVAL, "adjoint: a row id outside [0, %lld)", (long long)V);
  *n_in = h[0];
  *n_out = h[1];
  e = launch_adjoint(dtype, d, n, V, h[3], h[4], in_ptr, in_ids, in_first, out_ptr, out_ids, out_meta, wih, woh, loss,
                     grad_in, grad_out, ds->buf, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(nullptr, SGNS_ECUDA, "adjoint kernels: %s", cudaGetErrorString(e));
  return SGNS_OK;
}

}  // extern "C"
