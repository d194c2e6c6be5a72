// dsgl_ingest.cu -- walk-file text to the trainer's corpus, on the GPU.
//
// The text is the reference's walk format (include/path.hpp:92,108: " %u" per vertex,
// "\n" after each walk), tokenised on the separators the reference's reader uses
// (word2vec.cu:1008, " \n\r\t").  Output: vertex ids with -1 after each walk that holds
// at least one id -- the layout of graph->local_corpus (path.hpp:96,110) that
// Train_SGNS_MPI reads.  The buffer is read as one file: position n acts as a final
// newline, so the last walk ends even without one.
//
// Three passes over 8 KB tiles (256 threads x 32 bytes, staged in shared memory):
//   1. each thread summarises its 32 bytes as a Span (outputs it emits, whether its first
//      significant byte is a newline whose walk end depends on what precedes it, and the
//      kind of its last significant byte); a block scan gives the tile's Span;
//   2. one block scans the tile Spans (64-bit output counts);
//   3. each thread rebuilds its exclusive prefix and writes ids and walk ends at their
//      final offsets; an id is parsed backward from its last digit (at most 10 digits, a
//      16-byte halo before the tile holds the start of an id cut by the tile edge).
// Span combination is associative, so the order of the scans does not matter.
#include <cuda_runtime.h>

#include <cstdint>

#include "dsgl_device.cuh"

namespace sgns {

namespace {

constexpr int kIngThreads = 256;
constexpr int kIngBytes = 32;                       // bytes per thread
constexpr int kIngTile = kIngThreads * kIngBytes;   // 8192 bytes per tile
constexpr int kIngHalo = 16;                        // bytes staged before the tile
constexpr int kScanBlock = 1024;

enum : uint32_t { SIG_NONE = 0, SIG_DIGIT = 1, SIG_NL = 2 };

struct Span {
  unsigned long long cnt;  // outputs, not counting a pending first newline
  uint32_t pend;           // first significant byte is a newline
  uint32_t last;           // kind of the last significant byte
};

__host__ __device__ __forceinline__ Span span_combine(Span a, Span b) {
  Span r;
  r.cnt = a.cnt + b.cnt + ((b.pend && a.last == SIG_DIGIT) ? 1ull : 0ull);
  r.pend = a.last != SIG_NONE ? a.pend : b.pend;
  r.last = b.last != SIG_NONE ? b.last : a.last;
  return r;
}

__device__ __forceinline__ Span span_identity() { return Span{0ull, 0u, SIG_NONE}; }

__device__ __forceinline__ bool is_digit(uint8_t c) { return c >= '0' && c <= '9'; }
__device__ __forceinline__ bool is_blank(uint8_t c) { return c == ' ' || c == '\t' || c == '\r'; }

// byte i of the text with a virtual newline at n and blanks after it
__device__ __forceinline__ uint8_t text_byte(const uint8_t* b, int64_t n, int64_t i) {
  return i < n ? __ldg(b + i) : (i == n ? (uint8_t)'\n' : (uint8_t)' ');
}

// Stages tile bytes [base - halo, base + kIngTile] (one byte of look-ahead) in shared memory.
__device__ __forceinline__ void stage_tile(const uint8_t* b, int64_t n, int64_t base, uint8_t* s) {
  for (int k = threadIdx.x; k < kIngHalo + kIngTile + 1; k += blockDim.x) {
    const int64_t i = base - kIngHalo + k;
    s[k] = i < 0 ? (uint8_t)' ' : text_byte(b, n, i);
  }
  __syncthreads();
}

// Span of one thread's 32 bytes; s points at the thread's first byte in shared memory.
__device__ __forceinline__ Span thread_span(const uint8_t* s, int64_t first, int64_t* bad) {
  Span sp = span_identity();
  uint32_t cnt = 0;
#pragma unroll 4
  for (int j = 0; j < kIngBytes; j++) {
    const uint8_t c = s[j];
    if (is_digit(c)) {
      if (!is_digit(s[j + 1])) cnt++;
      sp.last = SIG_DIGIT;
    } else if (c == '\n') {
      if (sp.last == SIG_DIGIT) cnt++;
      else if (sp.last == SIG_NONE) sp.pend = 1;
      sp.last = SIG_NL;
    } else if (!is_blank(c)) {
      if (*bad < 0) *bad = first + j;
    }
  }
  sp.cnt = cnt;
  return sp;
}

// Block-wide exclusive scan of Spans (blockDim.x == kIngThreads); returns the thread's
// exclusive prefix and writes the block total to *total.
__device__ __forceinline__ Span block_exclusive(Span v, Span* total) {
  __shared__ Span warp_tot[kIngThreads / 32];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  Span inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    Span u;
    u.cnt = __shfl_up_sync(kFull, inc.cnt, o);
    u.pend = __shfl_up_sync(kFull, inc.pend, o);
    u.last = __shfl_up_sync(kFull, inc.last, o);
    if (lane >= o) inc = span_combine(u, inc);
  }
  if (lane == 31) warp_tot[wp] = inc;
  __syncthreads();
  Span before = span_identity();
  for (int k = 0; k < wp; k++) before = span_combine(before, warp_tot[k]);
  Span ex;
  ex.cnt = __shfl_up_sync(kFull, inc.cnt, 1);
  ex.pend = __shfl_up_sync(kFull, inc.pend, 1);
  ex.last = __shfl_up_sync(kFull, inc.last, 1);
  if (lane == 0) ex = span_identity();
  Span all = span_identity();
  for (int k = 0; k < kIngThreads / 32; k++) all = span_combine(all, warp_tot[k]);
  *total = all;
  __syncthreads();
  return span_combine(before, ex);
}

__device__ __forceinline__ void record_bad(long long* err, int64_t bad) {
  if (bad >= 0) atomicMin(err, (long long)bad);
}

__global__ void __launch_bounds__(kIngThreads) ingest_count_kernel(const uint8_t* b, int64_t n, Span* tile_span,
                                                                  long long* err) {
  __shared__ uint8_t s[kIngHalo + kIngTile + 1];
  const int64_t base = (int64_t)blockIdx.x * kIngTile;
  stage_tile(b, n, base, s);
  const int64_t first = base + (int64_t)threadIdx.x * kIngBytes;
  int64_t bad = -1;
  const Span v = first <= n ? thread_span(s + kIngHalo + threadIdx.x * kIngBytes, first, &bad) : span_identity();
  record_bad(err, bad);
  Span total;
  block_exclusive(v, &total);
  if (threadIdx.x == 0) tile_span[blockIdx.x] = total;
}

// Exclusive scan of the tile Spans by one block; the text starts as if after a newline.
// out[t] = prefix of tile t; out[ntiles] = the whole text.
__global__ void __launch_bounds__(kScanBlock) ingest_scan_kernel(const Span* tile_span, int64_t ntiles, Span* out) {
  __shared__ Span part[kScanBlock];
  const int64_t per = (ntiles + kScanBlock - 1) / kScanBlock;
  const int64_t lo = (int64_t)threadIdx.x * per, hi = lo + per < ntiles ? lo + per : ntiles;
  Span acc = span_identity();
  for (int64_t t = lo; t < hi; t++) acc = span_combine(acc, tile_span[t]);
  part[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {  // 1024 partials: a short serial pass
    Span run = Span{0ull, 0u, SIG_NL};
    for (int k = 0; k < kScanBlock; k++) {
      const Span p = part[k];
      part[k] = run;
      run = span_combine(run, p);
    }
    out[ntiles] = run;
  }
  __syncthreads();
  Span run = part[threadIdx.x];
  for (int64_t t = lo; t < hi; t++) {
    out[t] = run;
    run = span_combine(run, tile_span[t]);
  }
}

__global__ void __launch_bounds__(kIngThreads) ingest_emit_kernel(const uint8_t* b, int64_t n, const Span* tile_prefix,
                                                                 int32_t* tokens, long long* err,
                                                                 unsigned long long* max_id /* largest id + 1 */) {
  __shared__ uint8_t s[kIngHalo + kIngTile + 1];
  const int64_t base = (int64_t)blockIdx.x * kIngTile;
  stage_tile(b, n, base, s);
  const int64_t first = base + (int64_t)threadIdx.x * kIngBytes;
  const uint8_t* my = s + kIngHalo + threadIdx.x * kIngBytes;
  int64_t bad = -1;
  const Span v = first <= n ? thread_span(my, first, &bad) : span_identity();
  Span total;
  const Span ex = span_combine(tile_prefix[blockIdx.x], block_exclusive(v, &total));
  long long mx = -1;
  if (first <= n) {
    unsigned long long pos = ex.cnt;
    uint32_t last = ex.last;
    for (int j = 0; j < kIngBytes; j++) {
      const uint8_t c = my[j];
      if (is_digit(c)) {
        if (!is_digit(my[j + 1])) {  // last digit of an id: read it backward
          long long val = 0, scale = 1;
          int k = j, nd = 0;
          while (nd <= 10 && is_digit(my[k])) {
            val += (long long)(my[k] - '0') * scale;
            scale *= 10;
            nd++;
            k--;
          }
          if (nd > 10 || val > 2147483647LL) {
            if (bad < 0) bad = first + j;
            val = 0;
          }
          tokens[pos++] = (int32_t)val;
          mx = val > mx ? val : mx;
        }
        last = SIG_DIGIT;
      } else if (c == '\n') {
        if (last == SIG_DIGIT) tokens[pos++] = -1;
        last = SIG_NL;
      }
    }
  }
  record_bad(err, bad);
  for (int o = 16; o > 0; o >>= 1) {
    const long long t = __shfl_xor_sync(kFull, mx, o);
    mx = t > mx ? t : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx >= 0) atomicMax(max_id, (unsigned long long)mx + 1);  // 0: no id
}

// Occurrences of each vertex (the reference's vertex_cn, path.hpp:98); lanes holding the
// same id add once per warp.
__global__ void vertex_count_kernel(const int32_t* tokens, int64_t n, int32_t* counts, int64_t V) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
    const int64_t i = i0 + threadIdx.x;
    const int32_t v = i < n ? tokens[i] : -1;
    const bool ok = v >= 0 && v < V;
    const unsigned grp = __match_any_sync(kFull, ok ? v : -1);
    if (ok && (__ffs(grp) - 1) == (int)(threadIdx.x & 31)) atomicAdd(&counts[v], __popc(grp));
  }
}

}  // namespace

size_t ingest_scratch_bytes(int64_t n) {
  const int64_t ntiles = (n + 1 + kIngTile - 1) / kIngTile;
  return sizeof(Span) * (size_t)(2 * ntiles + 1) + 64;
}

cudaError_t launch_ingest_count(const uint8_t* bytes, int64_t n, void* scratch, unsigned long long* n_out,
                                long long* err_pos, cudaStream_t s) {
  const int64_t ntiles = (n + 1 + kIngTile - 1) / kIngTile;
  Span* tile_span = static_cast<Span*>(scratch);
  Span* prefix = tile_span + ntiles;
  long long* err = reinterpret_cast<long long*>(prefix + ntiles + 1);
  const long long big = 0x7FFFFFFFFFFFFFFFLL;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(err, &big, sizeof big, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
  ingest_count_kernel<<<(unsigned)ntiles, kIngThreads, 0, s>>>(bytes, n, tile_span, err);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  ingest_scan_kernel<<<1, kScanBlock, 0, s>>>(tile_span, ntiles, prefix);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  Span whole;
  if ((e = cudaMemcpyAsync(&whole, prefix + ntiles, sizeof whole, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(err_pos, err, sizeof *err_pos, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return e;
  *n_out = whole.cnt;
  return cudaSuccess;
}

cudaError_t launch_ingest_emit(const uint8_t* bytes, int64_t n, void* scratch, int32_t* tokens, long long* err_pos,
                               long long* max_id, cudaStream_t s) {
  const int64_t ntiles = (n + 1 + kIngTile - 1) / kIngTile;
  Span* tile_span = static_cast<Span*>(scratch);
  Span* prefix = tile_span + ntiles;
  long long* err = reinterpret_cast<long long*>(prefix + ntiles + 1);
  unsigned long long* mx = reinterpret_cast<unsigned long long*>(err + 1);
  cudaError_t e;
  if ((e = cudaMemsetAsync(mx, 0, sizeof *mx, s)) != cudaSuccess) return e;
  ingest_emit_kernel<<<(unsigned)ntiles, kIngThreads, 0, s>>>(bytes, n, prefix, tokens, err, mx);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  unsigned long long m = 0;
  if ((e = cudaMemcpyAsync(err_pos, err, sizeof *err_pos, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&m, mx, sizeof m, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return e;
  *max_id = (long long)m - 1;
  return cudaSuccess;
}

cudaError_t launch_vertex_count(const int32_t* tokens, int64_t n, int32_t* counts, int64_t V, int num_sms,
                                cudaStream_t s) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(counts, 0, sizeof(int32_t) * (size_t)V, s)) != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
  vertex_count_kernel<<<(unsigned)blocks, 256, 0, s>>>(tokens, n, counts, V);
  return cudaGetLastError();
}

}  // namespace sgns
