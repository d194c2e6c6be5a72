// dsgl_ingest.cu -- walk-file text to the trainer's corpus, on the GPU.
//
// The text is the reference's walk format (include/path.hpp:92,108: " %u" per vertex,
// "\n" after each walk), tokenised on the separators the reference's reader uses
// (word2vec.cu:1008, " \n\r\t").  Output: vertex ids with -1 after each walk that holds
// at least one id -- the layout of graph->local_corpus (path.hpp:96,110) that
// Train_SGNS_MPI reads.  The buffer is read as one file: position n acts as a final
// newline, so the last walk ends even without one.
//
// Three passes over 8 KB tiles (256 threads x 32 bytes, staged in shared memory with
// 16-byte loads; each thread classifies its 32 bytes into digit / newline bit masks with
// byte-wise compares, so ids and walk ends are found with bit operations):
//   1. each thread summarises its 32 bytes as a Span (outputs it emits, whether its first
//      significant byte is a newline whose walk end depends on what precedes it, and the
//      kind of its last significant byte); a block scan gives the tile's Span;
//   2. the tile Spans are scanned in two levels (64-bit output counts): groups of 1024
//      tiles by one block each, the group totals by one block, then the group prefixes
//      are added to the tiles';
//   3. each thread rebuilds its exclusive prefix and writes ids and walk ends at their
//      final offsets; an id is parsed backward from its last digit (at most 10 digits, a
//      16-byte halo before the tile holds the start of an id cut by the tile edge).
// Span combination is associative, so the order of the scans does not matter.
#include <cuda_runtime.h>

#include <algorithm>
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

// byte i of the text with a virtual newline at n and blanks after it
__device__ __forceinline__ uint8_t text_byte(const uint8_t* b, int64_t n, int64_t i) {
  return i < n ? __ldg(b + i) : (i == n ? (uint8_t)'\n' : (uint8_t)' ');
}

__device__ __constant__ uint32_t kPow10[9] = {1u, 10u, 100u, 1000u, 10000u, 100000u, 1000000u, 10000000u,
                                              100000000u};

constexpr int kStageChunks = (kIngHalo + kIngTile + 16) / 16;  // 16-byte chunks staged per tile

// Stages tile bytes [base - halo, base + kIngTile + 16) in shared memory: 16 bytes per load
// where the chunk lies inside the text and the text starts on a 16-byte boundary (tiles
// are 8 KB apart, so every chunk is then aligned), byte by byte otherwise.
__device__ __forceinline__ void stage_tile(const uint8_t* b, int64_t n, int64_t base, bool aligned, uint8_t* s) {
  for (int c = threadIdx.x; c < kStageChunks; c += blockDim.x) {
    const int64_t g = base - kIngHalo + 16 * (int64_t)c;
    uint4 v;
    if (aligned && g >= 0 && g + 16 <= n) {
      v = __ldg(reinterpret_cast<const uint4*>(b + g));
    } else {
      uint8_t t[16];
#pragma unroll
      for (int k = 0; k < 16; k++) t[k] = g + k < 0 ? (uint8_t)' ' : text_byte(b, n, g + k);
      v = make_uint4(t[0] | t[1] << 8 | t[2] << 16 | (uint32_t)t[3] << 24, t[4] | t[5] << 8 | t[6] << 16 | (uint32_t)t[7] << 24,
                     t[8] | t[9] << 8 | t[10] << 16 | (uint32_t)t[11] << 24,
                     t[12] | t[13] << 8 | t[14] << 16 | (uint32_t)t[15] << 24);
    }
    reinterpret_cast<uint4*>(s)[c] = v;
  }
  __syncthreads();
}

// Byte-class tests on 4 bytes at once (SWAR; no carry crosses a byte): 0x80 in each byte
// that is NOT a decimal digit, resp. in each NONZERO byte.
__device__ __forceinline__ uint32_t nondigit80(uint32_t w) {
  const uint32_t t = w ^ 0x30303030u;  // digits become 0..9
  return (((t & 0x7F7F7F7Fu) + 0x76767676u) | t) & 0x80808080u;
}
__device__ __forceinline__ uint32_t nonzero80(uint32_t x) {
  return (((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u;
}
// one bit per byte from a 0x80-per-byte mask
__device__ __forceinline__ uint32_t nibble(uint32_t m80) { return (m80 * 0x00204081u) >> 28; }

// Class masks of a thread's 32 bytes (bit j = byte j): digits, newlines and, when
// kCheck, anything that is not a digit, newline, space, tab or CR.
struct Masks {
  uint32_t dig, nl, bad;
};
template <bool kCheck>
__device__ __forceinline__ Masks classify(const uint8_t* s) {
  const uint4 a = reinterpret_cast<const uint4*>(s)[0], c = reinterpret_cast<const uint4*>(s)[1];
  const uint32_t w[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
  Masks m{0u, 0u, 0u};
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const uint32_t dg = nondigit80(w[k]) ^ 0x80808080u;
    const uint32_t nl = nonzero80(w[k] ^ 0x0A0A0A0Au) ^ 0x80808080u;
    m.dig |= nibble(dg) << (4 * k);
    m.nl |= nibble(nl) << (4 * k);
    if (kCheck) {
      const uint32_t bl = (nonzero80(w[k] ^ 0x20202020u) & nonzero80(w[k] ^ 0x09090909u) &
                           nonzero80(w[k] ^ 0x0D0D0D0Du)) ^ 0x80808080u;
      m.bad |= nibble(0x80808080u & ~(dg | nl | bl)) << (4 * k);
    }
  }
  return m;
}

// Outputs of a thread's 32 bytes as bit masks: ends of ids (last digit) and newlines that
// end a walk given the kind of significant byte before the span (carry: SIG_*; SIG_NONE
// leaves the first newline undecided and reported in *pend).
struct Emits {
  uint32_t ids, walks;
};
__device__ __forceinline__ Emits emits(const Masks& m, bool next_digit, uint32_t carry, uint32_t* pend) {
  Emits e;
  e.ids = m.dig & ~((m.dig >> 1) | (next_digit ? 0x80000000u : 0u));
  e.walks = 0;
  *pend = 0;
  const uint32_t sig = m.dig | m.nl;
  uint32_t nls = m.nl;
  while (nls) {
    const int p = __ffs(nls) - 1;
    nls &= nls - 1;
    const uint32_t before = sig & ((1u << p) - 1u);
    if (before) {
      if ((m.dig >> (31 - __clz(before))) & 1u) e.walks |= 1u << p;
    } else if (carry == SIG_DIGIT) {
      e.walks |= 1u << p;
    } else if (carry == SIG_NONE) {
      *pend = 1;
    }
  }
  return e;
}

// Span of one thread's 32 bytes from its masks and its outputs with no carry.
__device__ __forceinline__ Span span_of(const Masks& m, const Emits& e, uint32_t pend) {
  const uint32_t sig = m.dig | m.nl;
  Span sp;
  sp.cnt = __popc(e.ids) + __popc(e.walks);
  sp.pend = pend;
  sp.last = sig == 0 ? SIG_NONE : (((m.dig >> (31 - __clz(sig))) & 1u) ? SIG_DIGIT : SIG_NL);
  return sp;
}

// Span of one thread's 32 bytes; s points at the thread's first byte in shared memory.
template <bool kCheck>
__device__ __forceinline__ Span thread_span(const uint8_t* s, int64_t first, int64_t* bad) {
  const Masks m = classify<kCheck>(s);
  if (m.bad) *bad = first + __ffs(m.bad) - 1;
  uint32_t pend;
  const Emits e = emits(m, is_digit(s[kIngBytes]), SIG_NONE, &pend);
  return span_of(m, e, pend);
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

__global__ void __launch_bounds__(kIngThreads) ingest_count_kernel(const uint8_t* b, int64_t n, bool aligned,
                                                                  Span* tile_span, long long* err) {
  __shared__ __align__(16) uint8_t s[kIngHalo + kIngTile + 16];
  const int64_t base = (int64_t)blockIdx.x * kIngTile;
  stage_tile(b, n, base, aligned, s);
  const int64_t first = base + (int64_t)threadIdx.x * kIngBytes;
  int64_t bad = -1;
  const Span v = first <= n ? thread_span<true>(s + kIngHalo + threadIdx.x * kIngBytes, first, &bad) : span_identity();
  record_bad(err, bad);
  Span total;
  block_exclusive(v, &total);
  if (threadIdx.x == 0) tile_span[blockIdx.x] = total;
}

// Exclusive scan of Spans by one block, 1024 consecutive Spans per round (coalesced reads,
// block scan, carry to the next round); the text starts as if after a newline.  Used on
// the group totals: out[g] = prefix of group g; out[ngroups] = the whole text.
__global__ void __launch_bounds__(kScanBlock) ingest_scan_kernel(const Span* tile_span, int64_t ntiles, Span* out) {
  __shared__ Span warp_tot[kScanBlock / 32];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  Span carry = Span{0ull, 0u, SIG_NL};
  for (int64_t r0 = 0; r0 < ntiles; r0 += kScanBlock) {
    const int64_t t = r0 + threadIdx.x;
    const Span v = t < ntiles ? tile_span[t] : span_identity();
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
    if (wp == 0) {  // scan of the 32 warp totals
      Span w = warp_tot[lane];
      for (int o = 1; o < 32; o <<= 1) {
        Span u;
        u.cnt = __shfl_up_sync(kFull, w.cnt, o);
        u.pend = __shfl_up_sync(kFull, w.pend, o);
        u.last = __shfl_up_sync(kFull, w.last, o);
        if (lane >= o) w = span_combine(u, w);
      }
      warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    Span before = wp > 0 ? warp_tot[wp - 1] : span_identity();
    Span ex;
    ex.cnt = __shfl_up_sync(kFull, inc.cnt, 1);
    ex.pend = __shfl_up_sync(kFull, inc.pend, 1);
    ex.last = __shfl_up_sync(kFull, inc.last, 1);
    if (lane == 0) ex = span_identity();
    if (t < ntiles) out[t] = span_combine(carry, span_combine(before, ex));
    carry = span_combine(carry, warp_tot[kScanBlock / 32 - 1]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[ntiles] = carry;
}

// Pass 2, first level: one block per group of kScanBlock consecutive tiles; out[t] = prefix
// of tile t within its group, group_tot[g] = the group's Span.
__global__ void __launch_bounds__(kScanBlock) ingest_scan_groups_kernel(const Span* tile_span, int64_t ntiles,
                                                                       Span* out, Span* group_tot) {
  __shared__ Span warp_tot[kScanBlock / 32];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int64_t t = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  const Span v = t < ntiles ? tile_span[t] : span_identity();
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
  if (wp == 0) {
    Span w = warp_tot[lane];
    for (int o = 1; o < 32; o <<= 1) {
      Span u;
      u.cnt = __shfl_up_sync(kFull, w.cnt, o);
      u.pend = __shfl_up_sync(kFull, w.pend, o);
      u.last = __shfl_up_sync(kFull, w.last, o);
      if (lane >= o) w = span_combine(u, w);
    }
    warp_tot[lane] = w;
  }
  __syncthreads();
  Span ex;
  ex.cnt = __shfl_up_sync(kFull, inc.cnt, 1);
  ex.pend = __shfl_up_sync(kFull, inc.pend, 1);
  ex.last = __shfl_up_sync(kFull, inc.last, 1);
  if (lane == 0) ex = span_identity();
  if (t < ntiles) out[t] = span_combine(wp > 0 ? warp_tot[wp - 1] : span_identity(), ex);
  if (threadIdx.x == 0) group_tot[blockIdx.x] = warp_tot[kScanBlock / 32 - 1];
}

// Pass 2, last step: every tile's prefix behind its group's; out[ntiles] = the whole text.
__global__ void ingest_scan_add_kernel(Span* out, int64_t ntiles, const Span* group_pre, int64_t ngroups) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= ntiles; t += (int64_t)gridDim.x * blockDim.x)
    out[t] = t < ntiles ? span_combine(group_pre[t / kScanBlock], out[t]) : group_pre[ngroups];
}

__global__ void __launch_bounds__(kIngThreads) ingest_emit_kernel(const uint8_t* b, int64_t n, bool aligned,
                                                                 const Span* tile_prefix,
                                                                 int32_t* tokens, long long* err,
                                                                 unsigned long long* max_id /* largest id + 1 */) {
  __shared__ __align__(16) uint8_t s[kIngHalo + kIngTile + 16];
  const int64_t base = (int64_t)blockIdx.x * kIngTile;
  stage_tile(b, n, base, aligned, s);
  const int64_t first = base + (int64_t)threadIdx.x * kIngBytes;
  const uint8_t* my = s + kIngHalo + threadIdx.x * kIngBytes;
  int64_t bad = -1;
  // the count pass has checked every byte; this pass only reads valid text.  The bytes are
  // classified once: the outputs with no carry give the thread's Span, and once the
  // prefix is known a pending first newline becomes a walk end when a digit precedes it.
  Masks m{0u, 0u, 0u};
  Emits e{0u, 0u};
  uint32_t pend = 0;
  if (first <= n) {
    m = classify<false>(my);
    e = emits(m, is_digit(my[kIngBytes]), SIG_NONE, &pend);
  }
  const Span v = first <= n ? span_of(m, e, pend) : span_identity();
  Span total;
  const Span ex = span_combine(tile_prefix[blockIdx.x], block_exclusive(v, &total));
  long long mx = -1;
  if (first <= n) {
    unsigned long long pos = ex.cnt;
    if (pend && ex.last == SIG_DIGIT) e.walks |= 1u << (__ffs(m.nl) - 1);
    uint32_t out = e.ids | e.walks;
    while (out) {  // outputs in text order
      const int j = __ffs(out) - 1;
      out &= out - 1;
      if ((e.walks >> j) & 1u) {
        tokens[pos++] = -1;
        continue;
      }
      // the id ending at byte j: its length from the digit mask when it starts inside this
      // thread's bytes, else by reading back over the bytes before them (at most eleven);
      // its last nine digits are loaded at once and summed in 32 bits, then a tenth (an
      // eleventh digit, or a ten-digit value above 2^31 - 1, is an error)
      const uint32_t nondig = ~m.dig & ((1u << j) - 1u);
      int L;
      if (nondig) {
        L = j - (31 - __clz(nondig));
      } else {
        L = j + 1;
        while (L < 11 && is_digit(my[j - L])) L++;
      }
      uint32_t low = 0;
#pragma unroll
      for (int t = 0; t < 9; t++) {
        const uint32_t dgt = (uint32_t)(my[j - t] - '0');  // bytes down to my[-8]: halo or earlier threads
        low += t < L ? dgt * kPow10[t] : 0u;
      }
      uint32_t val = low;
      if (L >= 10) {
        const uint32_t top = (uint32_t)(my[j - 9] - '0');
        if (L > 10 || top > 2u || (top == 2u && low > 147483647u)) {
          if (bad < 0) bad = first + j;
          val = 0;
        } else {
          val = top * 1000000000u + low;
        }
      }
      tokens[pos++] = (int32_t)val;
      mx = (long long)val > mx ? (long long)val : mx;
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

// scratch: tile Spans, tile prefixes (+ the whole text), the error and largest-id words
// (64 bytes), then the group totals and group prefixes (+ the whole text)
size_t ingest_scratch_bytes(int64_t n) {
  const int64_t ntiles = (n + 1 + kIngTile - 1) / kIngTile, ngroups = (ntiles + kScanBlock - 1) / kScanBlock;
  return sizeof(Span) * (size_t)(2 * ntiles + 1) + 64 + sizeof(Span) * (size_t)(2 * ngroups + 1);
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
  const bool aligned = (reinterpret_cast<uintptr_t>(bytes) & 15) == 0;
  ingest_count_kernel<<<(unsigned)ntiles, kIngThreads, 0, s>>>(bytes, n, aligned, tile_span, err);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // tile prefixes in two levels: within groups of kScanBlock tiles (one block each), the
  // group totals by one block, then the group prefixes added to the tiles'
  const int64_t ngroups = (ntiles + kScanBlock - 1) / kScanBlock;
  Span* group_tot = reinterpret_cast<Span*>(reinterpret_cast<char*>(prefix + ntiles + 1) + 64);
  Span* group_pre = group_tot + ngroups;
  ingest_scan_groups_kernel<<<(unsigned)ngroups, kScanBlock, 0, s>>>(tile_span, ntiles, prefix, group_tot);
  ingest_scan_kernel<<<1, kScanBlock, 0, s>>>(group_tot, ngroups, group_pre);
  ingest_scan_add_kernel<<<(unsigned)std::min<int64_t>((ntiles + 256) / 256, 152 * 8), 256, 0, s>>>(
      prefix, ntiles, group_pre, ngroups);
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
  const bool aligned = (reinterpret_cast<uintptr_t>(bytes) & 15) == 0;
  ingest_emit_kernel<<<(unsigned)ntiles, kIngThreads, 0, s>>>(bytes, n, aligned, prefix, tokens, err, mx);
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
