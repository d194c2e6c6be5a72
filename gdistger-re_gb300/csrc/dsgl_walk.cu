// dsgl_walk.cu -- the corpus producer in front of the trainer: DistGER's
// information-oriented random walk (InCoM; include/walk.hpp:260-387 for the
// entropy/length correlation, :818-1042 for the walker loop) and the per-edge
// common-neighbour counts it reads (candidate->data, walk.hpp:920; the reference loads
// them from a file, graph.hpp:826).
//
// Random source.  The reference draws from std::mt19937 seeded by std::random_device and
// from rand(), so no run can be reproduced; here walker w draws from its own SplitMix64
// stream (Steele, Lea and Flood 2014): r_k = mix64(base_w + k G), base_w = mix64(seed ^
// w G), G = 0x9E3779B97F4A7C15.  A neighbour index is (r >> 32) * deg >> 32 (Lemire's
// multiply-shift); a uniform double is (r >> 11) 2^-53.  Walker w starts at w % V
// (walk.hpp:503-506); the corpus lists walks in walker order, -1 after each.
//
// One move from vertex c of degree ds: ds == 0 ends the walk; u = adj[c][index]; ds == 2
// with adj[c][0] == c ends it; before the first move u == c draws again (at most 64 times
// in a row, then the walk ends -- the reference spins forever there); p = uniform;
// pa = ((1 / (ds - cn)) max(ds, du)) / min(ds, du); trace = tanh(pa) <= p; u is appended,
// then c again on a trace; the walk moves to u only without one.  With trace steps off
// there is no p draw and every move goes on to u.  Every appended vertex
// updates the correlation state (Correlation::iterate, step 1) with f = its earlier visits,
// and the walk stops after more than min_length moves once R*R < r_threshold or R < 0
// (walk.hpp:868-874), or when it holds max_length vertices.
//
// Arithmetic: IEEE double through explicit _rn intrinsics (no contraction), so every
// decision equals the CPU restatement's bit for bit.  x log2 x comes from a host-built
// table of integers; tanh is (E - 1) / (E + 1) with E = exp(2x) = 2^k exp(r), Cody-Waite
// reduction with ln 2 split into its float head and the remainder, exp(r) by Taylor's
// series to r^13 (Horner); tanh(x) = 1 for x >= 20.
//
// Kernels: one warp per directed edge for the common-neighbour counts (lanes binary-search
// the shorter list's entries in the longer one); one thread per walker for the walks, its
// path history in shared memory (column-major by thread, so a warp scanning position i
// reads 32 consecutive words).  The walks run twice -- lengths, then, after an exclusive
// scan of length + 1, the tokens at their offsets -- so no per-walk buffer is needed.
#include <cuda_runtime.h>

#include <cstdint>

#include "sgns_internal.h"

namespace sgns {
namespace {

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ULL;
constexpr int kMaxRedraws = 64;
constexpr int kScanBlock = 1024;

__device__ __forceinline__ double pow2i(int k) { return __longlong_as_double((long long)(1023 + k) << 52); }

__device__ __forceinline__ double tanh_pos(double x) {
  if (!(x < 20.0)) return 1.0;
  const double y = __dmul_rn(2.0, x);
  const double ln2_hi = (double)(float)0.6931471805599453;
  const double ln2_lo = 0.6931471805599453 - ln2_hi;
  const int k = __double2int_rz(__dadd_rn(__dmul_rn(y, 1.4426950408889634), 0.5));
  const double kd = (double)k;
  const double r = __dsub_rn(__dsub_rn(y, __dmul_rn(kd, ln2_hi)), __dmul_rn(kd, ln2_lo));
  const double c[14] = {1.0,         1.0,          1.0 / 2.0,      1.0 / 6.0,       1.0 / 24.0,
                        1.0 / 120.0, 1.0 / 720.0,  1.0 / 5040.0,   1.0 / 40320.0,   1.0 / 362880.0,
                        1.0 / 3628800.0, 1.0 / 39916800.0, 1.0 / 479001600.0, 1.0 / 6227020800.0};
  double p = c[13];
#pragma unroll
  for (int i = 12; i >= 0; i--) p = __dadd_rn(__dmul_rn(p, r), c[i]);
  const double E = __dmul_rn(p, pow2i(k));
  return __ddiv_rn(__dsub_rn(E, 1.0), __dadd_rn(E, 1.0));
}

struct Corr {
  double H, EH, ES, EHS, EHH, ESS, N, R;
};

// Correlation::iterate (walk.hpp:330-365) with step 1; S = the walk's vertex count
__device__ __forceinline__ void corr_iterate(Corr& c, const double* __restrict__ xl, int S, int f) {
  const double t = __dsub_rn(__dadd_rn(__dsub_rn(__ldg(&xl[S]), __ldg(&xl[S + 1])), __ldg(&xl[f + 1])), __ldg(&xl[f]));
  const double S0 = (double)S, S1 = (double)(S + 1);
  const double H1 = __ddiv_rn(__dsub_rn(__dmul_rn(S0, c.H), t), S1);
  const double N1 = __dadd_rn(c.N, 1.0);
  c.EH = __dadd_rn(c.EH, __ddiv_rn(__dsub_rn(H1, c.EH), N1));
  c.ES = __dadd_rn(c.ES, __ddiv_rn(__dsub_rn(S1, c.ES), N1));
  c.EHS = __dadd_rn(c.EHS, __ddiv_rn(__dsub_rn(__dmul_rn(H1, S1), c.EHS), N1));
  c.EHH = __dadd_rn(c.EHH, __ddiv_rn(__dsub_rn(__dmul_rn(H1, H1), c.EHH), N1));
  c.ESS = __dadd_rn(c.ESS, __ddiv_rn(__dsub_rn(__dmul_rn(S1, S1), c.ESS), N1));
  const double DH = __dsub_rn(c.EHH, __dmul_rn(c.EH, c.EH));
  const double DS = __dsub_rn(c.ESS, __dmul_rn(c.ES, c.ES));
  const double ex = __dsub_rn(c.EHS, __dmul_rn(c.EH, c.ES));
  c.R = ex == 0.0 ? 0.0 : __ddiv_rn(ex, __dsqrt_rn(__dmul_rn(DH, DS)));
  c.H = H1;
  c.N = N1;
}

struct WalkArgs {
  const int64_t* indptr;
  const int32_t* indices;
  const int32_t* cn;
  const double* xl;
  int64_t V, walker_num;
  int32_t min_length, max_length;
  double r_threshold;
  uint64_t seed;
  int32_t trace;           // 1: the trace step of walk.hpp:920-1031; 0: moves only
  int32_t* lengths;        // pass 1 output
  const int64_t* offsets;  // pass 2 input (exclusive scan of length + 1)
  int32_t* corpus;         // pass 2 output
};

// kWrite = false: lengths[w]; kWrite = true: the walk's tokens and its -1 at offsets[w].
template <bool kWrite>
__global__ void __launch_bounds__(256) info_walk_kernel(WalkArgs a) {
  extern __shared__ int32_t hist_s[];  // [max_length][blockDim.x]
  const int T = blockDim.x, tid = threadIdx.x;
  int32_t* hist = hist_s + tid;
  for (int64_t w = (int64_t)blockIdx.x * T + tid; w < a.walker_num; w += (int64_t)gridDim.x * T) {
    const int64_t start = w % a.V;
    uint64_t ctr = mix64(a.seed ^ ((uint64_t)w * kGolden));
    int len = 1;
    hist[0] = (int32_t)start;
    Corr c{0.0, 0.0, 1.0, 0.0, 0.0, 1.0, 1.0, 1.0};
    int steps = 0, redraws = 0;
    int64_t cur = start;
    bool done = len >= a.max_length;
    // appends v; returns true when the walk stops there
    auto append = [&](int32_t v) -> bool {
      int f = 0;
      for (int i = 0; i < len; i++) f += hist[i * T] == v;
      corr_iterate(c, a.xl, len, f);
      hist[len * T] = v;
      len++;
      steps++;
      if (steps > a.min_length && (__dmul_rn(c.R, c.R) < a.r_threshold || c.R < 0.0)) return true;
      return len >= a.max_length;
    };
    while (!done) {
      const int64_t b = __ldg(&a.indptr[cur]);
      const int64_t ds = __ldg(&a.indptr[cur + 1]) - b;
      if (ds == 0) break;
      uint64_t r = mix64(ctr);
      ctr += kGolden;
      const int64_t e = b + (int64_t)(((r >> 32) * (uint64_t)ds) >> 32);
      const int32_t u = __ldg(&a.indices[e]);
      if (ds == 2 && __ldg(&a.indices[b]) == cur) break;
      if (steps == 0 && u == cur) {
        if (++redraws >= kMaxRedraws) break;
        continue;
      }
      bool trace = false;
      if (a.trace) {
        r = mix64(ctr);
        ctr += kGolden;
        const double p = __dmul_rn((double)(r >> 11), 1.0 / 9007199254740992.0);
        const int64_t du = __ldg(&a.indptr[(int64_t)u + 1]) - __ldg(&a.indptr[u]);
        const int64_t mx = ds > du ? ds : du, mn = ds < du ? ds : du;
        const double pa =
            __ddiv_rn(__dmul_rn(__ddiv_rn(1.0, (double)(ds - __ldg(&a.cn[e]))), (double)mx), (double)mn);
        trace = tanh_pos(pa) <= p;
      }
      if (append(u)) break;
      if (trace) {
        if (append((int32_t)cur)) break;
      } else {
        cur = u;
      }
    }
    if (!kWrite) {
      a.lengths[w] = len;
    } else {
      int32_t* out = a.corpus + a.offsets[w];
      for (int i = 0; i < len; i++) out[i] = hist[i * T];
      out[len] = -1;
    }
  }
}

// ---- exclusive scan of (lengths[w] + 1) into offsets[0..n] (int64) -------------------
__device__ __forceinline__ int64_t block_inclusive_scan(int64_t v, int64_t* warp_sums) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) warp_sums[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int64_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xFFFFFFFFu, s, o);
      if (lane >= o) s += t;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  if (wid > 0) v += warp_sums[wid - 1];
  return v;
}

__global__ void __launch_bounds__(kScanBlock) scan_tiles_kernel(const int32_t* lengths, int64_t n, int64_t* offsets,
                                                                int64_t* tile_sums) {
  __shared__ int64_t ws[32];
  const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  const int64_t v = i < n ? (int64_t)lengths[i] + 1 : 0;
  const int64_t inc = block_inclusive_scan(v, ws);
  if (i < n) offsets[i] = inc - v;  // exclusive within the tile
  if (threadIdx.x == kScanBlock - 1) tile_sums[blockIdx.x] = inc;
}

// one block: exclusive scan of the tile sums in rounds of kScanBlock; tile_sums[n_tiles]
// receives the total
__global__ void __launch_bounds__(kScanBlock) scan_tile_sums_kernel(int64_t* tile_sums, int64_t n_tiles) {
  __shared__ int64_t ws[32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < n_tiles; base += kScanBlock) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = i < n_tiles ? tile_sums[i] : 0;
    const int64_t inc = block_inclusive_scan(v, ws);
    const int64_t c0 = carry;
    if (i < n_tiles) tile_sums[i] = c0 + inc - v;
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1) carry = c0 + inc;
    __syncthreads();
  }
  if (threadIdx.x == 0) tile_sums[n_tiles] = carry;
}

__global__ void add_tile_offsets_kernel(int64_t* offsets, int64_t n, const int64_t* tile_sums, int64_t n_tiles) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) offsets[i] += tile_sums[i / kScanBlock];
  if (i == 0) offsets[n] = tile_sums[n_tiles];
}

// ---- common-neighbour counts ----------------------------------------------------------
// One warp per directed edge e = (u, v): u is found by binary search in indptr; lanes take
// entries of the shorter adjacency list and binary-search them in the longer one.
// status bits: 1 = a neighbour outside [0, V), 2 = an adjacency list not strictly increasing.
__global__ void __launch_bounds__(256) edge_cn_kernel(const int64_t* __restrict__ indptr,
                                                      const int32_t* __restrict__ indices, int64_t V, int64_t E,
                                                      int32_t* __restrict__ cn, int32_t* status) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < E; e += warps) {
    int64_t lo = 0, hi = V;  // the largest u with indptr[u] <= e
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (__ldg(&indptr[mid]) <= e) lo = mid;
      else hi = mid;
    }
    const int64_t u = lo;
    const int32_t v = __ldg(&indices[e]);
    const int64_t ub = __ldg(&indptr[u]), ue = __ldg(&indptr[u + 1]);
    if (v < 0 || v >= V) {
      if (lane == 0) atomicOr(status, 1);
      if (lane == 0) cn[e] = 0;
      continue;
    }
    if (lane == 0 && e > ub && __ldg(&indices[e - 1]) >= v) atomicOr(status, 2);
    const int64_t vb = __ldg(&indptr[v]), ve = __ldg(&indptr[v + 1]);
    const bool u_short = ue - ub <= ve - vb;
    const int64_t sb = u_short ? ub : vb, se = u_short ? ue : ve;
    const int64_t lb = u_short ? vb : ub, le = u_short ? ve : ue;
    int c = 0;
    for (int64_t i = sb + lane; i < se; i += 32) {
      const int32_t x = __ldg(&indices[i]);
      int64_t l = lb, h = le;  // first position with indices >= x
      while (l < h) {
        const int64_t m = (l + h) >> 1;
        if (__ldg(&indices[m]) < x) l = m + 1;
        else h = m;
      }
      c += (l < le && __ldg(&indices[l]) == x);
    }
    c = __reduce_add_sync(0xFFFFFFFFu, c);
    if (lane == 0) cn[e] = c;
  }
}

// CSR checks before any kernel follows the graph's pointers.  status bits: 4 = indptr[0]
// != 0, indptr[V] != E or indptr decreasing; 1 = a neighbour outside [0, V).
__global__ void __launch_bounds__(256) validate_csr_kernel(const int64_t* __restrict__ indptr,
                                                           const int32_t* __restrict__ indices, int64_t V, int64_t E,
                                                           int32_t* status) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t u = t0; u <= V; u += stride) {
    const int64_t x = indptr[u];
    const bool bad = (u == 0 && x != 0) || (u == V && x != E) || (u > 0 && indptr[u - 1] > x);
    if (bad) atomicOr(status, 4);
  }
  for (int64_t e = t0; e < E; e += stride) {
    const int32_t v = indices[e];
    if (v < 0 || v >= V) atomicOr(status, 1);
  }
}

}  // namespace

cudaError_t launch_validate_csr(const int64_t* indptr, const int32_t* indices, int64_t V, int64_t E,
                                int32_t* status, int num_sms, cudaStream_t s) {
  const int64_t want = ((V > E ? V : E) + 256) / 256;
  const int64_t cap = (int64_t)num_sms * 16;
  validate_csr_kernel<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(indptr, indices, V, E, status);
  return cudaGetLastError();
}

int walk_block_threads(int max_length) {
  // history words per thread: max_length; at most 96 KB of shared memory per block
  int t = (96 * 1024) / (4 * max_length);
  t = t >= 256 ? 256 : (t / 32) * 32;
  return t < 32 ? 32 : t;
}

size_t walk_scratch_bytes(int64_t walker_num) {
  const int64_t tiles = (walker_num + kScanBlock - 1) / kScanBlock;
  return sizeof(int32_t) * (size_t)walker_num + sizeof(int64_t) * (size_t)(walker_num + 1) +
         sizeof(int64_t) * (size_t)(tiles + 1) + 64;
}

// Pass 1 (lengths) and the scan; *offsets_out points into scratch (walker_num + 1 entries,
// the last = total tokens).
cudaError_t launch_info_walks_count(const int64_t* indptr, const int32_t* indices, const int32_t* cn,
                                    const double* xl, int64_t V, int64_t walker_num, int min_length,
                                    int max_length, double r_threshold, uint64_t seed, int trace, void* scratch,
                                    int num_sms, int64_t** offsets_out, cudaStream_t s) {
  char* p = static_cast<char*>(scratch);
  int64_t* offsets = reinterpret_cast<int64_t*>(p);
  p += sizeof(int64_t) * (size_t)(walker_num + 1);
  const int64_t tiles = (walker_num + kScanBlock - 1) / kScanBlock;
  int64_t* tile_sums = reinterpret_cast<int64_t*>(p);
  p += sizeof(int64_t) * (size_t)(tiles + 1);
  int32_t* lengths = reinterpret_cast<int32_t*>(p);
  WalkArgs a{indptr, indices, cn, xl, V, walker_num, min_length, max_length, r_threshold, seed, trace, lengths,
             nullptr, nullptr};
  const int T = walk_block_threads(max_length);
  const size_t smem = sizeof(int32_t) * (size_t)T * max_length;
  cudaError_t e = cudaFuncSetAttribute(info_walk_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(info_walk_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, info_walk_kernel<false>, T, smem);
  if (e != cudaSuccess) return e;
  const int64_t want = (walker_num + T - 1) / T;
  const int64_t resident = (int64_t)num_sms * (per_sm > 0 ? per_sm : 1);
  const unsigned grid = (unsigned)(want < resident * 8 ? want : resident * 8);
  info_walk_kernel<false><<<grid, T, smem, s>>>(a);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  scan_tiles_kernel<<<(unsigned)tiles, kScanBlock, 0, s>>>(lengths, walker_num, offsets, tile_sums);
  scan_tile_sums_kernel<<<1, kScanBlock, 0, s>>>(tile_sums, tiles);
  add_tile_offsets_kernel<<<(unsigned)((walker_num + 256) / 256), 256, 0, s>>>(offsets, walker_num, tile_sums, tiles);
  *offsets_out = offsets;
  return cudaGetLastError();
}

// Pass 2: the walks again, written at their offsets.
cudaError_t launch_info_walks_emit(const int64_t* indptr, const int32_t* indices, const int32_t* cn,
                                   const double* xl, int64_t V, int64_t walker_num, int min_length, int max_length,
                                   double r_threshold, uint64_t seed, int trace, const int64_t* offsets,
                                   int32_t* corpus, int num_sms, cudaStream_t s) {
  WalkArgs a{indptr, indices, cn, xl, V, walker_num, min_length, max_length, r_threshold, seed, trace, nullptr,
             offsets, corpus};
  const int T = walk_block_threads(max_length);
  const size_t smem = sizeof(int32_t) * (size_t)T * max_length;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, info_walk_kernel<true>, T, smem);
  if (e != cudaSuccess) return e;
  const int64_t want = (walker_num + T - 1) / T;
  const int64_t resident = (int64_t)num_sms * (per_sm > 0 ? per_sm : 1);
  const unsigned grid = (unsigned)(want < resident * 8 ? want : resident * 8);
  info_walk_kernel<true><<<grid, T, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_edge_common_neighbors(const int64_t* indptr, const int32_t* indices, int64_t V, int64_t E,
                                         int32_t* cn, int32_t* status, int num_sms, cudaStream_t s) {
  if (E == 0) return cudaSuccess;
  const int64_t want = (E * 32 + 255) / 256;
  const int64_t cap = (int64_t)num_sms * 64;
  edge_cn_kernel<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(indptr, indices, V, E, cn, status);
  return cudaGetLastError();
}

}  // namespace sgns
