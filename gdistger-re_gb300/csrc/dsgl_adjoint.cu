// dsgl_adjoint.cu -- SGNS loss and its hand-written adjoint with sparse row gradients.
//
// The loss of one minibatch of the reference step (include/dsgl.hpp:1136-1272) is
//   L = sum_i sum_j meta_i * softplus(-(2 l_ij - 1) f_ij),   f_ij = <Woh[o_i], Wih[x_j]>,
// with l_ij = 1 for (i = 0, j < first) and (i = O-1, j >= first), else 0.  Its adjoint
//   dL/df_ij = meta_i (sigma(f_ij) - l_ij),
//   dL/dWih[x_j] += sum_i dL/df_ij Woh[o_i],   dL/dWoh[o_i] += sum_j dL/df_ij Wih[x_j],
// is the negative of the reference's update direction divided by alpha (the reference
// uses its 1000-entry sigmoid table; the adjoint uses the exact sigmoid so it can be
// checked against finite differences).
//
// Sparse output: every row referenced by the batch appears once, in ascending row order.
// Rows are marked in a V-sized array, the marks are prefix-summed (row -> compact slot),
// the compact gradient rows are zeroed, and each minibatch adds its row gradients into
// its rows' slots.
//
// Gradient kernels.  adjoint_pipe_kernel (tables whose rows are whole 16-byte chunks at
// 16-byte aligned addresses) runs persistent warps that copy the next minibatch's rows
// into shared memory with cp.async while the current one computes, when both fit in the
// warp's ring of rows (its comment below gives the details).  adjoint_kernel takes every other shape, one warp per
// minibatch and four per block:
//   * rows are staged in shared memory with 16-byte loads (8 bytes per 4 bf16 elements),
//     input rows padded to a stride of d + 4 words so lanes reading different rows at the
//     same column fall in different banks;
//   * the dot products run one lane per input (lane j holds f_ij for every output i,
//     summed over k in order), reading its own padded row and the output rows by broadcast;
//   * the gradient rows are column-parallel (lane l owns columns 4l..4l+3 of each
//     128-column chunk) and leave with one 16-byte atomic add per lane (red.global.add of
//     four floats; fp64 adds element by element);
//   * the loss is reduced per warp, then per block, with one fp64 atomic per block;
//   * sizes and ids are checked on the device (status bits), so a call makes no host round
//     trip before its launches.
#include <cuda_runtime.h>

#include <algorithm>

#include "dsgl_device.cuh"

namespace sgns {

namespace {

constexpr int kWarpsPerBlock = 4;
// status bits: 1 = an id outside [0, V); 2 = a minibatch outside the size limits
constexpr int kBadId = 1, kBadSize = 2;

template <int DT> struct Elem;
template <> struct Elem<0> {  // fp32 tables
  typedef float T;
  __device__ static __forceinline__ void load4(const void* p, int64_t i, T (&v)[4]) {
    const float4 f = *reinterpret_cast<const float4*>(static_cast<const float*>(p) + i);
    v[0] = f.x, v[1] = f.y, v[2] = f.z, v[3] = f.w;
  }
  __device__ static __forceinline__ T get(const void* p, int64_t i) { return static_cast<const float*>(p)[i]; }
};
template <> struct Elem<1> {  // bf16 tables, fp32 arithmetic
  typedef float T;
  __device__ static __forceinline__ void load4(const void* p, int64_t i, T (&v)[4]) {
    const uint2 u = *reinterpret_cast<const uint2*>(static_cast<const uint16_t*>(p) + i);
    v[0] = __uint_as_float(u.x << 16), v[1] = __uint_as_float(u.x & 0xFFFF0000u);
    v[2] = __uint_as_float(u.y << 16), v[3] = __uint_as_float(u.y & 0xFFFF0000u);
  }
  __device__ static __forceinline__ T get(const void* p, int64_t i) { return bf16_bits_to_f32(static_cast<const uint16_t*>(p)[i]); }
};
template <> struct Elem<2> {  // fp64 tables and arithmetic
  typedef double T;
  __device__ static __forceinline__ void load4(const void* p, int64_t i, T (&v)[4]) {
    const double2 a = *reinterpret_cast<const double2*>(static_cast<const double*>(p) + i);
    const double2 b = *reinterpret_cast<const double2*>(static_cast<const double*>(p) + i + 2);
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
  }
  __device__ static __forceinline__ T get(const void* p, int64_t i) { return static_cast<const double*>(p)[i]; }
};

// loss term and coefficient of one pair from one exponential: with e = exp(-|f|),
// softplus(z) = max(z, 0) + log1p(e) for z = +-f, and sigma(f) = 1 / (1 + e) (f >= 0) or
// e / (1 + e) (f < 0)
__device__ __forceinline__ void pair_terms(float f, int label, float meta, float& loss, float& coef) {
  const float e = expf(-fabsf(f));
  const float z = label ? -f : f;
  loss += meta * (fmaxf(z, 0.f) + log1pf(e));
  const float r = 1.0f / (1.0f + e);
  coef = meta * ((f >= 0.f ? r : e * r) - (float)label);
}
__device__ __forceinline__ void pair_terms(double f, int label, double meta, double& loss, double& coef) {
  const double e = exp(-fabs(f));
  const double z = label ? -f : f;
  loss += meta * (fmax(z, 0.0) + log1p(e));
  const double r = 1.0 / (1.0 + e);
  coef = meta * ((f >= 0.0 ? r : e * r) - (double)label);
}

__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }

__device__ __forceinline__ void atomic_add4(float* dst, const float (&v)[4]) {
  atomicAdd(reinterpret_cast<float4*>(dst), make_float4(v[0], v[1], v[2], v[3]));
}
__device__ __forceinline__ void atomic_add4(double* dst, const double (&v)[4]) {
#pragma unroll
  for (int k = 0; k < 4; k++) atomicAdd(dst + k, v[k]);
}

// Marks the rows of every minibatch (one warp per minibatch, one lane per id), checks its
// extents and records the largest input and output counts (dims[0], dims[1]).
__global__ void mark_rows_kernel(int n, const int32_t* in_ptr, const int32_t* in_ids, const int32_t* in_first,
                                 const int32_t* out_ptr, const int32_t* out_ids, int64_t V, int32_t* mark_in,
                                 int32_t* mark_out, int32_t* status, int32_t* dims) {
  const int lane = lane_id();
  const int warps = (int)((gridDim.x * blockDim.x) >> 5);
  int imax = 0, omax = 0;
  for (int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); b < n; b += warps) {
    const int i0 = in_ptr[b], i1 = in_ptr[b + 1], o0 = out_ptr[b], o1 = out_ptr[b + 1];
    if (i0 < 0 || o0 < 0 || i1 - i0 < 0 || i1 - i0 > kIMax || o1 - o0 < 0 || o1 - o0 > kOMax ||
        in_first[b] < 0 || in_first[b] > i1 - i0) {
      if (lane == 0) atomicOr(status, kBadSize);
      continue;
    }
    imax = max(imax, i1 - i0);
    omax = max(omax, o1 - o0);
    for (int t = i0 + lane; t < i1; t += 32) {
      const int32_t r = in_ids[t];
      if (r < 0 || r >= V) atomicOr(status, kBadId);
      else mark_in[r] = 1;
    }
    for (int t = o0 + lane; t < o1; t += 32) {
      const int32_t r = out_ids[t];
      if (r < 0 || r >= V) atomicOr(status, kBadId);
      else mark_out[r] = 1;
    }
  }
  imax = __reduce_max_sync(kFull, imax);
  omax = __reduce_max_sync(kFull, omax);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&dims[0], imax);
    atomicMax(&dims[1], omax);
  }
}

// ---- inclusive scan of int32 marks: tiles of 4096, then the tile sums in one block -----
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int32_t block_exclusive_prefix(int32_t run, int32_t* warp_sums, int32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t x = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int32_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
      if (lane >= o) s += y;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  *total = warp_sums[31];
  return (x - run) + (warp > 0 ? warp_sums[warp - 1] : 0);
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(int32_t* a, int64_t n, int32_t* tile_sums) {
  __shared__ int32_t warp_sums[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t run = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = base + k < n ? a[base + k] : 0;
    run += v[k];
    v[k] = run;
  }
  int32_t total;
  const int32_t prefix = block_exclusive_prefix(run, warp_sums, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    if (base + k < n) a[base + k] = v[k] + prefix;
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// one block: tile sums -> exclusive tile prefixes, in rounds of kScanThreads
__global__ void __launch_bounds__(kScanThreads) scan_tile_sums_kernel(int32_t* tile_sums, int64_t ntiles) {
  __shared__ int32_t warp_sums[32];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < ntiles; base += kScanThreads) {
    const int64_t i = base + threadIdx.x;
    const int32_t v = i < ntiles ? tile_sums[i] : 0;
    int32_t total;
    const int32_t ex = block_exclusive_prefix(v, warp_sums, &total);
    const int32_t c0 = carry;
    if (i < ntiles) tile_sums[i] = c0 + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry = c0 + total;
    __syncthreads();
  }
}

// adds the tile prefixes; marked rows (incl[r] - incl[r-1] == 1) -> ids[incl[r] - 1] = r
// (the previous row's value is recomputed from its own tile prefix, so one pass suffices)
__global__ void add_prefix_emit_kernel(const int32_t* a, int64_t n, const int32_t* tile_prefix, int32_t* ids) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = a[i] + tile_prefix[i / kScanTile];
    const int32_t prev = i == 0 ? 0 : a[i - 1] + tile_prefix[(i - 1) / kScanTile];
    if (v != prev) ids[v - 1] = (int32_t)i;
  }
}

// final pass: a[i] += its tile prefix (after the ids were emitted from the tile-local values)
__global__ void add_prefix_kernel(int32_t* a, int64_t n, const int32_t* tile_prefix) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] += tile_prefix[i / kScanTile];
}

// zeroes the first incl[V-1] rows of a gradient array (the rows the call emits)
template <class T>
__global__ void zero_rows_kernel(T* g, const int32_t* incl_last, int d) {
  const int64_t n = (int64_t)(*incl_last) * d;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    g[i] = T(0);
}

// Shared memory of one warp: input rows (imax x DP), output rows (omax x d), coefficients
// (omax x imax), row slots (imax + omax ints stored as T), rounded up to 16 bytes.
__host__ __device__ inline size_t adjoint_warp_elems(int d, int imax, int omax) {
  const size_t e = (size_t)imax * (d + 4) + (size_t)omax * d + (size_t)omax * imax + (size_t)(imax + omax);
  return (e + 3) & ~(size_t)3;
}

// four consecutive elements of a shared-memory row (16-byte aligned)
__device__ __forceinline__ void lds4(const float* p, float (&v)[4]) {
  const float4 f = *reinterpret_cast<const float4*>(p);
  v[0] = f.x, v[1] = f.y, v[2] = f.z, v[3] = f.w;
}
__device__ __forceinline__ void lds4(const double* p, double (&v)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
}
__device__ __forceinline__ void sts4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void sts4(double* p, const double (&v)[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}

// One warp per minibatch.  OMX: output-row capacity of the register arrays (7 covers K <= 5).
// VW: elements per column group (4 when d % 4 == 0, else 1).  loss_parts: 256 fp64 partial
// sums (warp b adds to slot b % 256), summed by finish_loss_kernel.
template <int DT, int VW, int OMX>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) adjoint_kernel(
    int d, int n, int imax, int omax, const int32_t* in_ptr, const int32_t* in_ids, const int32_t* in_first,
    const int32_t* out_ptr, const int32_t* out_ids, const int32_t* out_meta, const void* wih, const void* woh,
    int64_t V, const int32_t* incl_in, const int32_t* incl_out, typename Elem<DT>::T* g_in,
    typename Elem<DT>::T* g_out, double* loss_parts) {
  typedef typename Elem<DT>::T T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = lane_id(), wpb = blockDim.x >> 5;
  const int b = blockIdx.x * wpb + warp;
  if (b >= n) return;
  const int DP = d + 4;
  T* x = reinterpret_cast<T*>(smem_raw) + (size_t)warp * adjoint_warp_elems(d, imax, omax);
  T* o = x + (size_t)imax * DP;
  T* coef = o + (size_t)omax * d;
  int32_t* slot = reinterpret_cast<int32_t*>(coef + (size_t)omax * imax);  // inputs, then outputs
  const int i0 = in_ptr[b], I = in_ptr[b + 1] - i0, o0 = out_ptr[b], O = out_ptr[b + 1] - o0, first = in_first[b];
  // minibatches over the limits or with ids outside [0, V) were flagged by the marking
  // pass; they are skipped here
  bool ok = i0 >= 0 && o0 >= 0 && I >= 0 && I <= imax && O >= 0 && O <= omax && O <= OMX && first >= 0 &&
            first <= I;
  if (ok) {
    for (int j = lane; j < I + O; j += 32) {
      const int32_t r = j < I ? in_ids[i0 + j] : out_ids[o0 + j - I];
      ok &= r >= 0 && r < V;
      // the row's gradient slot, looked up now so the atomics below wait on nothing
      if (r >= 0 && r < V) slot[j] = (j < I ? incl_in[r] : incl_out[r]) - 1;
    }
  }
  if (!__all_sync(kFull, ok)) return;
  const int nq = d / VW;
  // stage the rows, eight at a time with every load in flight before its stores
  for (int u0 = 0; u0 < I + O; u0 += 8) {
    T v[8][4];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int j = u0 + u;
      if (j < I + O) {
        const int64_t r = j < I ? in_ids[i0 + j] : out_ids[o0 + j - I];
        const void* tab = j < I ? wih : woh;
        for (int q = lane; q < nq; q += 32) {  // one group per lane when d <= 128
          if (VW == 4) Elem<DT>::load4(tab, r * d + 4 * q, v[u]);
          else v[u][0] = Elem<DT>::get(tab, r * d + q);
          if (q + 32 < nq) {  // wider rows: store this group now, keep the loop simple
            T* dst = j < I ? x + (size_t)j * DP : o + (size_t)(j - I) * d;
            if (VW == 4) sts4(dst + 4 * q, v[u]);
            else dst[q] = v[u][0];
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int j = u0 + u;
      if (j < I + O) {
        int q = lane;
        while (q + 32 < nq) q += 32;  // the last group of this lane (held in v[u])
        if (q < nq) {
          T* dst = j < I ? x + (size_t)j * DP : o + (size_t)(j - I) * d;
          if (VW == 4) sts4(dst + 4 * q, v[u]);
          else dst[q] = v[u][0];
        }
      }
    }
  }
  __syncwarp();
  // dot products, one lane per input: f_ij for every output i, summed over k in order
  T loss = 0;
  for (int j0 = 0; j0 < I; j0 += 32) {
    const int j = j0 + lane;
    const T* xr = x + (size_t)(j < I ? j : 0) * DP;
    T f[OMX];
#pragma unroll
    for (int i = 0; i < OMX; i++) f[i] = 0;
    for (int k = 0; k < d; k += VW) {
      T xv[4];
      if (VW == 4) lds4(xr + k, xv);
      else xv[0] = xr[k];
#pragma unroll
      for (int i = 0; i < OMX; i++) {
        if (i < O) {
          T ov[4];
          if (VW == 4) lds4(o + (size_t)i * d + k, ov);
          else ov[0] = o[(size_t)i * d + k];
#pragma unroll
          for (int t = 0; t < VW; t++) f[i] = fma_t(ov[t], xv[t], f[i]);
        }
      }
    }
    if (j < I) {
#pragma unroll
      for (int i = 0; i < OMX; i++)
        if (i < O) coef[i * I + j] = f[i];
      for (int i = 0; i < O; i++) {
        const int label = j < first ? (i == 0) : (i == O - 1);
        T c;
        pair_terms(coef[i * I + j], label, (T)out_meta[o0 + i], loss, c);
        coef[i * I + j] = c;
      }
    }
  }
  __syncwarp();
  // dL/dWih[x_j] = sum_i coef_ij Woh[o_i], column-parallel
  for (int j = 0; j < I; j++) {
    T* dst = g_in + (size_t)slot[j] * d;
    for (int q = lane; q < nq; q += 32) {
      T acc[4] = {0, 0, 0, 0};
      for (int i = 0; i < O; i++) {
        const T c = coef[i * I + j];
        T ov[4];
        if (VW == 4) lds4(o + (size_t)i * d + 4 * q, ov);
        else ov[0] = o[(size_t)i * d + q];
#pragma unroll
        for (int t = 0; t < VW; t++) acc[t] = fma_t(c, ov[t], acc[t]);
      }
      if (VW == 4) atomic_add4(dst + 4 * q, acc);
      else atomicAdd(dst + q, acc[0]);
    }
  }
  // dL/dWoh[o_i] = sum_j coef_ij Wih[x_j]
  for (int i = 0; i < O; i++) {
    T* dst = g_out + (size_t)slot[I + i] * d;
    for (int q = lane; q < nq; q += 32) {
      T acc[4] = {0, 0, 0, 0};
      for (int j = 0; j < I; j++) {
        const T c = coef[i * I + j];
        T xv[4];
        if (VW == 4) lds4(x + (size_t)j * DP + 4 * q, xv);
        else xv[0] = x[(size_t)j * DP + q];
#pragma unroll
        for (int t = 0; t < VW; t++) acc[t] = fma_t(c, xv[t], acc[t]);
      }
      if (VW == 4) atomic_add4(dst + 4 * q, acc);
      else atomicAdd(dst + q, acc[0]);
    }
  }
  for (int sh = 16; sh > 0; sh >>= 1) loss += __shfl_xor_sync(kFull, loss, sh);
  if (lane == 0 && loss != 0) atomicAdd(&loss_parts[b & 255], (double)loss);
}

// ---- pipelined gradient kernel: tables whose rows are whole 16-byte chunks ----------------
// Persistent warps: warp g runs minibatches g, g + S, g + 2S, ... (S = warps in the grid).
// Each warp holds a ring of imax + omax rows (one largest minibatch).  After the forward,
// the next minibatch's rows are copied with cp.async (16 bytes per lane and copy, cached in
// L2 only) behind the current ones or at the ring's start when they fit beside them, so
// their gathers overlap the backward; otherwise they are copied once the backward is
// done.  A ring of one minibatch leaves room for more resident warps, which measured
// faster than a second full buffer (12 warps per SM against 7 at d = 128, bf16, K = 5:
// 2.08 against 2.86 ms per call on the 4M-vertex case).  The next minibatch's ids are
// loaded at the top of an iteration, its gradient slots with its copies, and the extents
// one minibatch further ahead.  Rows stay in their storage format in the ring (row stride
// = row bytes + 16, so lanes reading different rows at one column hit different banks);
// the output rows are widened once into an fp32 (fp64) copy for the forward's broadcast
// reads.  Sums keep the order of adjoint_kernel except the forward's dot products, which
// run as an even and an odd partial sum for fp32.

template <int DT> struct Pipe;
template <> struct Pipe<0> {  // fp32 rows: 4 elements per 16 bytes
  typedef float T;
  static constexpr int kBytes = 4;
  __device__ static __forceinline__ void chunk4(const unsigned char* p, float (&v)[4]) {  // 4 elements at p
    const float4 f = *reinterpret_cast<const float4*>(p);
    v[0] = f.x, v[1] = f.y, v[2] = f.z, v[3] = f.w;
  }
};
template <> struct Pipe<1> {  // bf16 rows
  typedef float T;
  static constexpr int kBytes = 2;
  __device__ static __forceinline__ void chunk4(const unsigned char* p, float (&v)[4]) {
    const uint2 u = *reinterpret_cast<const uint2*>(p);
    v[0] = __uint_as_float(u.x << 16), v[1] = __uint_as_float(u.x & 0xFFFF0000u);
    v[2] = __uint_as_float(u.y << 16), v[3] = __uint_as_float(u.y & 0xFFFF0000u);
  }
};
template <> struct Pipe<2> {  // fp64 rows
  typedef double T;
  static constexpr int kBytes = 8;
  __device__ static __forceinline__ void chunk4(const unsigned char* p, double (&v)[4]) {
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
  }
};

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Per-warp shared memory of the pipelined kernel, in bytes (every region 16-byte aligned):
// the ring of `ring` rows, the widened output rows, the coefficients
// (imax rows of round4(omax)) and the gradient slots.
struct PipeLayout {
  int RS, CS, buf, ofp, coef, slot, bytes;
};
__host__ __device__ inline PipeLayout pipe_layout(int dtype, int d, int imax, int omax, int omx, int ring) {
  const int eb = dtype == 2 ? 8 : dtype == 1 ? 2 : 4, tb = dtype == 2 ? 8 : 4;
  PipeLayout L;
  L.RS = d * eb + 16;
  L.CS = (omx + 3) & ~3;
  L.buf = ring * L.RS;
  L.ofp = L.buf;
  L.coef = L.ofp + omx * d * tb;
  L.slot = L.coef + imax * L.CS * tb;
  L.bytes = (L.slot + 4 * (imax + omax) + 15) & ~15;
  return L;
}

// minibatch extents: i0, I, o0, O, first
struct Extent {
  int i0, I, o0, O, first;
};
__device__ __forceinline__ Extent load_extent(int b, int n, const int32_t* in_ptr, const int32_t* in_first,
                                              const int32_t* out_ptr) {
  Extent e{0, 0, 0, 0, 0};
  if (b < n) {
    e.i0 = in_ptr[b], e.I = in_ptr[b + 1] - e.i0, e.o0 = out_ptr[b], e.O = out_ptr[b + 1] - e.o0;
    e.first = in_first[b];
  }
  return e;
}
// lane l holds the ids of rows l, l + 32 and l + 64 (inputs, then outputs)
__device__ __forceinline__ void load_ids(const Extent& e, bool valid, const int32_t* in_ids, const int32_t* out_ids,
                                         int (&id)[3]) {
  const int lane = lane_id();
#pragma unroll
  for (int m = 0; m < 3; m++) {
    const int j = lane + 32 * m;
    id[m] = !valid ? 0 : j < e.I ? in_ids[e.i0 + j] : j < e.I + e.O ? out_ids[e.o0 + j - e.I] : 0;
  }
}
__device__ __forceinline__ int row_id(const int (&id)[3], int r) {  // uniform or per-lane r < 96
  const int a = __shfl_sync(kFull, id[0], r & 31), b = __shfl_sync(kFull, id[1], r & 31),
            c = __shfl_sync(kFull, id[2], r & 31);
  return r < 32 ? a : r < 64 ? b : c;
}

// f = Out x X^T for one minibatch on the tensor cores (bf16 tables): A = the output rows
// (16 x 16 per MMA, rows past O zero), B = the input rows (8 inputs x 16 columns per MMA,
// "col" layout = each input row contiguous), both read as bf16 pairs straight from the
// ring (row stride RS = 2d + 16 bytes: the 32 lanes' words fall in 32 banks).  The
// products of bf16 values are exact in fp32 and the sums run in fp32, as in the lane-per-
// input form (in another order).  Thread (g = lane / 4, t = lane % 4) ends with f for
// outputs g and g + 8 and inputs 8n + 2t, 8n + 2t + 1 of tile n; it computes those pairs'
// loss terms and coefficients, so all 32 lanes work on them.  Coefficients of outputs
// O .. OMX-1 are zero (the backward runs over OMX outputs).
__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                               uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t lds_u32(const unsigned char* p) { return *reinterpret_cast<const uint32_t*>(p); }

template <int OMX>
__device__ __forceinline__ void forward_mma_bf16(const unsigned char* buf, int RS, int d, int I, int O, int first,
                                                 const int32_t* meta, float* coef, int CS, float& loss) {
  static_assert(OMX <= 16, "one MMA row block holds the outputs");
  const int lane = lane_id(), g = lane >> 2, t = lane & 3;
  for (int e = lane; e < I * OMX; e += 32) {  // zero coefficients past O
    const int j = e / OMX, i = e - j * OMX;
    if (i >= O) coef[(size_t)j * CS + i] = 0.f;
  }
  const float meta0 = g < O ? (float)meta[g] : 0.f, meta1 = g + 8 < O ? (float)meta[g + 8] : 0.f;
  const unsigned char* arow0 = buf + (size_t)(I + (g < O ? g : 0)) * RS + 4 * t;
  const unsigned char* arow1 = buf + (size_t)(I + (g + 8 < O ? g + 8 : 0)) * RS + 4 * t;
  const int ntiles = (I + 7) >> 3;
  for (int n0 = 0; n0 < ntiles; n0 += 4) {  // up to four tiles (32 inputs) per round
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int r = 0; r < 4; r++) acc[u][r] = 0.f;
    const unsigned char* brow[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int j = (n0 + u) * 8 + g;
      brow[u] = buf + (size_t)(j < I ? j : 0) * RS + 4 * t;
    }
    for (int k0 = 0; k0 < d; k0 += 16) {
      const int kb = 2 * k0;            // byte offset of column k0
      const bool hi = k0 + 8 < d;       // columns k0+8 .. k0+15 exist (d % 8 == 0)
      const uint32_t a0 = g < O ? lds_u32(arow0 + kb) : 0u;
      const uint32_t a2 = g < O && hi ? lds_u32(arow0 + kb + 16) : 0u;
      const uint32_t a1 = OMX > 8 && g + 8 < O ? lds_u32(arow1 + kb) : 0u;
      const uint32_t a3 = OMX > 8 && g + 8 < O && hi ? lds_u32(arow1 + kb + 16) : 0u;
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (n0 + u < ntiles) {  // uniform
          const uint32_t b0 = lds_u32(brow[u] + kb), b1 = hi ? lds_u32(brow[u] + kb + 16) : 0u;
          mma_bf16_16816(acc[u], a0, a1, a2, a3, b0, b1);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int i = g + 8 * h;
        if ((h == 1 && OMX <= 8) || i >= O) continue;
#pragma unroll
        for (int e = 0; e < 2; e++) {
          const int j = (n0 + u) * 8 + 2 * t + e;
          if (j < I) {
            const int label = j < first ? (i == 0) : (i == O - 1);
            float c;
            pair_terms(acc[u][2 * h + e], label, h ? meta1 : meta0, loss, c);
            coef[(size_t)j * CS + i] = c;
          }
        }
      }
    }
  }
}

template <int DT, int OMX>
__global__ void __launch_bounds__(256) adjoint_pipe_kernel(
    int d, int n, int imax, int omax, int ring, const int32_t* in_ptr, const int32_t* in_ids,
    const int32_t* in_first, const int32_t* out_ptr, const int32_t* out_ids, const int32_t* out_meta,
    const void* wih, const void* woh, int64_t V, const int32_t* incl_in, const int32_t* incl_out,
    typename Pipe<DT>::T* g_in,
    typename Pipe<DT>::T* g_out, double* loss_parts) {
  typedef typename Pipe<DT>::T T;
  constexpr int EB = Pipe<DT>::kBytes;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = lane_id(), wpb = blockDim.x >> 5;
  const int gw = blockIdx.x * wpb + (threadIdx.x >> 5), S = gridDim.x * wpb;
  const PipeLayout L = pipe_layout(DT, d, imax, omax, OMX, ring);
  unsigned char* wbase = smem_raw + (size_t)(threadIdx.x >> 5) * L.bytes;
  T* ofp = reinterpret_cast<T*>(wbase + L.ofp);
  T* coef = reinterpret_cast<T*>(wbase + L.coef);
  int32_t* slot = reinterpret_cast<int32_t*>(wbase + L.slot);
  const int row_bytes = d * EB, C = row_bytes >> 4;  // 16-byte chunks per row
  const int rpi = C <= 32 ? 32 / C : 1, lane_row = C <= 32 ? lane / C : 0, lane_chunk = C <= 32 ? lane % C : 0;
  const unsigned char* tin = static_cast<const unsigned char*>(wih);
  const unsigned char* tout = static_cast<const unsigned char*>(woh);

  // sizes within this launch's buffers and ids inside [0, V) (the marking pass flagged
  // any minibatch that is not; it is skipped)
  auto extent_ok = [&](const Extent& e) {
    return e.i0 >= 0 && e.o0 >= 0 && e.I >= 0 && e.I <= imax && e.O >= 0 && e.O <= omax && e.O <= OMX &&
           e.first >= 0 && e.first <= e.I;
  };
  auto ids_ok = [&](const Extent& e, const int (&id)[3]) {
    bool ok = true;
#pragma unroll
    for (int m = 0; m < 3; m++) ok &= lane + 32 * m >= e.I + e.O || (id[m] >= 0 && id[m] < V);
    return __all_sync(kFull, ok);
  };
  auto issue_copies = [&](const Extent& e, const int (&id)[3], unsigned char* buf) {
    const int R = e.I + e.O;
    if (C <= 32) {
      for (int r0 = 0; r0 < R; r0 += rpi) {
        const int r = r0 + lane_row;
        const int rid = row_id(id, r);
        if (lane_row < rpi && r < R)
          cp_async16(buf + (size_t)r * L.RS + 16 * lane_chunk,
                     (r < e.I ? tin : tout) + (int64_t)rid * row_bytes + 16 * lane_chunk);
      }
    } else {
      for (int r = 0; r < R; r++) {
        const int rid = row_id(id, r);
        for (int k = lane; k < C; k += 32)
          cp_async16(buf + (size_t)r * L.RS + 16 * k, (r < e.I ? tin : tout) + (int64_t)rid * row_bytes + 16 * k);
      }
    }
    cp_async_commit();
  };
  auto load_slots = [&](const Extent& e, const int (&id)[3], int (&sl)[3]) {
#pragma unroll
    for (int m = 0; m < 3; m++) {
      const int j = lane + 32 * m;
      sl[m] = j < e.I ? incl_in[id[m]] - 1 : j < e.I + e.O ? incl_out[id[m]] - 1 : 0;
    }
  };

  // prologue: the first minibatch's rows in flight, the second one's extent loaded
  int b = gw;
  Extent cur = load_extent(b, n, in_ptr, in_first, out_ptr);
  bool cur_ok = b < n && extent_ok(cur);
  int idc[3], slc[3] = {0, 0, 0};
  load_ids(cur, cur_ok, in_ids, out_ids, idc);
  cur_ok = cur_ok && ids_ok(cur, idc);
  if (cur_ok) {
    issue_copies(cur, idc, wbase);
    load_slots(cur, idc, slc);
  }
  Extent nxt = load_extent(b + S, n, in_ptr, in_first, out_ptr);
  int sc = 0;  // ring row of the current minibatch's first row
  T loss = 0;
  const int nq = d >> 2;
  while (b < n) {
    const int bn = b + S;
    bool nxt_ok = bn < n && extent_ok(nxt);
    int idn[3], sln[3] = {0, 0, 0};
    load_ids(nxt, nxt_ok, in_ids, out_ids, idn);
    const Extent nn = load_extent(bn + S, n, in_ptr, in_first, out_ptr);
    unsigned char* buf = wbase + (size_t)sc * L.RS;
    cp_async_wait_all();
    if (cur_ok) {
#pragma unroll
      for (int m = 0; m < 3; m++)
        if (lane + 32 * m < cur.I + cur.O) slot[lane + 32 * m] = slc[m];
    }
    __syncwarp();
    const int I = cur.I, O = cur.O;
    if (cur_ok) {
      // widen the output rows once (column-parallel); rows O .. OMX-1 are zero, so the
      // products below run over the kernel's full output capacity without tests
      for (int i = 0; i < OMX; i++)
        for (int q = lane; q < nq; q += 32) {
          T v[4] = {0, 0, 0, 0};
          if (i < O) Pipe<DT>::chunk4(buf + (size_t)(I + i) * L.RS + 4 * q * EB, v);
          sts4(ofp + (size_t)i * d + 4 * q, v);
        }
      __syncwarp();
      if constexpr (DT == 1) {
        forward_mma_bf16<OMX>(buf, L.RS, d, I, O, cur.first, out_meta + cur.o0, coef, L.CS, loss);
      } else {
        // dot products, one lane per input
        for (int j0 = 0; j0 < I; j0 += 32) {
          const int j = j0 + lane;
          const unsigned char* xr = buf + (size_t)(j < I ? j : 0) * L.RS;
          T f[OMX];
          if constexpr (DT == 2) {
  #pragma unroll
            for (int i = 0; i < OMX; i++) f[i] = 0;
            for (int k = 0; k < d; k += 4) {
              T xv[4];
              Pipe<DT>::chunk4(xr + k * EB, xv);
  #pragma unroll
              for (int i = 0; i < OMX; i++) {
                T ov[4];
                lds4(ofp + (size_t)i * d + k, ov);
  #pragma unroll
                for (int t = 0; t < 4; t++) f[i] = fma_t(ov[t], xv[t], f[i]);
              }
            }
          } else {
            // 16 bytes of the input row per step: 8 bf16 or 4 fp32 elements, even and odd
            // partial sums in packed fp32 pairs
            constexpr int VK = 16 / EB;
            float2 fp[OMX];
  #pragma unroll
            for (int i = 0; i < OMX; i++) fp[i] = make_float2(0.f, 0.f);
  #pragma unroll 2
            for (int k = 0; k < d; k += VK) {
              float xv[VK];
              Pipe<DT>::chunk4(xr + k * EB, *reinterpret_cast<float(*)[4]>(xv));
              if constexpr (VK == 8) Pipe<DT>::chunk4(xr + k * EB + 8, *reinterpret_cast<float(*)[4]>(xv + 4));
  #pragma unroll
              for (int i = 0; i < OMX; i++) {
  #pragma unroll
                for (int h = 0; h < VK; h += 4) {
                  const float4 o4 = *reinterpret_cast<const float4*>(ofp + (size_t)i * d + k + h);
                  fp[i] = __ffma2_rn(make_float2(o4.x, o4.y), make_float2(xv[h], xv[h + 1]), fp[i]);
                  fp[i] = __ffma2_rn(make_float2(o4.z, o4.w), make_float2(xv[h + 2], xv[h + 3]), fp[i]);
                }
              }
            }
  #pragma unroll
            for (int i = 0; i < OMX; i++) f[i] = __fadd_rn(fp[i].x, fp[i].y);
          }
          if (j < I) {
  #pragma unroll
            for (int i = 0; i < OMX; i++) {
              T c = 0;
              if (i < O) {
                const int label = j < cur.first ? (i == 0) : (i == O - 1);
                pair_terms(f[i], label, (T)out_meta[cur.o0 + i], loss, c);
              }
              coef[(size_t)j * L.CS + i] = c;  // zero past O: those products add nothing
            }
          }
        }
      }
      __syncwarp();
    }
    // the next minibatch's rows into the other buffer, its slots behind them
    nxt_ok = nxt_ok && ids_ok(nxt, idn);
    // the next minibatch's rows go after the current ones, or at the ring's start, when
    // they fit beside them; otherwise once the current rows are done with
    const int rc = cur_ok ? cur.I + cur.O : 0, rn = nxt.I + nxt.O;
    int sn = sc + rc + rn <= ring ? sc + rc : rn <= sc ? 0 : -1;
    if (nxt_ok && sn >= 0) {
      issue_copies(nxt, idn, wbase + (size_t)sn * L.RS);
      load_slots(nxt, idn, sln);
    }
    if (cur_ok) {
      // gradient rows, column-parallel: dL/dWih[x_j] = sum_i c_ij Woh[o_i] (order i) and
      // dL/dWoh[o_i] = sum_j c_ij Wih[x_j] (order j)
      for (int q = lane; q < nq; q += 32) {
        if constexpr (DT == 2) {
          T ov[OMX][4], ao[OMX][4];
#pragma unroll
          for (int i = 0; i < OMX; i++)
#pragma unroll
            for (int t = 0; t < 4; t++) ov[i][t] = ao[i][t] = 0;
#pragma unroll
          for (int i = 0; i < OMX; i++) lds4(ofp + (size_t)i * d + 4 * q, ov[i]);
#pragma unroll 2
          for (int j = 0; j < I; j++) {
            T xv[4];
            Pipe<DT>::chunk4(buf + (size_t)j * L.RS + 4 * q * EB, xv);
            const T* cj = coef + (size_t)j * L.CS;
            T ai[4] = {0, 0, 0, 0};
#pragma unroll
            for (int i = 0; i < OMX; i++) {
              const T c = cj[i];
#pragma unroll
              for (int t = 0; t < 4; t++) {
                ai[t] = fma_t(c, ov[i][t], ai[t]);
                ao[i][t] = fma_t(c, xv[t], ao[i][t]);
              }
            }
            atomic_add4(g_in + (size_t)slot[j] * d + 4 * q, ai);
          }
#pragma unroll
          for (int i = 0; i < OMX; i++)
            if (i < O) atomic_add4(g_out + (size_t)slot[I + i] * d + 4 * q, ao[i]);
        } else {
          // packed fp32 pairs: the same fused multiply-adds in the same order
          float2 ov[OMX][2], ao[OMX][2];
#pragma unroll
          for (int i = 0; i < OMX; i++) {
            const float4 o4 = *reinterpret_cast<const float4*>(ofp + (size_t)i * d + 4 * q);
            ov[i][0] = make_float2(o4.x, o4.y), ov[i][1] = make_float2(o4.z, o4.w);
            ao[i][0] = ao[i][1] = make_float2(0.f, 0.f);
          }
#pragma unroll 2
          for (int j = 0; j < I; j++) {
            float xv[4];
            Pipe<DT>::chunk4(buf + (size_t)j * L.RS + 4 * q * EB, xv);
            const float2 x01 = make_float2(xv[0], xv[1]), x23 = make_float2(xv[2], xv[3]);
            const float* cj = coef + (size_t)j * L.CS;
            float2 a01 = make_float2(0.f, 0.f), a23 = a01;
#pragma unroll
            for (int i = 0; i < OMX; i++) {
              const float2 c2 = make_float2(cj[i], cj[i]);
              a01 = __ffma2_rn(c2, ov[i][0], a01);
              a23 = __ffma2_rn(c2, ov[i][1], a23);
              ao[i][0] = __ffma2_rn(c2, x01, ao[i][0]);
              ao[i][1] = __ffma2_rn(c2, x23, ao[i][1]);
            }
            const float ai[4] = {a01.x, a01.y, a23.x, a23.y};
            atomic_add4(g_in + (size_t)slot[j] * d + 4 * q, ai);
          }
#pragma unroll
          for (int i = 0; i < OMX; i++)
            if (i < O) {
              const float v[4] = {ao[i][0].x, ao[i][0].y, ao[i][1].x, ao[i][1].y};
              atomic_add4(g_out + (size_t)slot[I + i] * d + 4 * q, v);
            }
        }
      }
    }
    __syncwarp();
    if (nxt_ok && sn < 0) {
      sn = 0;
      issue_copies(nxt, idn, wbase);
      load_slots(nxt, idn, sln);
    }
    b = bn;
    cur = nxt;
    nxt = nn;
    cur_ok = nxt_ok;
#pragma unroll
    for (int m = 0; m < 3; m++) idc[m] = idn[m], slc[m] = sln[m];
    sc = sn < 0 ? 0 : sn;
  }
  cp_async_wait_all();
  for (int sh = 16; sh > 0; sh >>= 1) loss += __shfl_xor_sync(kFull, loss, sh);
  if (lane == 0 && loss != 0) atomicAdd(&loss_parts[gw & 255], (double)loss);
}

__global__ void finish_loss_kernel(const double* parts, double* loss) {
  double v = parts[threadIdx.x];  // 256 threads
  for (int sh = 16; sh > 0; sh >>= 1) v += __shfl_xor_sync(kFull, v, sh);
  __shared__ double w[8];
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < 8; k++) t += w[k];
    *loss = t;
  }
}

void scan_and_emit(int32_t* a, int64_t V, int32_t* tile_sums, int32_t* ids, cudaStream_t s) {
  const int64_t tiles = (V + kScanTile - 1) / kScanTile;
  scan_tiles_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(a, V, tile_sums);
  scan_tile_sums_kernel<<<1, kScanThreads, 0, s>>>(tile_sums, tiles);
  const unsigned g = (unsigned)std::min<int64_t>((V + 255) / 256, 152 * 32);
  add_prefix_emit_kernel<<<g, 256, 0, s>>>(a, V, tile_sums, ids);
  add_prefix_kernel<<<g, 256, 0, s>>>(a, V, tile_sums);
}

}  // namespace

size_t adjoint_scratch_bytes(int64_t V) {
  const int64_t tiles = (V + kScanTile - 1) / kScanTile;
  // marks (2V), tile sums, status words, then 256 fp64 loss partials (8-byte aligned)
  return sizeof(int32_t) * (size_t)(2 * V + 2 * tiles + 8) + 8 + 256 * sizeof(double);
}
double* loss_parts_of(void* scratch, int64_t V) {
  const int64_t tiles = (V + kScanTile - 1) / kScanTile;
  const size_t off = (sizeof(int32_t) * (size_t)(2 * V + 2 * tiles + 8) + 7) & ~(size_t)7;
  return reinterpret_cast<double*>(static_cast<char*>(scratch) + off);
}

// Phase 1: marks, checks, the row -> slot prefix sums, the emitted ids and the zeroed
// gradient rows.  info[0..1] = distinct input / output rows, info[2] = status bits,
// info[3..4] = the largest input / output count of a minibatch (device memory; the host
// reads them before phase 2).  scratch: adjoint_scratch_bytes(V) bytes, arbitrary on entry.
cudaError_t launch_adjoint_prepare(int dtype, int d, int n, int64_t V, const int32_t* in_ptr, const int32_t* in_ids,
                                   const int32_t* in_first, const int32_t* out_ptr, const int32_t* out_ids,
                                   double* loss, int32_t* grad_in_ids, void* grad_in, int32_t* grad_out_ids,
                                   void* grad_out, int32_t* info, void* scratch, cudaStream_t s) {
  const int64_t tiles = (V + kScanTile - 1) / kScanTile;
  int32_t* incl_in = static_cast<int32_t*>(scratch);
  int32_t* incl_out = incl_in + V;
  int32_t* sums_in = incl_out + V;
  int32_t* sums_out = sums_in + tiles;
  int32_t* status = sums_out + tiles;  // status, imax, omax
  cudaError_t e;
  if ((e = cudaMemsetAsync(incl_in, 0, sizeof(int32_t) * 2 * V, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(status, 0, sizeof(int32_t) * 3, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(loss, 0, sizeof(double), s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(loss_parts_of(scratch, V), 0, 256 * sizeof(double), s)) != cudaSuccess) return e;
  if (n > 0)
    mark_rows_kernel<<<(unsigned)std::min<int64_t>(((int64_t)n + 7) / 8, 152 * 16), 256, 0, s>>>(
        n, in_ptr, in_ids, in_first, out_ptr, out_ids, V, incl_in, incl_out, status, status + 1);
  scan_and_emit(incl_in, V, sums_in, grad_in_ids, s);
  scan_and_emit(incl_out, V, sums_out, grad_out_ids, s);
  const unsigned zg = 152 * 16;
  if (dtype == 2) {
    zero_rows_kernel<double><<<zg, 256, 0, s>>>(static_cast<double*>(grad_in), incl_in + V - 1, d);
    zero_rows_kernel<double><<<zg, 256, 0, s>>>(static_cast<double*>(grad_out), incl_out + V - 1, d);
  } else {
    zero_rows_kernel<float><<<zg, 256, 0, s>>>(static_cast<float*>(grad_in), incl_in + V - 1, d);
    zero_rows_kernel<float><<<zg, 256, 0, s>>>(static_cast<float*>(grad_out), incl_out + V - 1, d);
  }
  if ((e = cudaMemcpyAsync(info, incl_in + V - 1, sizeof(int32_t), cudaMemcpyDeviceToDevice, s))) return e;
  if ((e = cudaMemcpyAsync(info + 1, incl_out + V - 1, sizeof(int32_t), cudaMemcpyDeviceToDevice, s))) return e;
  if ((e = cudaMemcpyAsync(info + 2, status, sizeof(int32_t) * 3, cudaMemcpyDeviceToDevice, s))) return e;
  return cudaGetLastError();
}

// warps (minibatches) per block: four, fewer when their rows do not fit a block's shared memory
int adjoint_warps_per_block(int dtype, int d, int imax, int omax) {
  const size_t per_warp = (dtype == 2 ? 8 : 4) * adjoint_warp_elems(d, imax, omax);
  const int fit = (int)((size_t)232448 / per_warp);
  return std::max(1, std::min(kWarpsPerBlock, fit));
}

// Phase 2: the loss and the row gradients, for minibatches of at most imax inputs and
// omax outputs (the values phase 1 found).
cudaError_t launch_adjoint(int dtype, int d, int n, int64_t V, int imax, int omax, const int32_t* in_ptr,
                           const int32_t* in_ids, const int32_t* in_first, const int32_t* out_ptr,
                           const int32_t* out_ids, const int32_t* out_meta, const void* wih, const void* woh,
                           double* loss, void* grad_in, void* grad_out, void* scratch, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  double* parts = loss_parts_of(scratch, V);
  const int32_t* incl_in = static_cast<const int32_t*>(scratch);
  const int32_t* incl_out = incl_in + V;
  imax = std::max(imax, 1);
  omax = std::max(omax, 1);
  const int wpb = adjoint_warps_per_block(dtype, d, imax, omax);
  const size_t smem = (size_t)(dtype == 2 ? 8 : 4) * wpb * adjoint_warp_elems(d, imax, omax);
  const unsigned blocks = (unsigned)((n + wpb - 1) / wpb);
  cudaError_t e;
#define SGNS_ADJ_LAUNCH1(DT, VW, OMX, TT)                                                                       \
  do {                                                                                                          \
    if ((e = cudaFuncSetAttribute(adjoint_kernel<DT, VW, OMX>, cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                  (int)smem)))                                                                  \
      return e;                                                                                                 \
    adjoint_kernel<DT, VW, OMX><<<blocks, 32 * wpb, smem, s>>>(                                                 \
        d, n, imax, omax, in_ptr, in_ids, in_first, out_ptr, out_ids, out_meta, wih, woh, V, incl_in, incl_out, \
        static_cast<TT*>(grad_in), static_cast<TT*>(grad_out), parts);                                          \
  } while (0)
#define SGNS_ADJ_LAUNCH(DT, VW, TT)                   \
  do {                                                \
    if (omax <= 7) SGNS_ADJ_LAUNCH1(DT, VW, 7, TT);   \
    else SGNS_ADJ_LAUNCH1(DT, VW, kOMax, TT);         \
  } while (0)
  const bool v4 = d % 4 == 0;
  // the pipelined kernel when rows are whole 16-byte chunks at 16-byte aligned addresses
  const int eb = dtype == 2 ? 8 : dtype == 1 ? 2 : 4;
  // a ring of one minibatch's rows (see adjoint_pipe_kernel)
  const int ring = imax + omax;
  const PipeLayout PL = pipe_layout(dtype, d, imax, omax, omax <= 7 ? 7 : kOMax, ring);
  if (v4 && (d * eb) % 16 == 0 && ((uintptr_t)wih & 15) == 0 && ((uintptr_t)woh & 15) == 0 &&
      PL.bytes <= 232448) {
    // warps per block: the most resident warps per SM (228 KB of shared memory, 1 KB
    // reserved per block), the larger block on a tie
    int pw = 1, best = 0;
    for (int w = 1; w <= 8; w++) {
      const int per_block = w * PL.bytes + 1024;
      if (w * PL.bytes > 232448) break;
      const int warps = (233472 / per_block) * w;
      if (warps >= best) best = warps, pw = w;
    }
    const size_t psmem = (size_t)pw * PL.bytes;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) || (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))) return e;
#define SGNS_ADJ_PIPE1(DT, OMX, TT)                                                                             \
  do {                                                                                                          \
    if ((e = cudaFuncSetAttribute(adjoint_pipe_kernel<DT, OMX>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                  (int)psmem)))                                                                 \
      return e;                                                                                                 \
    int per_sm = 0;                                                                                             \
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint_pipe_kernel<DT, OMX>, 32 * pw,      \
                                                           psmem)))                                             \
      return e;                                                                                                 \
    const unsigned pb = (unsigned)std::max<int64_t>(                                                            \
        1, std::min<int64_t>((n + pw - 1) / pw, (int64_t)sms * std::max(per_sm, 1)));                           \
    adjoint_pipe_kernel<DT, OMX><<<pb, 32 * pw, psmem, s>>>(d, n, imax, omax, ring, in_ptr, in_ids, in_first, out_ptr, \
                                                            out_ids, out_meta, wih, woh, V, incl_in, incl_out,   \
                                                            static_cast<TT*>(grad_in),                          \
                                                            static_cast<TT*>(grad_out), parts);                 \
  } while (0)
#define SGNS_ADJ_PIPE(DT, TT)                  \
  do {                                         \
    if (omax <= 7) SGNS_ADJ_PIPE1(DT, 7, TT);  \
    else SGNS_ADJ_PIPE1(DT, kOMax, TT);        \
  } while (0)
    if (dtype == 2) SGNS_ADJ_PIPE(2, double);
    else if (dtype == 1) SGNS_ADJ_PIPE(1, float);
    else SGNS_ADJ_PIPE(0, float);
#undef SGNS_ADJ_PIPE
#undef SGNS_ADJ_PIPE1
    finish_loss_kernel<<<1, 256, 0, s>>>(parts, loss);
    return cudaGetLastError();
  }
  if (dtype == 2) {
    if (v4) SGNS_ADJ_LAUNCH(2, 4, double);
    else SGNS_ADJ_LAUNCH(2, 1, double);
  } else if (dtype == 1) {
    if (v4) SGNS_ADJ_LAUNCH(1, 4, float);
    else SGNS_ADJ_LAUNCH(1, 1, float);
  } else {
    if (v4) SGNS_ADJ_LAUNCH(0, 4, float);
    else SGNS_ADJ_LAUNCH(0, 1, float);
  }
#undef SGNS_ADJ_LAUNCH
#undef SGNS_ADJ_LAUNCH1
  finish_loss_kernel<<<1, 256, 0, s>>>(parts, loss);
  return cudaGetLastError();
}

}  // namespace sgns
