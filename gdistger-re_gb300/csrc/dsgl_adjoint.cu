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
// Kernels (one warp per minibatch, four per block):
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

// Marks the rows of every minibatch (one thread per minibatch), checks its extents and
// records the largest input and output counts (dims[0], dims[1]).
__global__ void mark_rows_kernel(int n, const int32_t* in_ptr, const int32_t* in_ids, const int32_t* in_first,
                                 const int32_t* out_ptr, const int32_t* out_ids, int64_t V, int32_t* mark_in,
                                 int32_t* mark_out, int32_t* status, int32_t* dims) {
  int imax = 0, omax = 0;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
    const int i0 = in_ptr[b], i1 = in_ptr[b + 1], o0 = out_ptr[b], o1 = out_ptr[b + 1];
    if (i0 < 0 || o0 < 0 || i1 - i0 < 0 || i1 - i0 > kIMax || o1 - o0 < 0 || o1 - o0 > kOMax ||
        in_first[b] < 0 || in_first[b] > i1 - i0) {
      atomicOr(status, kBadSize);
      continue;
    }
    imax = max(imax, i1 - i0);
    omax = max(omax, o1 - o0);
    for (int t = i0; t < i1; t++) {
      const int32_t r = in_ids[t];
      if (r < 0 || r >= V) atomicOr(status, kBadId);
      else mark_in[r] = 1;
    }
    for (int t = o0; t < o1; t++) {
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
    mark_rows_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(
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
