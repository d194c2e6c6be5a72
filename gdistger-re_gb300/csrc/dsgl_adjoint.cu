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
// and each minibatch warp adds its row gradients into the compact slots.
#include <cuda_runtime.h>

#include <algorithm>

#include "dsgl_device.cuh"

namespace sgns {

namespace {

template <int DT> struct Elem;
template <> struct Elem<0> {  // fp32 tables
  typedef float T;
  __device__ static float get(const void* p, int64_t i) { return static_cast<const float*>(p)[i]; }
};
template <> struct Elem<1> {  // bf16 tables, fp32 arithmetic
  typedef float T;
  __device__ static float get(const void* p, int64_t i) {
    return bf16_bits_to_f32(static_cast<const uint16_t*>(p)[i]);
  }
};
template <> struct Elem<2> {  // fp64 tables and arithmetic
  typedef double T;
  __device__ static double get(const void* p, int64_t i) { return static_cast<const double*>(p)[i]; }
};

__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float sigmoid_t(float x) { return 1.0f / (1.0f + expf(-x)); }
__device__ __forceinline__ double sigmoid_t(double x) { return 1.0 / (1.0 + exp(-x)); }
__device__ __forceinline__ float softplus_t(float z) { return fmaxf(z, 0.f) + log1pf(expf(-fabsf(z))); }
__device__ __forceinline__ double softplus_t(double z) { return fmax(z, 0.0) + log1p(exp(-fabs(z))); }

__global__ void mark_rows_kernel(const int32_t* ids, int64_t n, int32_t* mark, int64_t V, int32_t* bad) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = ids[t];
    if (r < 0 || r >= V) atomicExch(bad, 1);
    else mark[r] = 1;
  }
}

// inclusive scan, three passes: per-block scan of 4096 elements, scan of block totals,
// add the block prefix
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(int32_t* a, int64_t n, int32_t* tile_sums) {
  __shared__ int32_t warp_sums[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t run = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = base + k < n ? a[base + k] : 0;
    run += v[k];
    v[k] = run;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t x = run;
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int32_t s = warp_sums[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
      if (lane >= o) s += y;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  const int32_t prefix = (x - run) + (warp > 0 ? warp_sums[warp - 1] : 0);
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    if (base + k < n) a[base + k] = v[k] + prefix;
  if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = prefix + run;
}

__global__ void scan_tile_sums_kernel(int32_t* tile_sums, int64_t ntiles) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int32_t run = 0;
    for (int64_t i = 0; i < ntiles; i++) {
      run += tile_sums[i];
      tile_sums[i] = run;
    }
  }
}

__global__ void add_tile_prefix_kernel(int32_t* a, int64_t n, const int32_t* tile_sums) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t tile = i / kScanTile;
  if (tile > 0) a[i] += tile_sums[tile - 1];
}

// marked rows (incl[r] - incl[r-1] == 1) -> ids[incl[r] - 1] = r
__global__ void emit_ids_kernel(const int32_t* incl, int64_t V, int32_t* ids) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < V; r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t prev = r > 0 ? incl[r - 1] : 0;
    if (incl[r] != prev) ids[incl[r] - 1] = (int32_t)r;
  }
}

template <int DT>
__global__ void __launch_bounds__(32) adjoint_kernel(int d, int n, const int32_t* in_ptr, const int32_t* in_ids,
                                                     const int32_t* in_first, const int32_t* out_ptr,
                                                     const int32_t* out_ids, const int32_t* out_meta,
                                                     const void* wih, const void* woh, int64_t V,
                                                     const int32_t* incl_in, const int32_t* incl_out,
                                                     typename Elem<DT>::T* g_in, typename Elem<DT>::T* g_out,
                                                     double* loss_out) {
  typedef typename Elem<DT>::T T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int b = blockIdx.x, lane = lane_id();
  if (b >= n) return;
  const int i0 = in_ptr[b], I = in_ptr[b + 1] - i0, o0 = out_ptr[b], O = out_ptr[b + 1] - o0;
  const int first = in_first[b];
  // ids outside [0, V) were flagged by mark_rows_kernel; this minibatch is skipped
  bool ok = true;
  for (int j = lane; j < I; j += 32) ok &= in_ids[i0 + j] >= 0 && in_ids[i0 + j] < V;
  for (int i = lane; i < O; i += 32) ok &= out_ids[o0 + i] >= 0 && out_ids[o0 + i] < V;
  if (!__all_sync(kFull, ok)) return;
  T* x = sm;                           // I x d
  T* o = x + (size_t)I * d;            // O x d
  T* coef = o + (size_t)O * d;         // O x I
  for (int j = 0; j < I; j++) {
    const int64_t r = in_ids[i0 + j];
    for (int c = lane; c < d; c += 32) x[(size_t)j * d + c] = Elem<DT>::get(wih, r * d + c);
  }
  for (int i = 0; i < O; i++) {
    const int64_t r = out_ids[o0 + i];
    for (int c = lane; c < d; c += 32) o[(size_t)i * d + c] = Elem<DT>::get(woh, r * d + c);
  }
  __syncwarp();
  T loss = 0;
  for (int p = lane; p < O * I; p += 32) {
    const int i = p / I, j = p % I;
    T f = 0;
    for (int k = 0; k < d; k++) f = fma_t(o[(size_t)i * d + k], x[(size_t)j * d + k], f);
    const int label = j < first ? (i == 0) : (i == O - 1);
    const T meta = (T)out_meta[o0 + i];
    loss += meta * softplus_t(label ? -f : f);
    coef[p] = meta * (sigmoid_t(f) - (T)label);
  }
  __syncwarp();
  for (int o2 = 16; o2 > 0; o2 >>= 1) loss += __shfl_xor_sync(kFull, loss, o2);
  if (lane == 0) atomicAdd(loss_out, (double)loss);
  // dL/dWih[x_j] = sum_i coef_ij Woh[o_i]
  for (int j = 0; j < I; j++) {
    T* dst = g_in + (size_t)(incl_in[in_ids[i0 + j]] - 1) * d;
    for (int c = lane; c < d; c += 32) {
      T acc = 0;
      for (int i = 0; i < O; i++) acc = fma_t(coef[i * I + j], o[(size_t)i * d + c], acc);
      atomicAdd(dst + c, acc);
    }
  }
  // dL/dWoh[o_i] = sum_j coef_ij Wih[x_j]
  for (int i = 0; i < O; i++) {
    T* dst = g_out + (size_t)(incl_out[out_ids[o0 + i]] - 1) * d;
    for (int c = lane; c < d; c += 32) {
      T acc = 0;
      for (int j = 0; j < I; j++) acc = fma_t(coef[i * I + j], x[(size_t)j * d + c], acc);
      atomicAdd(dst + c, acc);
    }
  }
}

cudaError_t scan_inclusive(int32_t* a, int64_t n, int32_t* tile_sums, cudaStream_t s) {
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  scan_tiles_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(a, n, tile_sums);
  scan_tile_sums_kernel<<<1, 1, 0, s>>>(tile_sums, tiles);
  add_tile_prefix_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, n, tile_sums);
  return cudaGetLastError();
}

}  // namespace

size_t adjoint_scratch_bytes(int64_t V) {
  const int64_t tiles = (V + kScanTile - 1) / kScanTile;
  return sizeof(int32_t) * (size_t)(2 * V + 2 * tiles + 4);
}

// scratch: adjoint_scratch_bytes(V) bytes, contents arbitrary on entry.
// totals: host values of in_ptr[n] and out_ptr[n].
cudaError_t launch_adjoint(int dtype, int d, int n, int64_t V, int64_t total_in, int64_t total_out,
                           const int32_t* in_ptr, const int32_t* in_ids, const int32_t* in_first,
                           const int32_t* out_ptr, const int32_t* out_ids, const int32_t* out_meta,
                           const void* wih, const void* woh, double* loss, int32_t* grad_in_ids, void* grad_in,
                           int32_t* grad_out_ids, void* grad_out, int32_t* n_unique, void* scratch,
                           int imax, int omax, cudaStream_t s) {
  const int64_t tiles = (V + kScanTile - 1) / kScanTile;
  int32_t* incl_in = static_cast<int32_t*>(scratch);
  int32_t* incl_out = incl_in + V;
  int32_t* sums_in = incl_out + V;
  int32_t* sums_out = sums_in + tiles;
  int32_t* bad = sums_out + tiles;
  cudaError_t e;
  if ((e = cudaMemsetAsync(incl_in, 0, sizeof(int32_t) * 2 * V, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(bad, 0, sizeof(int32_t), s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(loss, 0, sizeof(double), s)) != cudaSuccess) return e;
  const int esz = dtype == 2 ? 8 : 4;
  if ((e = cudaMemsetAsync(grad_in, 0, (size_t)esz * total_in * d, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(grad_out, 0, (size_t)esz * total_out * d, s)) != cudaSuccess) return e;
  auto grid = [](int64_t m) { return (unsigned)std::min<int64_t>((m + 255) / 256, 152 * 16); };
  if (total_in) mark_rows_kernel<<<grid(total_in), 256, 0, s>>>(in_ids, total_in, incl_in, V, bad);
  if (total_out) mark_rows_kernel<<<grid(total_out), 256, 0, s>>>(out_ids, total_out, incl_out, V, bad);
  if ((e = scan_inclusive(incl_in, V, sums_in, s)) != cudaSuccess) return e;
  if ((e = scan_inclusive(incl_out, V, sums_out, s)) != cudaSuccess) return e;
  emit_ids_kernel<<<grid(V), 256, 0, s>>>(incl_in, V, grad_in_ids);
  emit_ids_kernel<<<grid(V), 256, 0, s>>>(incl_out, V, grad_out_ids);
  if (n > 0) {
    const size_t smem = (size_t)esz * ((size_t)(imax + omax) * d + (size_t)imax * omax);
    if (dtype == 2) {
      if ((e = cudaFuncSetAttribute(adjoint_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
        return e;
      adjoint_kernel<2><<<n, 32, smem, s>>>(d, n, in_ptr, in_ids, in_first, out_ptr, out_ids, out_meta, wih, woh,
                                            V, incl_in, incl_out, static_cast<double*>(grad_in),
                                            static_cast<double*>(grad_out), loss);
    } else if (dtype == 1) {
      if ((e = cudaFuncSetAttribute(adjoint_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
        return e;
      adjoint_kernel<1><<<n, 32, smem, s>>>(d, n, in_ptr, in_ids, in_first, out_ptr, out_ids, out_meta, wih, woh,
                                            V, incl_in, incl_out, static_cast<float*>(grad_in),
                                            static_cast<float*>(grad_out), loss);
    } else {
      if ((e = cudaFuncSetAttribute(adjoint_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
        return e;
      adjoint_kernel<0><<<n, 32, smem, s>>>(d, n, in_ptr, in_ids, in_first, out_ptr, out_ids, out_meta, wih, woh,
                                            V, incl_in, incl_out, static_cast<float*>(grad_in),
                                            static_cast<float*>(grad_out), loss);
    }
  }
  // n_unique[0..1] = number of marked rows; n_unique[2] = bad id flag
  if ((e = cudaMemcpyAsync(n_unique, incl_in + V - 1, sizeof(int32_t), cudaMemcpyDeviceToDevice, s))) return e;
  if ((e = cudaMemcpyAsync(n_unique + 1, incl_out + V - 1, sizeof(int32_t), cudaMemcpyDeviceToDevice, s))) return e;
  if ((e = cudaMemcpyAsync(n_unique + 2, bad, sizeof(int32_t), cudaMemcpyDeviceToDevice, s))) return e;
  return cudaGetLastError();
}

}  // namespace sgns
