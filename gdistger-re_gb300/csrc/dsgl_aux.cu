// dsgl_aux.cu -- set-up kernels (Wih initialisation, corpus mapping), the explicit-row
// minibatch update, and the SGNS loss with its hand-written adjoint.
#include <cuda_runtime.h>

#include <algorithm>

#include "dsgl_device.cuh"

namespace sgns {

namespace {

// InitNet (dsgl.hpp:451-456): element i of Wih takes LCG state r_{i+1} (r_0 = 1),
// value ((r & 0xFFFF) / 65536 - 0.5) / d.  Each thread owns 64 consecutive elements and
// starts from a jump-ahead; bf16 tables store the fp32 value rounded to nearest even.
__global__ void init_wih_kernel(void* wih, int storage, int64_t n, int32_t d, const LcgJumps* J) {
  const int64_t i0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 64;
  if (i0 >= n) return;
  uint64_t r = jump_any(1ULL, (uint64_t)i0, J);
  const float fd = (float)d;
  for (int k = 0; k < 64 && i0 + k < n; k++) {
    r = lcg_next(r);
    const float v = __fdiv_rn(__fsub_rn(__fdiv_rn((float)(uint32_t)(r & 0xFFFF), 65536.0f), 0.5f), fd);
    if (storage == STORE_BF16)
      static_cast<__nv_bfloat16*>(wih)[i0 + k] = __float2bfloat16_rn(v);
    else
      static_cast<float*>(wih)[i0 + k] = v;
  }
}

// vertex ids -> sorted rows; -1 separators kept; anything else outside [0, V) flagged
__device__ __forceinline__ int32_t map_id(int32_t t, const int32_t* row_of, int64_t V, bool* bad) {
  if (t == -1) return -1;
  if (t < 0 || (int64_t)t >= V) {
    *bad = true;
    return -1;
  }
  return __ldg(&row_of[t]);
}
// ids may be device memory or pinned host memory mapped into the device's address space
// (then every id crosses the host link once, read in 16-byte pieces when aligned).
__global__ void map_corpus_kernel(const int32_t* ids, const int32_t* row_of, int32_t* rows, int64_t n,
                                  int64_t V, int32_t* bad, bool vec4) {
  bool b = false;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (vec4) {  // ids and rows 16-byte aligned
    const int64_t n4 = n >> 2;
    for (int64_t i = t0; i < n4; i += stride) {
      const int4 v = reinterpret_cast<const int4*>(ids)[i];
      reinterpret_cast<int4*>(rows)[i] = make_int4(map_id(v.x, row_of, V, &b), map_id(v.y, row_of, V, &b),
                                                   map_id(v.z, row_of, V, &b), map_id(v.w, row_of, V, &b));
    }
    for (int64_t i = (n4 << 2) + t0; i < n; i += stride) rows[i] = map_id(ids[i], row_of, V, &b);
  } else {
    for (int64_t i = t0; i < n; i += stride) rows[i] = map_id(ids[i], row_of, V, &b);
  }
  if (b) atomicExch(bad, 1);
}

// ---- explicit-row minibatch update (the step arithmetic of both trainers) ----------
// kRound: instead of the updates, write each updated row (row + update) as bf16 bits with
// the trainers' stochastic rounding (RowIO<STORE_BF16>::store4), event keys from sr_seed
// and the minibatch index; d_in / d_out then point to uint16 rows.
template <int DCH, bool kRound = false>
__global__ void __launch_bounds__(32) minibatch_kernel(int d, int imax, int omax, const int32_t* in_count,
                                                       const int32_t* in_first, const int32_t* out_count,
                                                       const int32_t* out_meta_all, const float* alpha,
                                                       const int64_t* in_off, const int64_t* out_off,
                                                       const float* in_rows, const float* out_rows,
                                                       float* d_in, float* d_out, const float* exp_table,
                                                       int32_t* status, uint64_t sr_seed = 0) {
  extern __shared__ __align__(16) float smem[];
  const int b = blockIdx.x, lane = lane_id();
  const int I = in_count[b], first = in_first[b], O = out_count[b];
  if (I < 1 || I > imax || O < 2 || O > omax || first < 0 || first > I) {
    if (lane == 0) atomicExch(status, 1);
    return;
  }
  const int DP = d + 4;
  float* exp_s = smem;
  float* xin = smem + 1004;
  float* outI = xin + (size_t)imax * DP;
  float2* corrP = reinterpret_cast<float2*>(outI + (size_t)kOMax * d);
  int* meta = reinterpret_cast<int*>(corrP + (size_t)imax * (kOMax + 2));
  for (int i = lane; i < kExpTableSize + 1; i += 32) exp_s[i] = exp_table[i];
  const int d4 = d >> 2;
  const float* gin = in_rows + in_off[b] * d;
  const float* gout = out_rows + out_off[b] * d;
  for (int j = 0; j < I; j++)
    for (int q = lane; q < d4; q += 32)
      reinterpret_cast<float4*>(xin + (size_t)j * DP)[q] = reinterpret_cast<const float4*>(gin + (size_t)j * d)[q];
  {
    float4 v[kOMax][DCH];
#pragma unroll
    for (int i = 0; i < kOMax; i++)
#pragma unroll
      for (int t = 0; t < DCH; t++) {
        const int q = lane + 32 * t;
        v[i][t] = (i < O && q < d4) ? reinterpret_cast<const float4*>(gout + (size_t)i * d)[q]
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    store_out_interleaved<kOMax, DCH>(v, O, d, outI);
  }
  for (int i = lane; i < O; i += 32) meta[i] = out_meta_all[out_off[b] + i];
  __syncwarp();
  auto in_ptr = [&](int j) -> const float* { return xin + (size_t)j * DP; };
  float loss = 0.f;
  forward_gradient<kOMax>(I, first, O, d, in_ptr, outI, meta, exp_s, alpha[b], corrP, false, loss);
  float4 md[kOMax][DCH];
  if (!kRound) {
    float* gdin = d_in + in_off[b] * d;
    backward<kOMax, DCH>(I, O, d, in_ptr, [&](int pp, int q, float4& r0, float4& r1) { out_chunk_pair(outI, d, pp, q, r0, r1); }, corrP, md,
                         [&](int j, int q, float4 a) { reinterpret_cast<float4*>(gdin + (size_t)j * d)[q] = a; });
    float* gdout = d_out + out_off[b] * d;
#pragma unroll
    for (int i = 0; i < kOMax; i++)
#pragma unroll
      for (int t = 0; t < DCH; t++) {
        const int q = lane + 32 * t;
        if (i < O && q < d4) reinterpret_cast<float4*>(gdout + (size_t)i * d)[q] = md[i][t];
      }
  } else {
    // rows j of the inputs: event key EV_WALK0 of minibatch b; row index = j (outputs: the
    // key EV_NEG, row index = i) -- the same rounding rule and hash as the trainers' stores
    const uint64_t ev_in = sr_event_key(sr_seed, EV_WALK0, 0u, (uint64_t)b);
    const uint64_t ev_out = sr_event_key(sr_seed, EV_NEG, 0u, (uint64_t)b);
    uint16_t* gin16 = reinterpret_cast<uint16_t*>(d_in) + in_off[b] * d;
    backward<kOMax, DCH>(I, O, d, in_ptr, [&](int pp, int q, float4& r0, float4& r1) { out_chunk_pair(outI, d, pp, q, r0, r1); }, corrP, md,
                         [&](int j, int q, float4 a) {
                           const float4 x = reinterpret_cast<const float4*>(gin + (size_t)j * d)[q];
                           RowIO<STORE_BF16>::store4(gin16, j, d, q, add4(x, a), ev_in);
                         });
    uint16_t* gout16 = reinterpret_cast<uint16_t*>(d_out) + out_off[b] * d;
#pragma unroll
    for (int i = 0; i < kOMax; i++)
#pragma unroll
      for (int t = 0; t < DCH; t++) {
        const int q = lane + 32 * t;
        if (i < O && q < d4) {
          const float4 o = reinterpret_cast<const float4*>(gout + (size_t)i * d)[q];
          RowIO<STORE_BF16>::store4(gout16, i, d, q, add4(o, md[i][t]), ev_out);
        }
      }
  }
}

// each walk start scans forward to its separator (at most kMaxSentence tokens); one
// atomic per warp
__global__ void max_walk_kernel(const int32_t* rows, int64_t n, int32_t* out) {
  int best = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    if (rows[i] == -1 || (i > 0 && rows[i - 1] != -1)) continue;
    int len = 0;
    while (i + len < n && rows[i + len] != -1 && len < kMaxSentence) len++;
    best = len > best ? len : best;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const int t = __shfl_xor_sync(kFull, best, o);
    best = t > best ? t : best;
  }
  if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(out, best);
}

// A negative count (rejected by its own minibatch) adds nothing, so no later minibatch's
// offset points before the start of the caller's row arrays.
__global__ void prefix_offsets_kernel(const int32_t* cnt_a, const int32_t* cnt_b, int n, int64_t* off_a,
                                      int64_t* off_b) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int64_t a = 0, bb = 0;
    for (int i = 0; i < n; i++) {
      off_a[i] = a;
      off_b[i] = bb;
      a += cnt_a[i] > 0 ? cnt_a[i] : 0;
      bb += cnt_b[i] > 0 ? cnt_b[i] : 0;
    }
  }
}

}  // namespace

// bf16 bits -> fp32 (exact), 4 elements per thread; n % 4 == 0 (d is a multiple of 4)
__global__ void widen_bf16_kernel(const uint2* __restrict__ src, float4* __restrict__ dst, int64_t n4) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
    const uint2 u = src[i];
    dst[i] = make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xFFFF0000u), __uint_as_float(u.y << 16),
                         __uint_as_float(u.y & 0xFFFF0000u));
  }
}

// ---- hotness-block sync: rows out of and back into a table (one warp per row) ----------
__global__ void gather_rows_kernel(const void* tab, int storage, int d, const int32_t* rows, int64_t n, float* buf) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const int64_t r = rows[i];
    for (int c = lane; c < d; c += 32)
      buf[i * d + c] = storage == STORE_BF16 ? bf16_bits_to_f32(static_cast<const uint16_t*>(tab)[r * d + c])
                                             : static_cast<const float*>(tab)[r * d + c];
  }
}
// row = buf / divisor (fp32 division, as the reference averages, dsgl.hpp:741-745); bf16
// tables round to nearest even, so every rank stores the same bits
__global__ void scatter_rows_kernel(void* tab, int storage, int d, const int32_t* rows, int64_t n, const float* buf,
                                    float divisor) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const int64_t r = rows[i];
    for (int c = lane; c < d; c += 32) {
      const float v = __fdiv_rn(buf[i * d + c], divisor);
      if (storage == STORE_BF16) {
        const uint32_t u = __float_as_uint(v);
        uint16_t b;
        if ((u & 0x7F800000u) == 0x7F800000u) b = (uint16_t)((u >> 16) | ((u & 0xFFFFu) ? 0x40u : 0u));
        else b = (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
        static_cast<uint16_t*>(tab)[r * d + c] = b;
      } else {
        static_cast<float*>(tab)[r * d + c] = v;
      }
    }
  }
}

cudaError_t launch_gather_rows(const void* tab, int storage, int d, const int32_t* rows, int64_t n, float* buf,
                               cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((n + 7) / 8, 152 * 16);
  gather_rows_kernel<<<(unsigned)blocks, 256, 0, s>>>(tab, storage, d, rows, n, buf);
  return cudaGetLastError();
}
cudaError_t launch_scatter_rows(void* tab, int storage, int d, const int32_t* rows, int64_t n, const float* buf,
                                float divisor, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((n + 7) / 8, 152 * 16);
  scatter_rows_kernel<<<(unsigned)blocks, 256, 0, s>>>(tab, storage, d, rows, n, buf, divisor);
  return cudaGetLastError();
}

cudaError_t launch_widen_bf16(const void* src, float* dst, int64_t n, cudaStream_t s) {
  const int64_t n4 = n / 4;
  if (n4 == 0) return cudaSuccess;
  const int64_t blocks = (n4 + 255) / 256;
  widen_bf16_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, s>>>(static_cast<const uint2*>(src),
                                                                             reinterpret_cast<float4*>(dst), n4);
  return cudaGetLastError();
}

cudaError_t launch_init_wih(void* wih, int storage, int64_t V, int32_t d, const LcgJumps* jumps,
                            cudaStream_t s) {
  const int64_t n = V * d;
  const int64_t threads = (n + 63) / 64;
  init_wih_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(wih, storage, n, d, jumps);
  return cudaGetLastError();
}

cudaError_t launch_map_corpus(const int32_t* ids, const int32_t* row_of, int32_t* rows, int64_t n,
                              int64_t V, int32_t* bad, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  const bool vec4 = ((reinterpret_cast<uintptr_t>(ids) | reinterpret_cast<uintptr_t>(rows)) & 15) == 0;
  map_corpus_kernel<<<(unsigned)blocks, 256, 0, s>>>(ids, row_of, rows, n, V, bad, vec4);
  return cudaGetLastError();
}

cudaError_t launch_max_walk(const int32_t* rows, int64_t n, int32_t* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  max_walk_kernel<<<(unsigned)blocks, 256, 0, s>>>(rows, n, out);
  return cudaGetLastError();
}

cudaError_t launch_minibatch_bf16(int d, int n, int imax, const int32_t* in_count, const int32_t* in_first,
                                  const int32_t* out_count, const int32_t* out_meta, const float* alpha,
                                  const float* in_rows, const float* out_rows, uint16_t* new_in, uint16_t* new_out,
                                  uint64_t sr_seed, const float* exp_table, int64_t* offsets, int32_t* status,
                                  cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int64_t* in_off = offsets;
  int64_t* out_off = offsets + n;
  prefix_offsets_kernel<<<1, 1, 0, s>>>(in_count, out_count, n, in_off, out_off);
  const int DP = d + 4;
  const size_t smem = sizeof(float) * (1004 + (size_t)imax * DP + (size_t)kOMax * d +
                                       (size_t)imax * (kOMax + 2) * 2 + kOMax + 4);
  float* a = reinterpret_cast<float*>(new_in);
  float* b = reinterpret_cast<float*>(new_out);
  cudaError_t e;
  if (d > 128) {
    e = cudaFuncSetAttribute(minibatch_kernel<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    minibatch_kernel<2, true><<<n, 32, smem, s>>>(d, imax, kOMax, in_count, in_first, out_count, out_meta, alpha,
                                                  in_off, out_off, in_rows, out_rows, a, b, exp_table, status,
                                                  sr_seed);
  } else {
    e = cudaFuncSetAttribute(minibatch_kernel<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    minibatch_kernel<1, true><<<n, 32, smem, s>>>(d, imax, kOMax, in_count, in_first, out_count, out_meta, alpha,
                                                  in_off, out_off, in_rows, out_rows, a, b, exp_table, status,
                                                  sr_seed);
  }
  return cudaGetLastError();
}

cudaError_t launch_minibatch(int d, int n, int imax, int omax, const int32_t* in_count,
                             const int32_t* in_first, const int32_t* out_count, const int32_t* out_meta,
                             const float* alpha, const float* in_rows, const float* out_rows, float* d_in,
                             float* d_out, const float* exp_table, int64_t* offsets, int32_t* status,
                             cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int64_t* in_off = offsets;
  int64_t* out_off = offsets + n;
  prefix_offsets_kernel<<<1, 1, 0, s>>>(in_count, out_count, n, in_off, out_off);
  const int DP = d + 4;
  (void)omax;
  const size_t smem = sizeof(float) * (1004 + (size_t)imax * DP + (size_t)kOMax * d +
                                       (size_t)imax * (kOMax + 2) * 2 + kOMax + 4);
  cudaError_t e;
  if (d > 128) {
    e = cudaFuncSetAttribute(minibatch_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    minibatch_kernel<2><<<n, 32, smem, s>>>(d, imax, omax, in_count, in_first, out_count, out_meta, alpha,
                                            in_off, out_off, in_rows, out_rows, d_in, d_out, exp_table, status);
  } else {
    e = cudaFuncSetAttribute(minibatch_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    minibatch_kernel<1><<<n, 32, smem, s>>>(d, imax, omax, in_count, in_first, out_count, out_meta, alpha,
                                            in_off, out_off, in_rows, out_rows, d_in, d_out, exp_table, status);
  }
  return cudaGetLastError();
}

}  // namespace sgns
