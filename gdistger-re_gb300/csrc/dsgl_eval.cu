// dsgl_eval.cu -- link-prediction scores of held-out pairs: score = <row_u, row_v> of one
// embedding table (fp32 or bf16), the dot-product scoring applied to the holdout that
// src/tools/gtrain.cpp:226-385 writes (test edges and sampled non-edges).
//
// One warp per pair.  Lane l owns columns 4l..4l+3 of each 128-column chunk t (chunk
// order t = 0, 1, ...); it sums u[c] * v[c] over its columns in that order with one fused
// multiply-add per column, then the 32 partial sums are added by an xor butterfly
// (offsets 16, 8, 4, 2, 1).  The order is fixed, so the CPU restatement reproduces every
// score bit for bit.  Rows are read once: a pair costs 2 d s bytes (s = 4 or 2).
#include <cuda_runtime.h>

#include "dsgl_device.cuh"

namespace sgns {

namespace {

template <int S>
__global__ void __launch_bounds__(256) link_scores_kernel(const void* table, int d, int64_t V, const int32_t* pairs,
                                                        int64_t n, float* scores, int32_t* bad) {
  const int lane = lane_id();
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int d4 = d >> 2;
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const int32_t u = pairs[2 * i], v = pairs[2 * i + 1];
    if (u < 0 || v < 0 || (int64_t)u >= V || (int64_t)v >= V) {  // skipped, reported to the host
      if (lane == 0) {
        scores[i] = 0.f;
        atomicExch(bad, 1);
      }
      continue;
    }
    float acc = 0.f;
    for (int q = lane; q < d4; q += 32) {
      const float4 a = RowIO<S>::load4(table, u, d, q), b = RowIO<S>::load4(table, v, d, q);
      acc = __fmaf_rn(a.x, b.x, acc);
      acc = __fmaf_rn(a.y, b.y, acc);
      acc = __fmaf_rn(a.z, b.z, acc);
      acc = __fmaf_rn(a.w, b.w, acc);
    }
    for (int o = 16; o > 0; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, o));
    if (lane == 0) scores[i] = acc;
  }
}

}  // namespace

cudaError_t launch_link_scores(int storage, const void* table, int d, int64_t V, const int32_t* pairs, int64_t n,
                               float* scores, int32_t* bad, int num_sms, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int64_t blocks = (n + 7) / 8;  // 8 warps per block, one pair per warp
  if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
  if (storage == STORE_BF16)
    link_scores_kernel<STORE_BF16><<<(unsigned)blocks, 256, 0, s>>>(table, d, V, pairs, n, scores, bad);
  else
    link_scores_kernel<STORE_F32><<<(unsigned)blocks, 256, 0, s>>>(table, d, V, pairs, n, scores, bad);
  return cudaGetLastError();
}

}  // namespace sgns
