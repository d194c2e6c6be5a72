// dsgl_device.cuh -- device building blocks shared by the DSGL engines: storage row
// access (fp32 / bf16 with stochastic rounding), LCG jump-ahead, warp-parallel walk fill,
// negative draws, and the step arithmetic (forward + gradient, both backward products).
//
// Arithmetic contract: every dot product and both backward products are sequential in
// the reduction index, one fused multiply-add per term (the order of the reference's
// loops, dsgl.hpp:1226-1229, 1282-1285, 1301-1304); every other float expression is an
// explicit _rn intrinsic so no contraction can change it.  With one worker the engines
// therefore reproduce the CPU oracle bit for bit.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "sgns_internal.h"

namespace sgns {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
// index of the n-th (0-based) set bit of x; x has more than n bits set
__device__ __forceinline__ int nth_set_bit(unsigned x, int n) {
  for (int i = 0; i < n; i++) x &= x - 1;
  return __ffs(x) - 1;
}

// ---- storage rows ------------------------------------------------------------------
// A row of d elements; column chunk q holds columns 4q..4q+3 (d % 4 == 0).
template <int S> struct RowIO;

template <> struct RowIO<STORE_F32> {
  static constexpr int kBytes = 4;
  __device__ static __forceinline__ float4 load4(const void* base, int64_t row, int d, int q) {
    return reinterpret_cast<const float4*>(static_cast<const float*>(base) + row * d)[q];
  }
  __device__ static __forceinline__ float4 store4(void* base, int64_t row, int d, int q, float4 v,
                                                  uint64_t) {
    reinterpret_cast<float4*>(static_cast<float*>(base) + row * d)[q] = v;
    return v;
  }
};

template <> struct RowIO<STORE_BF16> {
  static constexpr int kBytes = 2;
  __device__ static __forceinline__ float4 load4(const void* base, int64_t row, int d, int q) {
    uint2 u = reinterpret_cast<const uint2*>(static_cast<const uint16_t*>(base) + row * d)[q];
    return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xFFFF0000u),
                       __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xFFFF0000u));
  }
  // Stores with stochastic rounding; returns the values actually stored (as fp32).
  __device__ static __forceinline__ float4 store4(void* base, int64_t row, int d, int q, float4 v,
                                                  uint64_t ev) {
    uint64_t bits = sr_bits4(ev, (uint32_t)row, (uint32_t)q);
    uint32_t h0 = bf16_sr(v.x, (uint32_t)(bits)&0xFFFF);
    uint32_t h1 = bf16_sr(v.y, (uint32_t)(bits >> 16) & 0xFFFF);
    uint32_t h2 = bf16_sr(v.z, (uint32_t)(bits >> 32) & 0xFFFF);
    uint32_t h3 = bf16_sr(v.w, (uint32_t)(bits >> 48) & 0xFFFF);
    uint2 u = make_uint2(h0 | (h1 << 16), h2 | (h3 << 16));
    reinterpret_cast<uint2*>(static_cast<uint16_t*>(base) + row * d)[q] = u;
    return make_float4(__uint_as_float(h0 << 16), __uint_as_float(h1 << 16),
                       __uint_as_float(h2 << 16), __uint_as_float(h3 << 16));
  }
};

__device__ __forceinline__ float4 add4(float4 a, float4 b) {
  return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z),
                     __fadd_rn(a.w, b.w));
}
__device__ __forceinline__ float4 fma4s(float s, float4 x, float4 acc) {
  return make_float4(__fmaf_rn(s, x.x, acc.x), __fmaf_rn(s, x.y, acc.y), __fmaf_rn(s, x.z, acc.z),
                     __fmaf_rn(s, x.w, acc.w));
}

// ---- LCG jumps ---------------------------------------------------------------------
struct SmallJumps {
  uint64_t mul[33], add[33];
};
__device__ __forceinline__ uint64_t jump_small(uint64_t r, int k, const SmallJumps& j) {
  return j.mul[k] * r + j.add[k];
}
__device__ __forceinline__ uint64_t jump_any(uint64_t r, uint64_t n, const LcgJumps* J) {
  for (int i = 0; n; i++, n >>= 1)
    if (n & 1) r = __ldg(&J->pow2_mul[i]) * r + __ldg(&J->pow2_add[i]);
  return r;
}

// ---- learning rate (dsgl.hpp:886-897) ----------------------------------------------
__device__ __forceinline__ float alpha_update(const TrainParams& p, unsigned long long wca_now) {
  float a = __fmul_rn(p.start_alpha,
                      __fsub_rn(1.0f, __fdiv_rn(__ull2float_rn(wca_now), p.alpha_denom)));
  float floor_a = __fmul_rn(p.start_alpha, 0.0001f);
  return a < floor_a ? floor_a : a;
}

// ---- walk fill with subsampling (dsgl.hpp:909-933), one warp ------------------------
// Reads tokens from cur until a -1, the slice end (whose last token is consumed and
// dropped, as the reference does) or kMaxSentence kept tokens.  Kept rows go to sen[].
// Returns the kept length; cur, word_count and rng advance exactly as the reference's.
// cap: capacity of sen (>= the longest walk of the corpus, checked by the host); a
// longer walk sets the kernel status to SGNS_EINVAL and is truncated.
__device__ __forceinline__ int fill_walk(const TrainParams& p, const SmallJumps& sj, int* sen,
                                         int64_t& cur, int64_t end, uint64_t& word_count,
                                         uint64_t& rng, int cap) {
  const int lane = lane_id();
  int L = 0;
  while (true) {
    const int64_t q = cur + lane;
    const bool in_range = q < end;
    const int tok = in_range ? __ldg(&p.corpus[q]) : -1;
    const unsigned stop = __ballot_sync(kFull, in_range && (tok == -1 || q == end - 1));
    const int first_stop = stop ? __ffs(stop) - 1 : 32;
    const bool valid = lane < first_stop;
    bool keep = valid;
    if (p.sample_on && valid) {
      uint64_t st = jump_small(rng, lane + 1, sj);
      float u = __fdiv_rn((float)(uint32_t)(st & 0xFFFF), 65536.0f);
      keep = !(__ldg(&p.ran[tok]) < u);
    }
    const unsigned keep_mask = __ballot_sync(kFull, keep);
    const int nk = __popc(keep_mask);
    int consumed, draws;
    bool done;
    if (L + nk >= kMaxSentence) {
      const int cap_lane = nth_set_bit(keep_mask, kMaxSentence - L - 1);
      if (keep && lane <= cap_lane) {
        const int at = L + __popc(keep_mask & lanemask_lt());
        if (at < cap) sen[at] = tok;
      }
      L = kMaxSentence;
      consumed = cap_lane + 1;
      draws = p.sample_on ? cap_lane + 1 : 0;
      done = true;
    } else {
      if (keep) {
        const int at = L + __popc(keep_mask & lanemask_lt());
        if (at < cap) sen[at] = tok;
      }
      L += nk;
      if (first_stop < 32) {
        consumed = first_stop + 1;
        draws = p.sample_on ? first_stop : 0;
        done = true;
      } else {
        consumed = 32;
        draws = p.sample_on ? 32 : 0;
        done = false;
      }
    }
    cur += consumed;
    word_count += (uint64_t)consumed;
    rng = jump_small(rng, draws, sj);
    if (done) break;
  }
  if (L > cap) {
    if (lane == 0) atomicExch(&p.ctr->status, 1);
    L = cap;
  }
  __syncwarp();
  return L;
}

// ---- one group of negatives and the output list (dsgl.hpp:1136-1159) ---------------
// gstate: LCG state before the group's first draw.  Lanes < K draw; equal draws merge
// (meta = multiplicity, first occurrence keeps its place); draws equal to t1 are dropped.
// Writes out_id/out_meta[0..O) in the reference's order; returns O.
__device__ __forceinline__ int select_outputs(const TrainParams& p, const SmallJumps& sj,
                                              uint64_t gstate, int t1, int t2, int* out_id,
                                              int* out_meta) {
  const int lane = lane_id();
  const bool valid = lane < p.K;
  int s = -2 - lane;
  if (valid) {
    uint64_t st = jump_small(gstate, lane + 1, sj);
    s = __ldg(&p.table[fast_mod(st >> 16, p.div_table)]);
    if (!s) s = (int)(fast_mod(st, p.div_vm1) + 1);
  }
  const unsigned same = __match_any_sync(kFull, s);
  const bool leader = (__ffs(same) - 1) == lane;
  const unsigned distinct = __ballot_sync(kFull, valid && leader && s != t1);
  const int O = __popc(distinct) + 2;
  if (valid && leader && s != t1) {
    int idx = 1 + __popc(distinct & lanemask_lt());
    out_id[idx] = s;
    out_meta[idx] = __popc(same);
  }
  if (lane == 0) {
    out_id[0] = t1;
    out_meta[0] = 1;
    out_id[O - 1] = t2;
    out_meta[O - 1] = 1;
  }
  __syncwarp();
  return O;
}

// Same output list from K stored draws words[0..K) (the reference's neg_words group);
// also returns, for each output i in 1..O-2, the index k of its first draw in kidx.
__device__ __forceinline__ int select_outputs_stored(int K, const int* words, int t1, int t2,
                                                     int* out_id, int* out_meta, int* kidx) {
  const int lane = lane_id();
  const bool valid = lane < K;
  const int s = valid ? words[lane] : -2 - lane;
  const unsigned same = __match_any_sync(kFull, s);
  const bool leader = (__ffs(same) - 1) == lane;
  const unsigned distinct = __ballot_sync(kFull, valid && leader && s != t1);
  const int O = __popc(distinct) + 2;
  if (valid && leader && s != t1) {
    int idx = 1 + __popc(distinct & lanemask_lt());
    out_id[idx] = s;
    out_meta[idx] = __popc(same);
    kidx[idx] = lane;
  }
  if (lane == 0) {
    out_id[0] = t1;
    out_meta[0] = 1;
    out_id[O - 1] = t2;
    out_meta[O - 1] = 1;
  }
  __syncwarp();
  return O;
}

// trainers: buffered input row += update
template <class InPtr>
struct AddToInput {
  InPtr in_ptr;
  __device__ __forceinline__ void operator()(int j, int q, float4 a) const {
    float4* x = reinterpret_cast<float4*>(const_cast<float*>(in_ptr(j)));
    x[q] = add4(x[q], a);
  }
};
template <class InPtr>
__device__ __forceinline__ AddToInput<InPtr> add_to_input(InPtr f) {
  return AddToInput<InPtr>{f};
}

// ---- window input list (dsgl.hpp:1100-1132) ------------------------------------------
// Appends the positions c = pos - w + i, i in [b, 2w+1-b), i != w, 0 <= c < len in
// increasing order; slot_of(c) gives the row index stored in in_row.  Returns the count.
template <class SlotOf>
__device__ __forceinline__ int window_inputs(int pos, int len, int w, int b, int base, int* in_row,
                                             SlotOf slot_of) {
  const int lane = lane_id();
  int n = 0;
  for (int i0 = 0; i0 < 2 * w + 1; i0 += 32) {
    const int i = i0 + lane;
    const int c = pos - w + i;
    const bool ok = i >= b && i < 2 * w + 1 - b && i != w && c >= 0 && c < len;
    const unsigned m = __ballot_sync(kFull, ok);
    if (ok) in_row[base + n + __popc(m & lanemask_lt())] = slot_of(c);
    n += __popc(m);
  }
  return n;
}

// ---- step arithmetic ---------------------------------------------------------------
// in_ptr(j) -> const float* row of input j (16-byte aligned; shared or global memory).
// out_rows: O float rows of stride DP (shared memory).
// Forward: lane j computes f_ij for every output i, sequentially over k, then the
// reference gradient g = (label - sigma_table(f)) * alpha * meta (dsgl.hpp:1243-1272),
// stored transposed: corrT[j * OP + i].  Optional fp32 per-lane loss.
template <class InPtr>
__device__ __forceinline__ void forward_gradient(int I, int first, int O, int d, InPtr in_ptr,
                                                 const float* out_rows, int DP,
                                                 const int* out_meta, const float* exp_table,
                                                 float alpha, float* corrT, int OP,
                                                 bool want_loss, float& loss) {
  const int lane = lane_id();
  const int d4 = d >> 2;
  for (int j0 = 0; j0 < I; j0 += 32) {
    const int j = j0 + lane;
    const float4* x = reinterpret_cast<const float4*>(in_ptr(j < I ? j : I - 1));
    float f[kOMax];
#pragma unroll
    for (int i = 0; i < kOMax; i++) f[i] = 0.f;
    for (int k4 = 0; k4 < d4; k4++) {
      const float4 xv = x[k4];
#pragma unroll
      for (int i = 0; i < kOMax; i++) {
        if (i < O) {
          const float4 o = reinterpret_cast<const float4*>(out_rows + (size_t)i * DP)[k4];
          f[i] = __fmaf_rn(o.x, xv.x, f[i]);
          f[i] = __fmaf_rn(o.y, xv.y, f[i]);
          f[i] = __fmaf_rn(o.z, xv.z, f[i]);
          f[i] = __fmaf_rn(o.w, xv.w, f[i]);
        }
      }
    }
    if (j < I) {
#pragma unroll
      for (int i = 0; i < kOMax; i++) {
        if (i < O) {
          const int label = j < first ? (i == 0) : (i == O - 1);
          const float fi = f[i];
          float g;
          if (fi > (float)kMaxExp) {
            g = __fmul_rn((float)(label - 1), alpha);
          } else if (fi < -(float)kMaxExp) {
            g = __fmul_rn((float)label, alpha);
          } else {
            const int idx =
                __float2int_rz(__fmul_rn(__fadd_rn(fi, (float)kMaxExp), (float)kTableScale));
            g = __fmul_rn(__fsub_rn((float)label, exp_table[idx]), alpha);
          }
          corrT[j * OP + i] = __fmul_rn(g, (float)out_meta[i]);
          if (want_loss) {  // meta * softplus(-(2 label - 1) f) = -meta log sigma(+-f)
            const float z = label ? -fi : fi;
            loss += (float)out_meta[i] * (fmaxf(z, 0.f) + log1pf(__expf(-fabsf(z))));
          }
        }
      }
    }
  }
  __syncwarp();
}

// Backward.  Lane owns column chunks q = lane + 32 t (t < DCH, q < d/4).
//   md[i][t]  = sum_j corr[i][j] * in_j[q]     (outputMd, dsgl.hpp:1290), sequential j
//   in_j[q]  += sum_i corr[i][j] * out_i[q]     (inputM then buffer +=, dsgl.hpp:1309-1333),
//               sequential i, inputs applied in order j = 0..I-1.
// md is complete before any input row changes, as the reference's two GEMMs read the
// same pre-update inputM.
// apply_in(j, q, a) consumes input j's update chunk q (the trainers add it to the
// buffered row in place; the minibatch entry point stores it).
template <int DCH, class InPtr, class ApplyIn>
__device__ __forceinline__ void backward(int I, int O, int d, InPtr in_ptr, const float* out_rows,
                                         int DP, const float* corrT, int OP,
                                         float4 (&md)[kOMax][DCH], ApplyIn apply_in) {
  const int lane = lane_id();
  const int d4 = d >> 2;
#pragma unroll
  for (int i = 0; i < kOMax; i++)
#pragma unroll
    for (int t = 0; t < DCH; t++) md[i][t] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int j = 0; j < I; j++) {
    const float4* x = reinterpret_cast<const float4*>(in_ptr(j));
    float c[kOMax];
#pragma unroll
    for (int i = 0; i < kOMax; i++) c[i] = i < O ? corrT[j * OP + i] : 0.f;
#pragma unroll
    for (int t = 0; t < DCH; t++) {
      const int q = lane + 32 * t;
      if (q < d4) {
        const float4 xv = x[q];
#pragma unroll
        for (int i = 0; i < kOMax; i++)
          if (i < O) md[i][t] = fma4s(c[i], xv, md[i][t]);
      }
    }
  }
  float4 o[kOMax][DCH];
#pragma unroll
  for (int i = 0; i < kOMax; i++)
#pragma unroll
    for (int t = 0; t < DCH; t++) {
      const int q = lane + 32 * t;
      o[i][t] = (i < O && q < d4) ? reinterpret_cast<const float4*>(out_rows + (size_t)i * DP)[q]
                                  : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  for (int j = 0; j < I; j++) {
    float c[kOMax];
#pragma unroll
    for (int i = 0; i < kOMax; i++) c[i] = i < O ? corrT[j * OP + i] : 0.f;
#pragma unroll
    for (int t = 0; t < DCH; t++) {
      const int q = lane + 32 * t;
      if (q < d4) {
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int i = 0; i < kOMax; i++)
          if (i < O) a = fma4s(c[i], o[i][t], a);
        apply_in(j, q, a);
      }
    }
  }
  __syncwarp();
}

}  // namespace sgns
