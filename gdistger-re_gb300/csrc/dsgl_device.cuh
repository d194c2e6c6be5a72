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

// Stochastic rounding of two floats to a bf16 pair in one instruction (sm_100a and later):
// lo gets rbits[15:0] and lands in the low half, hi gets rbits[31:16].  For every non-NaN
// input the result equals truncating (bits(x) + r16) to its upper 16 bits; NaN becomes
// 0x7FFF.
__device__ __forceinline__ uint32_t cvt_rs_bf16x2(float lo, float hi, uint32_t rbits) {
  uint32_t d;
  asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
  return d;
}

// ---- storage rows ------------------------------------------------------------------
// A row of d elements; column chunk q holds columns 4q..4q+3 (d % 4 == 0).
template <int S> struct RowIO;

template <> struct RowIO<STORE_F32> {
  static constexpr int kBytes = 4;
  typedef float4 Raw;  // a chunk as loaded, before widening to fp32
  __device__ static __forceinline__ Raw load_raw(const void* base, int64_t row, int d, int q) {
    return reinterpret_cast<const float4*>(static_cast<const float*>(base) + row * d)[q];
  }
  __device__ static __forceinline__ float4 widen(Raw r) { return r; }
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
  typedef uint2 Raw;
  __device__ static __forceinline__ Raw load_raw(const void* base, int64_t row, int d, int q) {
    return reinterpret_cast<const uint2*>(static_cast<const uint16_t*>(base) + row * d)[q];
  }
  __device__ static __forceinline__ float4 widen(Raw u) {
    return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xFFFF0000u),
                       __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xFFFF0000u));
  }
  __device__ static __forceinline__ float4 load4(const void* base, int64_t row, int d, int q) {
    return widen(load_raw(base, row, d, q));
  }
  // Stores with stochastic rounding; returns the values actually stored (as fp32).
  // Column 4q+j takes random bits [16j, 16j+16) of sr_bits4.
  __device__ static __forceinline__ float4 store4(void* base, int64_t row, int d, int q, float4 v,
                                                  uint64_t ev) {
    const uint64_t bits = sr_bits4(ev, (uint32_t)row, (uint32_t)q);
    const uint2 u = make_uint2(cvt_rs_bf16x2(v.x, v.y, (uint32_t)bits),
                               cvt_rs_bf16x2(v.z, v.w, (uint32_t)(bits >> 32)));
    reinterpret_cast<uint2*>(static_cast<uint16_t*>(base) + row * d)[q] = u;
    return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xFFFF0000u),
                       __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xFFFF0000u));
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
// Draw k of the group starting at LCG state gstate is made by lane k: its state and
// the table entry it indexes (a global load that may be issued a step ahead).
struct NegDraw {
  uint64_t st;
  int raw;
};
__device__ __forceinline__ NegDraw neg_draw_issue(const TrainParams& p, const SmallJumps& sj, uint64_t gstate) {
  NegDraw n;
  n.st = 0;
  n.raw = 0;
  if (lane_id() < p.K) {
    n.st = jump_small(gstate, lane_id() + 1, sj);
    n.raw = __ldg(&p.table[fast_mod(n.st >> 16, p.div_table)]);
  }
  return n;
}
// Equal draws merge (meta = multiplicity, first occurrence keeps its place); draws equal
// to t1 are dropped.  Writes out_id/out_meta[0..O) and returns O.  The reference orders
// the outputs t1, negatives, t2; they are stored t1, t2, negatives, so that target 2 sits
// at a fixed index (a run-time index into register arrays would put them in local
// memory).  Every sum whose order matters walks them in the reference's order.
// t2_meta: multiplicity of target 2 (0 in single-window steps, where t2 is a placeholder
// whose coefficients are zero and whose row is not written)
__device__ __forceinline__ int select_outputs(const TrainParams& p, NegDraw nd, int t1, int t2, int* out_id,
                                              int* out_meta, int t2_meta = 1) {
  const int lane = lane_id();
  const bool valid = lane < p.K;
  int s = -2 - lane;
  if (valid) s = nd.raw ? nd.raw : (int)(fast_mod(nd.st, p.div_vm1) + 1);
  const unsigned same = __match_any_sync(kFull, s);
  const bool leader = (__ffs(same) - 1) == lane;
  const unsigned distinct = __ballot_sync(kFull, valid && leader && s != t1);
  const int O = __popc(distinct) + 2;
  if (valid && leader && s != t1) {
    int idx = 2 + __popc(distinct & lanemask_lt());
    out_id[idx] = s;
    out_meta[idx] = __popc(same);
  }
  if (lane == 0) {
    out_id[0] = t1;
    out_meta[0] = 1;
    out_id[1] = t2;
    out_meta[1] = t2_meta;
  }
  __syncwarp();
  return O;
}

// Same output list from K stored draws words[0..K) (the reference's neg_words group);
// also returns, for each output i in 1..O-2, the index k of its first draw in kidx.
__device__ __forceinline__ int select_outputs_stored(int K, const int* words, int t1, int t2,
                                                     int* out_id, int* out_meta, int* kidx, int t2_meta = 1) {
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
    out_meta[O - 1] = t2_meta;
  }
  __syncwarp();
  return O;
}

// ---- window input list (dsgl.hpp:1100-1132) ------------------------------------------
// Appends the positions c = pos - w + i, i in [b, 2w+1-b), i != w, 0 <= c < len in
// increasing order; slot_of(c) gives the row index stored in in_row.  Returns the count.
// kEveryLane: slot_of is called by all 32 lanes (it may be a warp shuffle) with any c,
// valid or not, and must be safe for every c; otherwise only for valid positions.
template <bool kEveryLane = false, class SlotOf>
__device__ __forceinline__ int window_inputs(int pos, int len, int w, int b, int base, int* in_row,
                                             SlotOf slot_of) {
  const int lane = lane_id();
  int n = 0;
  for (int i0 = 0; i0 < 2 * w + 1; i0 += 32) {
    const int i = i0 + lane;
    const int c = pos - w + i;
    const bool ok = i >= b && i < 2 * w + 1 - b && i != w && c >= 0 && c < len;
    const unsigned m = __ballot_sync(kFull, ok);
    if (kEveryLane) {
      const int sl = slot_of(c);
      if (ok) in_row[base + n + __popc(m & lanemask_lt())] = sl;
    } else {
      if (ok) in_row[base + n + __popc(m & lanemask_lt())] = slot_of(c);
    }
    n += __popc(m);
  }
  return n;
}

// ---- step arithmetic ---------------------------------------------------------------
// Packed fp32x2 arithmetic (Blackwell FFMA2/FADD2): each half is an ordinary IEEE
// operation, so pairing two independent sums changes no result.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) { return __fadd2_rn(a, b); }

// Output-row layout of one step for at most OM outputs (OM = K + 2):
//   normal rows:      out[i * DP + c]                          (backward, table updates)
//   interleaved rows: outI[(p * d + c) * 2 + b] = out_{2p+b}[c]   (forward; a float4
//                     holds the pair (2p, 2p+1) for two consecutive columns)
//   gradients:        corrP[j * CS + i] = {g_ij, g_ij}          (duplicated pairs)
template <int OM>
struct StepShape {
  static constexpr int OMP = (OM + 1) & ~1;  // outputs rounded up to pairs
  static constexpr int NPAIR = OMP / 2;
  static constexpr int CS = OMP + 2;        // corrP row stride in pairs (16-byte rows)
};

// Rows 2p and 2p+1, columns 4q..4q+3, read back from the interleaved layout.
__device__ __forceinline__ void out_chunk_pair(const float* outI, int d, int p, int q, float4& r0, float4& r1) {
  const float4* src = reinterpret_cast<const float4*>(outI + ((size_t)p * d + 4 * q) * 2);
  const float4 a = src[0], b = src[1];
  r0 = make_float4(a.x, a.z, b.x, b.z);
  r1 = make_float4(a.y, a.w, b.y, b.w);
}

// Forward: lane j computes f_ij for every output i, sequentially over k (pairs of
// outputs share one FFMA2), then the reference gradient g = (label - sigma_table(f)) *
// alpha * meta (dsgl.hpp:1243-1272).  Optional fp32 per-lane loss.
template <int OM, class InPtr>
__device__ __forceinline__ void forward_gradient(int I, int first, int O, int d, InPtr in_ptr,
                                                 const float* outI, const int* out_meta,
                                                 const float* exp_table, float alpha, float2* corrP,
                                                 bool want_loss, float& loss) {
  typedef StepShape<OM> SS;
  const int lane = lane_id();
  const int d4 = d >> 2;
  for (int j0 = 0; j0 < I; j0 += 32) {
    const int j = j0 + lane;
    const float4* x = reinterpret_cast<const float4*>(in_ptr(j < I ? j : I - 1));
    float2 f[SS::NPAIR];
#pragma unroll
    for (int q = 0; q < SS::NPAIR; q++) f[q] = make_float2(0.f, 0.f);
    for (int k4 = 0; k4 < d4; k4++) {
      const float4 xv = x[k4];
      const float2 x0 = make_float2(xv.x, xv.x), x1 = make_float2(xv.y, xv.y);
      const float2 x2 = make_float2(xv.z, xv.z), x3 = make_float2(xv.w, xv.w);
#pragma unroll
      for (int q = 0; q < SS::NPAIR; q++) {
        if (2 * q < O) {
          const float4* op = reinterpret_cast<const float4*>(outI + ((size_t)q * d + 4 * k4) * 2);
          const float4 a = op[0], b = op[1];
          f[q] = ffma2(make_float2(a.x, a.y), x0, f[q]);
          f[q] = ffma2(make_float2(a.z, a.w), x1, f[q]);
          f[q] = ffma2(make_float2(b.x, b.y), x2, f[q]);
          f[q] = ffma2(make_float2(b.z, b.w), x3, f[q]);
        }
      }
    }
    if (j < I) {
#pragma unroll
      for (int i = 0; i < OM; i++) {
        if (i < O) {
          const int label = j < first ? (i == 0) : (i == O - 1);
          const float fi = (i & 1) ? f[i >> 1].y : f[i >> 1].x;
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
          const float gm = __fmul_rn(g, (float)out_meta[i]);
          corrP[j * SS::CS + i] = make_float2(gm, gm);
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

// Forward of the persistent engine: the same gradient, with each dot product summed as
// eight independent sequential partial sums -- the even and the odd k of each quarter of
// [0, d), each pair advanced by one FFMA2 on {o[k], o[k+1]} x {x[k], x[k+1]} -- combined
// as s_m = even_m + odd_m, f = (s_0 + s_1) + (s_2 + s_3) when d % 16 == 0; when not,
// [0, d) is one range and f = even + odd.  The oracle's window policy uses the same
// order.  out_rows: normal layout, stride DP.
// One round over inputs j0..j0+nj-1 with L lanes per input (NQ * L == 4 quarters per
// input, or kWhole: the whole range, one lane per input).  Lane pairs (L == 2) each hold
// (s0 + s1) or (s2 + s3) and add the other's with a shuffle (a + b == b + a bit for bit).
template <int NQ, int L, bool kWhole, int OM, class InPtr>
__device__ __forceinline__ void forward_round(int j0, int nj, int first, int O, int q4, InPtr in_ptr,
                                              const float* out_rows, int DP, const int* out_meta,
                                              const float* exp_table, float alpha, float2* corrP,
                                              bool want_loss, float& loss) {
  typedef StepShape<OM> SS;
  const int lane = lane_id();
  const int jl = lane / L, sub = lane % L;
  const int j = j0 + jl;
  const bool active = jl < nj;
  const float4* x = reinterpret_cast<const float4*>(in_ptr(active ? j : j0));
  const int m0 = sub * NQ;
  float2 f[OM][NQ];
#pragma unroll
  for (int i = 0; i < OM; i++)
#pragma unroll
    for (int m = 0; m < NQ; m++) f[i][m] = make_float2(0.f, 0.f);
  for (int k4 = 0; k4 < q4; k4++) {
    float4 xv[NQ];
#pragma unroll
    for (int m = 0; m < NQ; m++) xv[m] = x[(m0 + m) * q4 + k4];
#pragma unroll
    for (int i = 0; i < OM; i++) {
      const float4* orow = reinterpret_cast<const float4*>(out_rows + (size_t)i * DP);
#pragma unroll
      for (int m = 0; m < NQ; m++) {
        const float4 o = orow[(m0 + m) * q4 + k4];
        f[i][m] = ffma2(make_float2(o.x, o.y), make_float2(xv[m].x, xv[m].y), f[i][m]);
        f[i][m] = ffma2(make_float2(o.z, o.w), make_float2(xv[m].z, xv[m].w), f[i][m]);
      }
    }
  }
  float fv[OM];
#pragma unroll
  for (int i = 0; i < OM; i++) {
    if (kWhole) {
      fv[i] = __fadd_rn(f[i][0].x, f[i][0].y);
    } else if (NQ == 4) {
      const float s0 = __fadd_rn(f[i][0].x, f[i][0].y), s1 = __fadd_rn(f[i][1 % NQ].x, f[i][1 % NQ].y);
      const float s2 = __fadd_rn(f[i][2 % NQ].x, f[i][2 % NQ].y), s3 = __fadd_rn(f[i][3 % NQ].x, f[i][3 % NQ].y);
      fv[i] = __fadd_rn(__fadd_rn(s0, s1), __fadd_rn(s2, s3));
    } else {
      const float a = __fadd_rn(__fadd_rn(f[i][0].x, f[i][0].y), __fadd_rn(f[i][1 % NQ].x, f[i][1 % NQ].y));
      fv[i] = __fadd_rn(a, __shfl_xor_sync(kFull, a, 1));
    }
  }
  if (active && sub == 0) {
#pragma unroll
    for (int i = 0; i < OM; i++) {
      if (i < O) {
        const float fi = fv[i];
        const int label = j < first ? (i == 0) : (i == 1);  // outputs t1, t2, negatives
        float g;
        if (fi > (float)kMaxExp) {
          g = __fmul_rn((float)(label - 1), alpha);
        } else if (fi < -(float)kMaxExp) {
          g = __fmul_rn((float)label, alpha);
        } else {
          const int idx = __float2int_rz(__fmul_rn(__fadd_rn(fi, (float)kMaxExp), (float)kTableScale));
          g = __fmul_rn(__fsub_rn((float)label, exp_table[idx]), alpha);
        }
        const float gm = __fmul_rn(g, (float)out_meta[i]);
        corrP[j * SS::CS + i] = make_float2(gm, gm);
        if (want_loss) {
          const float z = label ? -fi : fi;
          loss += (float)out_meta[i] * (fmaxf(z, 0.f) + log1pf(__expf(-fabsf(z))));
        }
      }
    }
  }
}

// The split forward with two lanes per input while at most 16 inputs remain (each lane sums
// two of the four quarters): half the k-loop per lane for those rounds, the same bits.
template <int OM, class InPtr>
__device__ __forceinline__ void forward_gradient_two_lanes(int I, int first, int O, int d, InPtr in_ptr,
                                                        const float* out_rows, int DP, const int* out_meta,
                                                        const float* exp_table, float alpha, float2* corrP,
                                                        bool want_loss, float& loss) {
  if ((d & 15) == 0) {
    const int q4 = d >> 4;
    for (int j0 = 0; j0 < I;) {
      const int rem = I - j0;
      if (rem <= 16) {
        forward_round<2, 2, false, OM>(j0, rem, first, O, q4, in_ptr, out_rows, DP, out_meta, exp_table, alpha,
                                       corrP, want_loss, loss);
        j0 += rem;
      } else {
        const int nj = rem < 32 ? rem : 32;
        forward_round<4, 1, false, OM>(j0, nj, first, O, q4, in_ptr, out_rows, DP, out_meta, exp_table, alpha,
                                       corrP, want_loss, loss);
        j0 += nj;
      }
    }
  } else {
    for (int j0 = 0; j0 < I; j0 += 32)
      forward_round<1, 1, true, OM>(j0, I - j0 < 32 ? I - j0 : 32, first, O, d >> 2, in_ptr, out_rows, DP,
                                    out_meta, exp_table, alpha, corrP, want_loss, loss);
  }
  __syncwarp();
}

template <int OM, class InPtr>
__device__ __forceinline__ void forward_gradient_split8(int I, int first, int O, int d, InPtr in_ptr,
                                                        const float* out_rows, int DP, const int* out_meta,
                                                        const float* exp_table, float alpha, float2* corrP,
                                                        bool want_loss, float& loss) {
  typedef StepShape<OM> SS;
  const int lane = lane_id();
  const int nq = (d & 15) == 0 ? 4 : 1;  // quarters of [0, d) (one range when d % 16 != 0)
  const int q4 = (d >> 2) / nq;          // chunks of 4 columns per quarter
  for (int j0 = 0; j0 < I; j0 += 32) {
    const int j = j0 + lane;
    const float4* x = reinterpret_cast<const float4*>(in_ptr(j < I ? j : I - 1));
    float2 f[OM][4];
#pragma unroll
    for (int i = 0; i < OM; i++)
#pragma unroll
      for (int m = 0; m < 4; m++) f[i][m] = make_float2(0.f, 0.f);
    for (int k4 = 0; k4 < q4; k4++) {
      float4 xv[4];
#pragma unroll
      for (int m = 0; m < 4; m++) xv[m] = m < nq ? x[m * q4 + k4] : make_float4(0.f, 0.f, 0.f, 0.f);
      // Rows i >= O hold stale but readable data; their sums are never used, so the loop
      // runs over all OM rows without a branch.
#pragma unroll
      for (int i = 0; i < OM; i++) {
        const float4* orow = reinterpret_cast<const float4*>(out_rows + (size_t)i * DP);
#pragma unroll
        for (int m = 0; m < 4; m++) {
          if (m >= nq) continue;
          const float4 o = orow[m * q4 + k4];
          f[i][m] = ffma2(make_float2(o.x, o.y), make_float2(xv[m].x, xv[m].y), f[i][m]);
          f[i][m] = ffma2(make_float2(o.z, o.w), make_float2(xv[m].z, xv[m].w), f[i][m]);
        }
      }
    }
    if (j < I) {
#pragma unroll
      for (int i = 0; i < OM; i++) {
        if (i < O) {
          const int label = j < first ? (i == 0) : (i == 1);  // outputs t1, t2, negatives
          const float s0 = __fadd_rn(f[i][0].x, f[i][0].y), s1 = __fadd_rn(f[i][1].x, f[i][1].y);
          const float s2 = __fadd_rn(f[i][2].x, f[i][2].y), s3 = __fadd_rn(f[i][3].x, f[i][3].y);
          const float fi = __fadd_rn(__fadd_rn(s0, s1), __fadd_rn(s2, s3));
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
          const float gm = __fmul_rn(g, (float)out_meta[i]);
          corrP[j * SS::CS + i] = make_float2(gm, gm);
          if (want_loss) {
            const float z = label ? -fi : fi;
            loss += (float)out_meta[i] * (fmaxf(z, 0.f) + log1pf(__expf(-fabsf(z))));
          }
        }
      }
    }
  }
  __syncwarp();
}

// Stores the step's output rows from registers in the normal layout (stride DP).
template <int OM, int DCH>
__device__ __forceinline__ void store_out_normal(const float4 (&v)[OM][DCH], int O, int d, float* out_rows,
                                                 int DP) {
  const int lane = lane_id(), d4 = d >> 2;
#pragma unroll
  for (int t = 0; t < DCH; t++) {
    const int q = lane + 32 * t;
    if (q < d4) {
#pragma unroll
      for (int i = 0; i < OM; i++)
        if (i < O) reinterpret_cast<float4*>(out_rows + (size_t)i * DP)[q] = v[i][t];
    }
  }
}

// Backward.  Lane owns column chunks q = lane + 32 t (t < DCH, q < d/4), as two pairs.
//   md[i][t]  = sum_j corr[i][j] * in_j[q]     (outputMd, dsgl.hpp:1290), sequential j
//   in_j[q]  += sum_i corr[i][j] * out_i[q]     (inputM then buffer +=, dsgl.hpp:1309-1333),
//               sequential i, inputs applied in order j = 0..I-1.
// md is complete before any input row changes, as the reference's two GEMMs read the
// same pre-update inputM.  apply_in(j, q, a) consumes input j's update of chunk q.
// out_pair(p, q, r0, r1): rows 2p and 2p+1 of the step's outputs, columns 4q..4q+3.
// kT2Second: outputs are stored t1, t2, negatives (select_outputs); the sum over i still
// runs in the reference's order t1, negatives, t2, i.e. stored rows 0, 2..O-1, 1.
template <int OM, int DCH, bool kT2Second = false, class InPtr, class OutPair, class ApplyIn>
__device__ __forceinline__ void backward(int I, int O, int d, InPtr in_ptr, OutPair out_pair,
                                         const float2* corrP, float4 (&md)[OM][DCH], ApplyIn apply_in) {
  typedef StepShape<OM> SS;
  const int lane = lane_id();
  const int d4 = d >> 2;
  float2 mlo[OM][DCH], mhi[OM][DCH];
#pragma unroll
  for (int i = 0; i < OM; i++)
#pragma unroll
    for (int t = 0; t < DCH; t++) mlo[i][t] = mhi[i][t] = make_float2(0.f, 0.f);
  // the next input's row address is fetched one iteration ahead, off the dependency chain
  const float4* x_next = I > 0 ? reinterpret_cast<const float4*>(in_ptr(0)) : nullptr;
  for (int j = 0; j < I; j++) {
    const float4* x = x_next;
    x_next = reinterpret_cast<const float4*>(in_ptr(j + 1 < I ? j + 1 : j));
    const float4* cj = reinterpret_cast<const float4*>(corrP + j * SS::CS);
    float2 c[SS::OMP];
#pragma unroll
    for (int q = 0; q < SS::NPAIR; q++) {
      const float4 v = cj[q];
      c[2 * q] = make_float2(v.x, v.y);
      c[2 * q + 1] = make_float2(v.z, v.w);
    }
#pragma unroll
    for (int t = 0; t < DCH; t++) {
      const int q = lane + 32 * t;
      if (q < d4) {
        const float4 xv = x[q];
        const float2 xl = make_float2(xv.x, xv.y), xh = make_float2(xv.z, xv.w);
#pragma unroll
        for (int i = 0; i < OM; i++)
          if (i < O) {
            mlo[i][t] = ffma2(c[i], xl, mlo[i][t]);
            mhi[i][t] = ffma2(c[i], xh, mhi[i][t]);
          }
      }
    }
  }
#pragma unroll
  for (int i = 0; i < OM; i++)
#pragma unroll
    for (int t = 0; t < DCH; t++) md[i][t] = make_float4(mlo[i][t].x, mlo[i][t].y, mhi[i][t].x, mhi[i][t].y);
  float2 olo[SS::OMP][DCH], ohi[SS::OMP][DCH];
#pragma unroll
  for (int pp = 0; pp < SS::NPAIR; pp++)
#pragma unroll
    for (int t = 0; t < DCH; t++) {
      const int q = lane + 32 * t;
      float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0;
      if (2 * pp < O && q < d4) out_pair(pp, q, r0, r1);
      olo[2 * pp][t] = make_float2(r0.x, r0.y);
      ohi[2 * pp][t] = make_float2(r0.z, r0.w);
      olo[2 * pp + 1][t] = make_float2(r1.x, r1.y);
      ohi[2 * pp + 1][t] = make_float2(r1.z, r1.w);
    }
  // four inputs per iteration: eight independent chains; updates applied in input order
  for (int j0 = 0; j0 < I; j0 += 4) {
    float2 c[4][SS::OMP];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int j = j0 + u < I ? j0 + u : I - 1;
      const float4* cj = reinterpret_cast<const float4*>(corrP + j * SS::CS);
#pragma unroll
      for (int q = 0; q < SS::NPAIR; q++) {
        const float4 v = cj[q];
        c[u][2 * q] = make_float2(v.x, v.y);
        c[u][2 * q + 1] = make_float2(v.z, v.w);
      }
    }
#pragma unroll
    for (int t = 0; t < DCH; t++) {
      const int q = lane + 32 * t;
      if (q < d4) {
        float2 al[4], ah[4];
#pragma unroll
        for (int u = 0; u < 4; u++) al[u] = ah[u] = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < OM; k++) {
          // k-th term in the reference's order, as a stored row index (t2 comes last)
          const int i = !kT2Second ? k : (k == 0 ? 0 : (k == OM - 1 ? 1 : k + 1));
          const bool used = !kT2Second ? k < O : (k == 0 || k == OM - 1 || k + 1 < O);
          if (used) {
#pragma unroll
            for (int u = 0; u < 4; u++) {
              al[u] = ffma2(c[u][i], olo[i][t], al[u]);
              ah[u] = ffma2(c[u][i], ohi[i][t], ah[u]);
            }
          }
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (j0 + u < I) apply_in(j0 + u, q, make_float4(al[u].x, al[u].y, ah[u].x, ah[u].y));
      }
    }
  }
  __syncwarp();
}

// The same backward in one pass over the inputs, for steps in which no two inputs share a
// row: input j's row is read for outputMd and then updated, and no later input reads it,
// so every accumulator sees the same operands in the same order as backward<> above (md
// sequential in j, each input's update summed over the outputs in the reference's order,
// then added to the row).  One pass loads each input row and its coefficients once.
template <int OM, int DCH, bool kT2Second = false, class InPtr, class OutPair>
__device__ __forceinline__ void backward_merged(int I, int O, int d, InPtr in_ptr, OutPair out_pair,
                                                const float2* corrP, float4 (&md)[OM][DCH]) {
  typedef StepShape<OM> SS;
  const int lane = lane_id();
  const int d4 = d >> 2;
  float2 olo[SS::OMP][DCH], ohi[SS::OMP][DCH];
#pragma unroll
  for (int pp = 0; pp < SS::NPAIR; pp++)
#pragma unroll
    for (int t = 0; t < DCH; t++) {
      const int q = lane + 32 * t;
      float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0;
      if (2 * pp < O && q < d4) out_pair(pp, q, r0, r1);
      olo[2 * pp][t] = make_float2(r0.x, r0.y);
      ohi[2 * pp][t] = make_float2(r0.z, r0.w);
      olo[2 * pp + 1][t] = make_float2(r1.x, r1.y);
      ohi[2 * pp + 1][t] = make_float2(r1.z, r1.w);
    }
  float2 mlo[OM][DCH], mhi[OM][DCH];
#pragma unroll
  for (int i = 0; i < OM; i++)
#pragma unroll
    for (int t = 0; t < DCH; t++) mlo[i][t] = mhi[i][t] = make_float2(0.f, 0.f);
  float4* x_next = I > 0 ? reinterpret_cast<float4*>(const_cast<float*>(in_ptr(0))) : nullptr;
  for (int j = 0; j < I; j++) {
    float4* x = x_next;
    x_next = reinterpret_cast<float4*>(const_cast<float*>(in_ptr(j + 1 < I ? j + 1 : j)));
    const float4* cj = reinterpret_cast<const float4*>(corrP + j * SS::CS);
    float2 c[SS::OMP];
#pragma unroll
    for (int q = 0; q < SS::NPAIR; q++) {
      const float4 v = cj[q];
      c[2 * q] = make_float2(v.x, v.y);
      c[2 * q + 1] = make_float2(v.z, v.w);
    }
#pragma unroll
    for (int t = 0; t < DCH; t++) {
      const int q = lane + 32 * t;
      if (q < d4) {
        const float4 xv = x[q];
        const float2 xl = make_float2(xv.x, xv.y), xh = make_float2(xv.z, xv.w);
#pragma unroll
        for (int i = 0; i < OM; i++)
          if (i < O) {
            mlo[i][t] = ffma2(c[i], xl, mlo[i][t]);
            mhi[i][t] = ffma2(c[i], xh, mhi[i][t]);
          }
        float2 al = make_float2(0.f, 0.f), ah = al;
#pragma unroll
        for (int k = 0; k < OM; k++) {
          const int i = !kT2Second ? k : (k == 0 ? 0 : (k == OM - 1 ? 1 : k + 1));
          const bool used = !kT2Second ? k < O : (k == 0 || k == OM - 1 || k + 1 < O);
          if (used) {
            al = ffma2(c[i], olo[i][t], al);
            ah = ffma2(c[i], ohi[i][t], ah);
          }
        }
        const float2 lo = fadd2(xl, al), hi = fadd2(xh, ah);
        x[q] = make_float4(lo.x, lo.y, hi.x, hi.y);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < OM; i++)
#pragma unroll
    for (int t = 0; t < DCH; t++) md[i][t] = make_float4(mlo[i][t].x, mlo[i][t].y, mhi[i][t].x, mhi[i][t].y);
  __syncwarp();
}

// Stores the step's output rows from registers in the interleaved layout (see StepShape).
template <int OM, int DCH>
__device__ __forceinline__ void store_out_interleaved(const float4 (&v)[OM][DCH], int O, int d, float* outI) {
  typedef StepShape<OM> SS;
  const int lane = lane_id(), d4 = d >> 2;
#pragma unroll
  for (int t = 0; t < DCH; t++) {
    const int q = lane + 32 * t;
    if (q < d4) {
#pragma unroll
      for (int p = 0; p < SS::NPAIR; p++) {
        if (2 * p < O) {
          const float4 a = v[2 * p][t];
          const float4 b = (2 * p + 1 < OM && 2 * p + 1 < O) ? v[(2 * p + 1) < OM ? 2 * p + 1 : 0][t]
                                                            : make_float4(0.f, 0.f, 0.f, 0.f);
          float4* dst = reinterpret_cast<float4*>(outI + ((size_t)p * d + 4 * q) * 2);
          dst[0] = make_float4(a.x, b.x, a.y, b.y);
          dst[1] = make_float4(a.z, b.z, a.w, b.w);
        }
      }
    }
  }
}

// trainers: buffered input row += update
template <class InPtr>
struct AddToInput {
  InPtr in_ptr;
  __device__ __forceinline__ void operator()(int j, int q, float4 a) const {
    float4* x = reinterpret_cast<float4*>(const_cast<float*>(in_ptr(j)));
    const float4 v = x[q];
    const float2 lo = fadd2(make_float2(v.x, v.y), make_float2(a.x, a.y));
    const float2 hi = fadd2(make_float2(v.z, v.w), make_float2(a.z, a.w));
    x[q] = make_float4(lo.x, lo.y, hi.x, hi.y);
  }
};
template <class InPtr>
__device__ __forceinline__ AddToInput<InPtr> add_to_input(InPtr f) {
  return AddToInput<InPtr>{f};
}

// Loads the step's output rows (all loads in flight before any use) into registers.
template <int S, int OM, int DCH>
__device__ __forceinline__ void load_out_rows(const void* tab, const int* ids, int O, int d,
                                              float4 (&v)[OM][DCH]) {
  const int lane = lane_id(), d4 = d >> 2;
#pragma unroll
  for (int i = 0; i < OM; i++) {
    const int row = i < O ? ids[i] : 0;
#pragma unroll
    for (int t = 0; t < DCH; t++) {
      const int q = lane + 32 * t;
      v[i][t] = (i < O && q < d4) ? RowIO<S>::load4(tab, row, d, q) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

}  // namespace sgns
