// dsgl_plain.cu -- the plain DSGL engine (SGNS_ENGINE_PLAIN).
//
// The reference's compute loop (include/dsgl.hpp:876-1407) with its memory policy kept
// literally: a walk's distinct context rows are copied from Wih when the walk is loaded
// (inputBuffer, dsgl.hpp:940-962) and copied back over Wih when it ends
// (dsgl.hpp:1377-1398); a negative pool of max(len1,len2)*K draws is deduplicated and
// its rows copied from Woh (negativeBuffer, dsgl.hpp:1054-1088), updated there, and
// copied back after two walk completions (dsgl.hpp:1399-1407); target rows are
// updated in Woh directly (dsgl.hpp:1346-1356).
//
// One warp per worker; every worker's state and buffers live in HBM and each launch
// advances every worker by one pass of the loop body (one minibatch).  With one worker
// the result equals the reference's single-compute-thread run bit for bit.
#include <cuda_runtime.h>

#include "dsgl_device.cuh"

namespace sgns {

namespace {

struct PlainState {
  uint64_t rng, word_count, last_wc, step_id;
  int64_t start, end, cur;
  int32_t local_iter, len0, len1, pos0, pos1, nu0, nu1, train_sen_num;
  int32_t change_neg, neg_count, neg_n, n_neg, done, pad0;
  double loss;
  unsigned long long pairs, steps, outs, loads, stores;
};

struct PlainLayout {  // byte offsets inside one worker's scratch
  size_t sen, slot, uniq, negw, negslot, negbuf_ids, buf, negbuf, bytes;
};

__host__ __device__ inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

__host__ __device__ inline PlainLayout plain_layout(int d, int K, int lmax) {
  PlainLayout L;
  size_t off = align_up(sizeof(PlainState), 256);
  const size_t npool = (size_t)lmax * (K > 0 ? K : 1);
  L.sen = off;
  off += 2 * (size_t)lmax * 4;
  L.slot = off;
  off += 2 * (size_t)lmax * 4;
  L.uniq = off;
  off += 2 * (size_t)lmax * 4;
  L.negw = off;
  off += npool * 4;
  L.negslot = off;
  off += npool * 4;
  L.negbuf_ids = off;
  off += npool * 4;
  off = align_up(off, 256);
  L.buf = off;
  off += 2 * (size_t)lmax * d * 4;
  L.negbuf = off;
  off += npool * d * 4;
  L.bytes = align_up(off, 256);
  return L;
}

constexpr int kPlainWarps = 4;

// per-warp shared memory (words): output rows, interleaved output rows, gradient pairs,
// input offsets, output ids/meta/draw index (kOMax outputs)
__host__ __device__ inline size_t plain_warp_words(int d, int w, int K) {
  (void)K;
  const int DP = d + 4;
  (void)DP;
  return align_up((size_t)kOMax * d + (size_t)4 * w * (kOMax + 2) * 2 + 4 * w + 3 * kOMax, 4);
}

template <int S>
__device__ __forceinline__ void copy_table_row_to_buf(const void* tab, int64_t row, int d, float* dst) {
  for (int q = lane_id(); q < (d >> 2); q += 32)
    reinterpret_cast<float4*>(dst)[q] = RowIO<S>::load4(tab, row, d, q);
}
template <int S>
__device__ __forceinline__ void copy_buf_to_table_row(void* tab, int64_t row, int d, const float* src,
                                                      uint64_t ev) {
  for (int q = lane_id(); q < (d >> 2); q += 32)
    RowIO<S>::store4(tab, row, d, q, reinterpret_cast<const float4*>(src)[q], ev);
}

// first-occurrence deduplication of vals[0..n) (the reference's linear find):
// slot_of[i] = index of vals[i] in the distinct list uniq[0..nu).  Returns nu.
__device__ int dedupe_first_occurrence(const int* vals, int n, int* slot_of, int* uniq) {
  const int lane = lane_id();
  int nu = 0;
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int i = c0 + lane;
    bool first = false;
    if (i < n) {
      const int v = vals[i];
      first = true;
      for (int k = 0; k < i; k++)
        if (vals[k] == v) {
          first = false;
          break;
        }
    }
    const unsigned m = __ballot_sync(kFull, first);
    if (first) {
      const int sidx = nu + __popc(m & lanemask_lt());
      uniq[sidx] = vals[i];
      slot_of[i] = sidx;
    }
    nu += __popc(m);
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) {
    const int v = vals[i];
    for (int k = 0; k < i; k++)
      if (vals[k] == v) {
        slot_of[i] = slot_of[k];
        break;
      }
  }
  __syncwarp();
  return nu;
}

template <int S, int DCH>
__global__ void __launch_bounds__(32 * kPlainWarps) plain_step_kernel(TrainParams p) {
  extern __shared__ __align__(16) float smem[];
  float* exp_s = smem;
  SmallJumps* sj = reinterpret_cast<SmallJumps*>(smem + 1004);
  for (int i = threadIdx.x; i < kExpTableSize + 1; i += blockDim.x) exp_s[i] = p.exp_table[i];
  for (int i = threadIdx.x; i < 33; i += blockDim.x) {
    sj->mul[i] = p.jumps->small_mul[i];
    sj->add[i] = p.jumps->small_add[i];
  }
  __syncthreads();
  const int lane = lane_id();
  const int wid = blockIdx.x * kPlainWarps + (threadIdx.x >> 5);
  if (wid >= p.workers) return;

  const int d = p.d, w = p.window, K = p.K, lmax = p.lmax;
  float* wsm = smem + 1136 + (size_t)(threadIdx.x >> 5) * plain_warp_words(d, w, K);
  float* outI = wsm;
  float2* corrP = reinterpret_cast<float2*>(outI + (size_t)kOMax * d);
  int* in_off = reinterpret_cast<int*>(corrP + (size_t)4 * w * (kOMax + 2));
  int* out_id = in_off + 4 * w;
  int* out_meta = out_id + kOMax;
  int* kidx = out_meta + kOMax;

  const PlainLayout L = plain_layout(d, K, lmax);
  char* scr = static_cast<char*>(p.plain_state) + (size_t)wid * (size_t)p.plain_stride;
  PlainState* stp = reinterpret_cast<PlainState*>(scr);
  PlainState st = *stp;
  if (st.done) return;
  int* sen = reinterpret_cast<int*>(scr + L.sen);
  int* slot = reinterpret_cast<int*>(scr + L.slot);
  int* uniq = reinterpret_cast<int*>(scr + L.uniq);
  int* negw = reinterpret_cast<int*>(scr + L.negw);
  int* negslot = reinterpret_cast<int*>(scr + L.negslot);
  int* negids = reinterpret_cast<int*>(scr + L.negbuf_ids);
  float* buf = reinterpret_cast<float*>(scr + L.buf);
  float* negbuf = reinterpret_cast<float*>(scr + L.negbuf);
  int len[2] = {st.len0, st.len1}, pos[2] = {st.pos0, st.pos1}, nu[2] = {st.nu0, st.nu1};
  float loss = 0.f;
  // windows per step: two walks (the reference's step) or one; a single-window step keeps
  // target 2's slot as a placeholder copy of target 1 with multiplicity 0
  const bool two = p.windows == 2;
  const int n_walks = two ? 2 : 1;

  do {
    if (st.word_count - st.last_wc > 10000) {  // dsgl.hpp:886-897
      const uint64_t diff = st.word_count - st.last_wc;
      if (lane == 0) {
        unsigned long long now = atomicAdd(&p.ctr->wca, (unsigned long long)diff) + diff;
        *reinterpret_cast<volatile float*>(&p.ctr->alpha) = alpha_update(p, now);
      }
      st.last_wc = st.word_count;
      __syncwarp();
    }
    for (int walk = 0; walk < n_walks; walk++) {  // dsgl.hpp:902-1030
      while (len[walk] == 0) {
        if (st.cur >= st.end) break;
        int* wsen = sen + walk * lmax;
        const int n = fill_walk(p, *sj, wsen, st.cur, st.end, st.word_count, st.rng, lmax);
        if (n <= 1) continue;
        len[walk] = n;
        pos[walk] = 0;
        nu[walk] = dedupe_first_occurrence(wsen, n, slot + walk * lmax, uniq + walk * lmax);
        float* wbuf = buf + (size_t)walk * lmax * d;
        for (int s = 0; s < nu[walk]; s++)
          copy_table_row_to_buf<S>(p.wih, uniq[walk * lmax + s], d, wbuf + (size_t)s * d);
        st.loads += (unsigned long long)nu[walk];
        __syncwarp();
      }
    }
    if (st.cur >= st.end) {  // dsgl.hpp:1031-1050
      if (lane == 0) atomicAdd(&p.ctr->wca, (unsigned long long)(st.word_count - st.last_wc));
      if (--st.local_iter == 0) {
        st.done = 1;
        if (lane == 0) {
          atomicAdd(&p.ctr->pairs, st.pairs);
          atomicAdd(&p.ctr->steps, st.steps);
          atomicAdd(&p.ctr->outputs, st.outs);
          atomicAdd(&p.ctr->row_loads, st.loads);
          atomicAdd(&p.ctr->row_stores, st.stores);
          if (p.compute_loss) atomicAdd(&p.ctr->loss, st.loss);
          atomicSub(&p.ctr->active, 1);
        }
        break;
      }
      st.word_count = 0;
      st.last_wc = 0;
      st.cur = st.start;
      len[0] = len[1] = 0;
      break;
    }
    if (st.change_neg) {  // dsgl.hpp:1054-1088
      const uint64_t base = st.rng;
      st.neg_n = two && len[1] > len[0] ? len[1] : len[0];
      const int total = st.neg_n * K;
      uint64_t chunk = base;
      for (int c0 = 0; c0 < total; c0 += 32) {
        const int q = c0 + lane;
        if (q < total) {
          const uint64_t r = jump_small(chunk, lane + 1, *sj);
          int s = __ldg(&p.table[fast_mod(r >> 16, p.div_table)]);
          if (!s) s = (int)(fast_mod(r, p.div_vm1) + 1);
          negw[q] = s;
        }
        chunk = jump_small(chunk, 32, *sj);
      }
      st.rng = jump_any(base, (uint64_t)total, p.jumps);
      __syncwarp();
      st.n_neg = dedupe_first_occurrence(negw, total, negslot, negids);
      for (int s = 0; s < st.n_neg; s++)
        copy_table_row_to_buf<S>(p.woh, negids[s], d, negbuf + (size_t)s * d);
      st.loads += (unsigned long long)st.n_neg;
      st.change_neg = 0;
      __syncwarp();
    }

    // ---- one step (dsgl.hpp:1089-1368) ----
    const int t1 = sen[pos[0]], t2 = two ? sen[lmax + pos[1]] : t1;
    st.rng = lcg_next(st.rng);
    const int b = (int)fast_mod(st.rng, p.div_window);
    const int I0 = window_inputs(pos[0], len[0], w, b, 0, in_off,
                                 [&](int c) { return slot[c]; });
    const int I = I0 + (two ? window_inputs(pos[1], len[1], w, b, I0, in_off,
                                            [&](int c) { return lmax + slot[lmax + c]; })
                            : 0);
    st.neg_count++;
    const int g = st.neg_count % st.neg_n;
    const int O = select_outputs_stored(K, negw + (size_t)g * K, t1, t2, out_id, out_meta, kidx, two ? 1 : 0);
    {  // outputs: targets from Woh (global), negatives from the pool buffer
      float4 v[kOMax][DCH];
      const int d4 = d >> 2;
#pragma unroll
      for (int i = 0; i < kOMax; i++)
#pragma unroll
        for (int t = 0; t < DCH; t++) {
          const int q = lane + 32 * t;
          float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
          if (i < O && q < d4) {
            if (i == 0 || i == O - 1) x = RowIO<S>::load4(p.woh, out_id[i], d, q);
            else x = reinterpret_cast<const float4*>(negbuf + (size_t)negslot[g * K + kidx[i]] * d)[q];
          }
          v[i][t] = x;
        }
      store_out_interleaved<kOMax, DCH>(v, O, d, outI);
    }
    __syncwarp();
    const float alpha = *reinterpret_cast<volatile float*>(&p.ctr->alpha);
    auto in_ptr = [&](int j) -> const float* { return buf + (size_t)in_off[j] * d; };
    forward_gradient<kOMax>(I, I0, O, d, in_ptr, outI, out_meta, exp_s, alpha, corrP, p.compute_loss != 0,
                            loss);
    float4 md[kOMax][DCH];
    backward<kOMax, DCH>(I, O, d, in_ptr, [&](int pp, int q, float4& r0, float4& r1) { out_chunk_pair(outI, d, pp, q, r0, r1); }, corrP, md, add_to_input(in_ptr));
    {
      uint64_t e1 = 0, e2 = 0;
      if (S == STORE_BF16) {
        e1 = sr_event_key(p.sr_seed, EV_TARGET1, (uint32_t)wid, st.step_id);
        e2 = sr_event_key(p.sr_seed, EV_TARGET2, (uint32_t)wid, st.step_id);
      }
      const int d4 = d >> 2;
#pragma unroll
      for (int t = 0; t < DCH; t++) {
        const int q = lane + 32 * t;
        if (q < d4) {
          float4 mlast = md[0][t];
#pragma unroll
          for (int i = 1; i < kOMax; i++)
            if (i == O - 1) mlast = md[i][t];
          // Woh[target] += outputMd, re-reading the table as the reference does
          RowIO<S>::store4(p.woh, t1, d, q, add4(RowIO<S>::load4(p.woh, t1, d, q), md[0][t]), e1);
          if (two) RowIO<S>::store4(p.woh, t2, d, q, add4(RowIO<S>::load4(p.woh, t2, d, q), mlast), e2);
#pragma unroll
          for (int i = 1; i < kOMax - 1; i++) {
            if (i < O - 1) {
              float4* nb = reinterpret_cast<float4*>(negbuf + (size_t)negslot[g * K + kidx[i]] * d);
              nb[q] = add4(nb[q], md[i][t]);
            }
          }
        }
      }
    }
    st.pairs += (unsigned long long)I;
    st.outs += (unsigned long long)(two ? O : O - 1);
    st.steps++;
    __syncwarp();

    pos[0]++;
    pos[1]++;
    for (int walk = 0; walk < n_walks; walk++) {  // dsgl.hpp:1377-1398
      if (pos[walk] >= len[walk]) {
        const uint64_t ev =
            S == STORE_BF16 ? sr_event_key(p.sr_seed, EV_WALK0 + walk, (uint32_t)wid, st.step_id) : 0;
        const float* wbuf = buf + (size_t)walk * lmax * d;
        for (int s = 0; s < nu[walk]; s++)
          copy_buf_to_table_row<S>(p.wih, uniq[walk * lmax + s], d, wbuf + (size_t)s * d, ev);
        st.stores += (unsigned long long)nu[walk];
        len[walk] = 0;
        st.train_sen_num++;
        __syncwarp();
      }
    }
    if (st.train_sen_num >= 2) {  // dsgl.hpp:1399-1407
      const uint64_t ev =
          S == STORE_BF16 ? sr_event_key(p.sr_seed, EV_POOL, (uint32_t)wid, st.step_id) : 0;
      for (int s = 0; s < st.n_neg; s++)
        copy_buf_to_table_row<S>(p.woh, negids[s], d, negbuf + (size_t)s * d, ev);
      st.stores += (unsigned long long)st.n_neg;
      st.change_neg = 1;
      st.train_sen_num = 0;
      __syncwarp();
    }
    st.step_id++;
  } while (false);

  if (p.compute_loss) {
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(kFull, loss, o);
    st.loss += (double)loss;
  }
  st.len0 = len[0];
  st.len1 = len[1];
  st.pos0 = pos[0];
  st.pos1 = pos[1];
  st.nu0 = nu[0];
  st.nu1 = nu[1];
  __syncwarp();
  if (lane == 0) *stp = st;
}

__global__ void plain_init_kernel(TrainParams p) {
  const int wid = blockIdx.x * blockDim.x + threadIdx.x;
  if (wid >= p.workers) return;
  PlainState st{};
  st.rng = (uint64_t)wid;  // dsgl.hpp:791
  const uint64_t words_num = (uint64_t)p.words_num, parts = (uint64_t)p.workers;
  uint64_t tw = words_num / parts;  // dsgl.hpp:811-821
  st.start = (int64_t)(tw * (uint64_t)wid);
  if (words_num % parts > 0 && (uint64_t)wid == parts - 1) tw = words_num - (parts - 1) * tw;
  st.end = st.start + (int64_t)tw;
  st.cur = st.start;
  st.local_iter = p.iter;
  st.change_neg = 1;
  st.neg_n = 1;
  *reinterpret_cast<PlainState*>(static_cast<char*>(p.plain_state) + (size_t)wid * (size_t)p.plain_stride) = st;
}

inline size_t plain_smem(int d, int window, int K) {
  return sizeof(float) * (1136 + kPlainWarps * plain_warp_words(d, window, K));
}

template <int S, int DCH>
cudaError_t plain_launch_t(const TrainParams& p, cudaStream_t s) {
  const size_t smem = plain_smem(p.d, p.window, p.K);
  cudaError_t e = cudaFuncSetAttribute(plain_step_kernel<S, DCH>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  plain_step_kernel<S, DCH><<<(p.workers + kPlainWarps - 1) / kPlainWarps, 32 * kPlainWarps, smem, s>>>(p);
  return cudaGetLastError();
}

}  // namespace

size_t plain_worker_bytes(int d, int window, int K, int lmax) {
  (void)window;
  return plain_layout(d, K, lmax).bytes;
}

cudaError_t launch_plain_init(const TrainParams& p, cudaStream_t s) {
  plain_init_kernel<<<(p.workers + 127) / 128, 128, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_plain_step(const TrainParams& p, cudaStream_t s) {
  const bool wide = p.d > 128;
  if (p.storage == STORE_BF16) return wide ? plain_launch_t<STORE_BF16, 2>(p, s) : plain_launch_t<STORE_BF16, 1>(p, s);
  return wide ? plain_launch_t<STORE_F32, 2>(p, s) : plain_launch_t<STORE_F32, 1>(p, s);
}

}  // namespace sgns
