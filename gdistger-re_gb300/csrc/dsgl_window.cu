// dsgl_window.cu -- the persistent DSGL engine (SGNS_ENGINE_PERSISTENT).
//
// One warp is one worker: the GPU counterpart of one compute thread of the reference's
// Train_SGNS_MPI (include/dsgl.hpp:783-1425).  A single launch runs every worker over
// its contiguous corpus slice (dsgl.hpp:811-826) for -iter passes, whatever the walk
// lengths, with no host round trip.  Per worker, shared memory holds
//   * the two walks in flight (rows after subsampling),
//   * their context rows while any position of the row lies in the sliding window
//     [pos-w, pos+w] -- one fp32 copy per distinct vertex per walk, exactly the
//     reference's per-walk deduplicated buffer, loaded when it enters the window and
//     written back (stochastically rounded for bf16 tables) when it leaves it,
//   * the step's output rows (target of each walk + shared negatives) and gradients;
// the window bookkeeping (vertex and count of each slot, slot of each position) lives in
// registers, one slot per lane.
// Negative rows are read from and added to Woh at each step, as the reference does for
// the two target rows (dsgl.hpp:1346-1356).  Dot products of the forward are summed as
// eight sequential partial sums (even and odd k of each quarter of [0, d)) combined
// pairwise; the backward keeps the reference's order.  The negative pool keeps the reference's
// draw stream (max(len1,len2)*K draws per pool, group neg_count % n per step,
// dsgl.hpp:1054-1073, 1136-1154) but is regenerated from its base LCG state instead of
// being stored.
#include <cuda_runtime.h>

#include "dsgl_device.cuh"

namespace sgns {

namespace {

constexpr int kHdrWords = 1004 + 132;  // sigmoid table (1001 -> 1004) + SmallJumps (528 B)

// Ring of position -> slot per walk, one entry per lane: position p's entry is held by
// lane p & 31, and at most 2w + 2 positions are in a window at once.
constexpr int kRing = 32;
static_assert(kRing >= 2 * (kWMax - 1) + 2, "the ring must hold 2w + 2 positions for every allowed window");

struct WinLayout {  // per-warp shared memory, in 4-byte words
  int NS, DP, OP, OM, IM, lmax, outI;
  int rows, corr, sen, inrow, outid, outmeta, pend, words;
};

__host__ __device__ inline WinLayout win_layout(int d, int w, int K, int lmax) {
  WinLayout L;
  L.NS = 2 * w + 2;  // resident slots per walk (2w+1 positions, +1 while a row enters)
  L.DP = d + 4;      // padded row stride: 32 lanes reading 32 rows hit 32 distinct banks
  L.OM = K <= 5 ? 7 : kOMax;  // the kernel variant's output capacity (K + 2 <= OM)
  L.OP = (L.OM + 1) & ~1;     // outputs rounded up to pairs
  L.IM = 4 * w;
  L.lmax = lmax;
  int off = 0;
  L.rows = off;  // window rows of both walks
  off += 2 * L.NS * L.DP;
  L.outI = off;  // the step's output rows, normal layout (stride DP)
  off += L.OP * L.DP;
  L.corr = off;  // duplicated gradient pairs, stride OP + 2 pairs per input
  off += L.IM * (L.OP + 2) * 2;
  L.sen = off;
  off += 2 * lmax;
  L.inrow = off;
  off += L.IM;
  L.outid = off;
  off += L.OM;
  L.outmeta = off;
  off += L.OM;
  L.pend = off;  // pending row loads: ids, then destination rows
  off += 2 * (w + 1);
  L.words = (off + 3) & ~3;
  return L;
}

template <int S>
__device__ __forceinline__ void load_row_to_smem(const void* tab, int64_t row, int d, float* dst) {
  const int d4 = d >> 2;
  for (int q = lane_id(); q < d4; q += 32)
    reinterpret_cast<float4*>(dst)[q] = RowIO<S>::load4(tab, row, d, q);
}
// Loads up to NB rows (ids[0..n)) into registers before storing any of them, so their
// DRAM round trips overlap; dst(u) is the shared-memory row of the u-th id.
template <int S, int DCH, int NB, class Dst>
__device__ __forceinline__ void load_rows_batched(const void* tab, const int* ids, int n, int d, Dst dst) {
  const int lane = lane_id(), d4 = d >> 2;
  for (int b0 = 0; b0 < n; b0 += NB) {
    float4 v[NB][DCH];
#pragma unroll
    for (int u = 0; u < NB; u++) {
      if (b0 + u < n) {
        const int row = ids[b0 + u];
#pragma unroll
        for (int t = 0; t < DCH; t++) {
          const int q = lane + 32 * t;
          if (q < d4) v[u][t] = RowIO<S>::load4(tab, row, d, q);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < NB; u++) {
      if (b0 + u < n) {
        float4* out = reinterpret_cast<float4*>(dst(b0 + u));
#pragma unroll
        for (int t = 0; t < DCH; t++) {
          const int q = lane + 32 * t;
          if (q < d4) out[q] = v[u][t];
        }
      }
    }
  }
}

template <int S>
__device__ __forceinline__ void store_row_from_smem(void* tab, int64_t row, int d, const float* src,
                                                    uint64_t ev) {
  const int d4 = d >> 2;
  for (int q = lane_id(); q < d4; q += 32)
    RowIO<S>::store4(tab, row, d, q, reinterpret_cast<const float4*>(src)[q], ev);
}

// kLoss: also accumulate the SGNS loss (compute_loss); without it no loss code is compiled
// into the step.  DFIX: the hidden size as a compile-time constant (0: read from p.d).  With
// d known, every shared-memory address of the step is a base register plus an immediate
// offset and the column-range guards vanish; the arithmetic is the same either way.
// TILE: lanes per input in the forward dot products (2: two lanes share an input while at
// most 16 inputs remain; the same bits), chosen by the autotuner.  NW: windows per step (2,
// the reference's step over two walks; 1, one walk per step).
template <int S, int DCH, int OM, bool kLoss, int DFIX, int TILE, int NW = 2>
__global__ void __launch_bounds__(256) window_engine_kernel(TrainParams p) {
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
  const int wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (wid >= p.workers) return;

  const int d = DFIX ? DFIX : p.d, w = p.window, K = p.K;
  // windows per step: two walks (the reference's step) or one; a single-window step keeps
  // target 2's slot as a placeholder copy of target 1 with multiplicity 0 (no coefficient,
  // no write)
  constexpr bool two = NW == 2;
  constexpr int n_walks = NW;
  const WinLayout L = win_layout(d, w, K, p.lmax);
  float* base = smem + kHdrWords + (threadIdx.x >> 5) * L.words;
  float* rows = base + L.rows;
  float* out_rows = base + L.outI;
  float2* corrP = reinterpret_cast<float2*>(base + L.corr);
  int* sen = reinterpret_cast<int*>(base + L.sen);
  int* in_row = reinterpret_cast<int*>(base + L.inrow);
  int* out_id = reinterpret_cast<int*>(base + L.outid);
  int* out_meta = reinterpret_cast<int*>(base + L.outmeta);
  int* pend_id = reinterpret_cast<int*>(base + L.pend);
  int* pend_row = pend_id + (w + 1);
  const int NS = L.NS, DP = L.DP, lmax = L.lmax;

  // dsgl.hpp:790-826
  uint64_t rng = (uint64_t)wid, word_count = 0, last_wc = 0, step_id = 0;
  const uint64_t words_num = (uint64_t)p.words_num, parts = (uint64_t)p.workers;
  uint64_t tw = words_num / parts;
  const int64_t start = (int64_t)(tw * (uint64_t)wid);
  if (words_num % parts > 0 && (uint64_t)wid == parts - 1) tw = words_num - (parts - 1) * tw;
  const int64_t end = start + (int64_t)tw;
  int64_t cur = start;
  int local_iter = p.iter;
  int len[2] = {0, 0}, pos[2] = {0, 0};
  // neg_g tracks neg_count % neg_n (the group of the step) without a division per step
  int train_sen_num = 0, neg_count = 0, neg_n = 1, neg_g = 0, grp_g = -1;
  bool change_neg = true;
  uint64_t pool_base = 0, grp_state = 0;
  float loss = 0.f;
  unsigned long long n_pairs = 0, n_steps = 0, n_outs = 0, n_loads = 0, n_stores = 0;
  // negatives of the next step, drawn one step ahead when the pool stays (pf_g >= 0)
  NegDraw pf{};
  int pf_g = -1;
  uint64_t pf_gs = 0;
  // rows entering the windows at the last transition: loaded then, widened and stored to
  // their slots just before the next forward (so no instruction waits on the load earlier)
  typename RowIO<S>::Raw ent[2][DCH];
  int ent_row[2] = {-1, -1};
  // the next step's output rows, gathered at the end of this step when both walks go on
  // and the pool stays (ov_ready): the loads then overlap the window transitions.  Only
  // the variant with registers to spare for them across the transitions does this (bf16,
  // d <= 128, K <= 5: +3.7%; the fp32 rows are twice the registers and spill, -10%).
  constexpr bool kPrefetchRows = S == STORE_BF16 && DCH == 1 && OM == 7;
  constexpr bool kMergedBackward = true;
  typename RowIO<S>::Raw ov[OM][DCH];
  bool ov_ready = false;
  int O_next = 0;
  __syncwarp();

  // The window slot tables live in registers: lane s holds, for each walk, the vertex of
  // slot s (sv), its count of window positions (sr; 0 = free) and, for the position p
  // with p & 31 == lane, the slot p is assigned to (rg).  Walk indices are run-time values
  // in some loops, so the per-walk copies are separate scalars selected by walk.
  int sv0 = 0, sv1 = 0, sr0 = 0, sr1 = 0, rg0 = 0, rg1 = 0;
  // Places position `position` of walk `walk` in the window: an existing slot of the same
  // vertex, or a free slot.  Returns the slot; *fresh says row *v_out must be loaded.
  auto enter_assign = [&](int walk, int position, bool* fresh_out, int* v_out) -> int {
    const int v = sen[walk * lmax + position];
    const int my_v = walk ? sv1 : sv0, my_r = walk ? sr1 : sr0;
    const unsigned hit = __ballot_sync(kFull, lane < NS && my_r > 0 && my_v == v);
    int s;
    bool fresh = false;
    if (hit) {
      s = __ffs(hit) - 1;
    } else {
      const unsigned fr = __ballot_sync(kFull, lane < NS && my_r == 0);
      s = __ffs(fr) - 1;
      fresh = true;
      if (s < 0) {  // cannot happen: at most 2w+2 distinct vertices are resident
        if (lane == 0) atomicExch(&p.ctr->status, 2);
        s = 0;
      }
    }
    if (lane == s) {
      if (walk) { sv1 = v; sr1 = my_r + 1; } else { sv0 = v; sr0 = my_r + 1; }
    }
    if (lane == (position & (kRing - 1))) {
      if (walk) rg1 = s; else rg0 = s;
    }
    *fresh_out = fresh;
    *v_out = v;
    return s;
  };
  // the first window of a freshly loaded walk: slots first, then one batched load
  auto enter_initial = [&](int walk, int hi) {
    int n = 0;
    for (int q = 0; q <= hi; q++) {
      bool fresh;
      int v;
      const int s = enter_assign(walk, q, &fresh, &v);
      if (fresh) {
        if (lane == 0) {
          pend_id[n] = v;
          pend_row[n] = walk * NS + s;
        }
        n++;
      }
    }
    __syncwarp();
    load_rows_batched<S, DCH, (DCH == 1 ? 8 : 4)>(p.wih, pend_id, n, d, [&](int u) { return rows + (size_t)pend_row[u] * DP; });
    n_loads += (unsigned long long)n;
    __syncwarp();
  };
  auto leave = [&](int walk, int position, uint64_t ev) {
    const int s = __shfl_sync(kFull, walk ? rg1 : rg0, position & (kRing - 1));
    const int r = __shfl_sync(kFull, walk ? sr1 : sr0, s) - 1;
    const int v = __shfl_sync(kFull, walk ? sv1 : sv0, s);
    if (lane == s) {
      if (walk) sr1 = r; else sr0 = r;
    }
    if (r == 0) {
      store_row_from_smem<S>(p.wih, v, d, rows + (size_t)(walk * NS + s) * DP, ev);
      n_stores++;
    }
  };
  auto flush_walk = [&](int walk, uint64_t ev) {
    const int my_r = walk ? sr1 : sr0, my_v = walk ? sv1 : sv0;
    unsigned live = __ballot_sync(kFull, lane < NS && my_r > 0);
    while (live) {
      const int s = __ffs(live) - 1;
      live &= live - 1;
      store_row_from_smem<S>(p.wih, __shfl_sync(kFull, my_v, s), d, rows + (size_t)(walk * NS + s) * DP, ev);
      n_stores++;
    }
    if (walk) sr1 = 0; else sr0 = 0;
  };

  while (true) {
    if (__builtin_expect(word_count - last_wc > 10000, 0)) {  // dsgl.hpp:886-897
      const uint64_t diff = word_count - last_wc;
      if (lane == 0) {
        unsigned long long now = atomicAdd(&p.ctr->wca, (unsigned long long)diff) + diff;
        *reinterpret_cast<volatile float*>(&p.ctr->alpha) = alpha_update(p, now);
      }
      last_wc = word_count;
      __syncwarp();
    }
    // Rare paths (learning-rate update, walk refill, epoch end, pool change, walk end) are
    // marked unlikely so the compiler keeps them off the per-step instruction stream.
    if (__builtin_expect(len[0] == 0 || (two && len[1] == 0), 0))
    for (int walk = 0; walk < n_walks; walk++) {  // dsgl.hpp:902-1030
      while (len[walk] == 0) {
        if (cur >= end) break;
        const int n = fill_walk(p, *sj, sen + walk * lmax, cur, end, word_count, rng, lmax);
        if (n <= 1) continue;
        len[walk] = n;
        pos[walk] = 0;
        enter_initial(walk, n - 1 < w ? n - 1 : w);
      }
    }
    if (__builtin_expect(cur >= end, 0)) {  // dsgl.hpp:1031-1050
      if (lane == 0) atomicAdd(&p.ctr->wca, (unsigned long long)(word_count - last_wc));
      if (--local_iter == 0) break;
      word_count = 0;
      last_wc = 0;
      cur = start;
      len[0] = len[1] = 0;
      ent_row[0] = ent_row[1] = -1;
      sr0 = sr1 = 0;
      ov_ready = false;
      continue;
    }
    if (__builtin_expect(change_neg, 0)) {  // dsgl.hpp:1054-1088: the pool is its base state and size
      pool_base = rng;
      neg_n = two && len[1] > len[0] ? len[1] : len[0];
      neg_g = neg_count % neg_n;
      rng = jump_any(rng, (uint64_t)neg_n * (uint64_t)K, p.jumps);
      change_neg = false;
      grp_g = -1;
      pf_g = -1;
      ov_ready = false;
    }

    // ---- one step (dsgl.hpp:1089-1368) ----
    // The step's stochastic-rounding event keys, computed off the write-back paths: lane k
    // holds the key of event kind k (targets 1 and 2, walks 0 and 1, negatives).
    const uint64_t sr_key =
        S == STORE_BF16 && lane <= EV_NEG ? sr_event_key(p.sr_seed, lane, (uint32_t)wid, step_id) : 0;
    const int t1 = sen[pos[0]], t2 = two ? sen[lmax + pos[1]] : t1;
    neg_count++;
    neg_g = neg_g + 1 == neg_n ? 0 : neg_g + 1;
    const int g = neg_g;
    NegDraw nd;
    if (__builtin_expect(g == pf_g, 1)) {
      nd = pf;
      grp_state = pf_gs;
    } else {
      uint64_t gs;
      if (g == 0) gs = pool_base;
      else if (g == grp_g + 1) gs = jump_small(grp_state, K, *sj);
      else gs = jump_any(pool_base, (uint64_t)g * (uint64_t)K, p.jumps);
      grp_state = gs;
      nd = neg_draw_issue(p, *sj, gs);
    }
    grp_g = g;
    const int d4 = d >> 2;
    // a walk that ends at this step completes at its transition below
    const bool end0 = pos[0] + 1 >= len[0], end1 = two && pos[1] + 1 >= len[1];
    int O;
    if (kPrefetchRows && __builtin_expect(ov_ready, 1)) {
      O = O_next;  // select_outputs and the gather ran at the end of the previous step
    } else {
      O = select_outputs(p, nd, t1, t2, out_id, out_meta, two ? 1 : 0);
      // Gather the output rows (targets and negatives) from Woh: every load is issued here
      // and kept raw; the window input lists are built while they are in flight.
#pragma unroll
      for (int i = 0; i < OM; i++) {
        const int row = i < O ? out_id[i] : 0;
#pragma unroll
        for (int t = 0; t < DCH; t++) {
          const int q = lane + 32 * t;
          ov[i][t] = (i < O && q < d4) ? RowIO<S>::load_raw(p.woh, row, d, q) : typename RowIO<S>::Raw{};
        }
      }
    }
    // The next step's negative draws (dsgl.hpp:1136-1154), issued a step ahead: the pool
    // stays unless two walks have completed once this step's transitions are done.
    if (train_sen_num + (int)end0 + (int)end1 < 2) {
      const int gn = neg_g + 1 == neg_n ? 0 : neg_g + 1;
      uint64_t gs;
      if (gn == 0) gs = pool_base;
      else if (gn == grp_g + 1) gs = jump_small(grp_state, K, *sj);
      else gs = jump_any(pool_base, (uint64_t)gn * (uint64_t)K, p.jumps);
      pf = neg_draw_issue(p, *sj, gs);
      pf_gs = gs;
      pf_g = gn;
    } else {
      pf_g = -1;
    }
    rng = lcg_next(rng);
    const int b = (int)fast_mod(rng, p.div_window);
    const int I0 = window_inputs<true>(pos[0], len[0], w, b, 0, in_row,
                                 [&](int c) { return __shfl_sync(kFull, rg0, c & (kRing - 1)); });
    const int I = I0 + (two ? window_inputs<true>(pos[1], len[1], w, b, I0, in_row,
                                                [&](int c) { return NS + __shfl_sync(kFull, rg1, c & (kRing - 1)); })
                            : 0);
#pragma unroll
    for (int i = 0; i < OM; i++)
#pragma unroll
      for (int t = 0; t < DCH; t++) {
        const int q = lane + 32 * t;
        if (i < O && q < d4) reinterpret_cast<float4*>(out_rows + (size_t)i * DP)[q] = RowIO<S>::widen(ov[i][t]);
      }
#pragma unroll
    for (int walk = 0; walk < 2; walk++) {
      if (ent_row[walk] >= 0) {
        float4* dst = reinterpret_cast<float4*>(rows + (size_t)ent_row[walk] * DP);
#pragma unroll
        for (int t = 0; t < DCH; t++) {
          const int q = lane + 32 * t;
          if (q < (d >> 2)) dst[q] = RowIO<S>::widen(ent[walk][t]);
        }
        ent_row[walk] = -1;
      }
    }
    __syncwarp();
    const float alpha = *reinterpret_cast<volatile float*>(&p.ctr->alpha);
    auto in_ptr = [&](int j) -> const float* { return rows + (size_t)in_row[j] * DP; };
    // two lanes per input for small rounds (d <= 128, K <= 5 only: the other variants have
    // no registers to spare)
    if (TILE == 2 && DCH == 1 && OM == 7)
      forward_gradient_two_lanes<OM>(I, I0, O, d, in_ptr, out_rows, DP, out_meta, exp_s, alpha, corrP, kLoss, loss);
    else
      forward_gradient_split8<OM>(I, I0, O, d, in_ptr, out_rows, DP, out_meta, exp_s, alpha, corrP,
                                  kLoss, loss);
    float4 md[OM][DCH];
    auto out_pair = [&](int pp, int q, float4& r0, float4& r1) {
      r0 = reinterpret_cast<const float4*>(out_rows + (size_t)(2 * pp) * DP)[q];
      r1 = 2 * pp + 1 < O ? reinterpret_cast<const float4*>(out_rows + (size_t)(2 * pp + 1) * DP)[q]
                          : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    // one pass over the inputs when no two of them share a window row (at most 32
    // inputs, distinct slots); otherwise outputMd first, then the updates
    bool merged = false;
    if (kMergedBackward && I <= 32) {
      const int r = lane < I ? in_row[lane] : -1 - lane;
      merged = !__any_sync(kFull, __popc(__match_any_sync(kFull, r)) > 1);
    }
    if (merged) backward_merged<OM, DCH, true>(I, O, d, in_ptr, out_pair, corrP, md);
    else backward<OM, DCH, true>(I, O, d, in_ptr, out_pair, corrP, md, add_to_input(in_ptr));
    {  // Woh += outputMd: target 1, target 2, then each negative (aliases follow that order)
      uint64_t e1 = 0, e2 = 0, en = 0;
      if (S == STORE_BF16) {
        e1 = __shfl_sync(kFull, sr_key, EV_TARGET1);
        e2 = __shfl_sync(kFull, sr_key, EV_TARGET2);
        en = __shfl_sync(kFull, sr_key, EV_NEG);
      }
      const int d4 = d >> 2;
#pragma unroll
      for (int t = 0; t < DCH; t++) {
        const int q = lane + 32 * t;
        if (q < d4) {
          // outputs are stored t1, t2, negatives (see select_outputs)
          const float4 b1 = reinterpret_cast<const float4*>(out_rows)[q];
          const float4 n1 = RowIO<S>::store4(p.woh, t1, d, q, add4(b1, md[0][t]), e1);
          float4 n2 = n1;
          if (two) {
            const float4 b2 = t2 == t1 ? n1 : reinterpret_cast<const float4*>(out_rows + DP)[q];
            n2 = RowIO<S>::store4(p.woh, t2, d, q, add4(b2, md[1][t]), e2);
          }
#pragma unroll
          for (int i = 2; i < OM; i++) {
            if (i < O) {
              const int row = out_id[i];
              const float4 bi = row == t2 ? n2 : reinterpret_cast<const float4*>(out_rows + (size_t)i * DP)[q];
              RowIO<S>::store4(p.woh, row, d, q, add4(bi, md[i][t]), en);
            }
          }
        }
      }
    }
    n_pairs += (unsigned long long)I;
    n_outs += (unsigned long long)(two ? O : O - 1);
    n_steps++;
    __syncwarp();
    // Both walks go on and the pool stays: select the next step's outputs and issue their
    // Woh loads now (after this step's Woh stores in program order, so they read the
    // updated rows); the window transitions below run while they are in flight.
    ov_ready = false;
    if (kPrefetchRows && !end0 && !end1 && pf_g >= 0) {
      const int t1n = sen[pos[0] + 1], t2n = two ? sen[lmax + pos[1] + 1] : t1n;
      O_next = select_outputs(p, pf, t1n, t2n, out_id, out_meta, two ? 1 : 0);
#pragma unroll
      for (int i = 0; i < OM; i++) {
        const int row = i < O_next ? out_id[i] : 0;
#pragma unroll
        for (int t = 0; t < DCH; t++) {
          const int q = lane + 32 * t;
          ov[i][t] = (i < O_next && q < d4) ? RowIO<S>::load_raw(p.woh, row, d, q) : typename RowIO<S>::Raw{};
        }
      }
      ov_ready = true;
    }

    // ---- positions, window moves, walk ends (dsgl.hpp:1372-1407) ----
    pos[0]++;
    pos[1]++;
    {
      // The memory order of the oracle: walk 0 (enter, leave), then walk 1 (enter, leave).
      // An entering row's load is issued at its place in that order; its value is stored
      // to the slot just before the next forward, so the load overlaps the next step's
      // set-up.  A later write-back of the same vertex in this transition (walk 0's leave
      // or flush before walk 1's enter reads) is ordered after the load by program order.
      const int d4 = d >> 2;
      for (int walk = 0; walk < n_walks; walk++) {
        const uint64_t ev = S == STORE_BF16 ? __shfl_sync(kFull, sr_key, EV_WALK0 + walk) : 0;
        if (__builtin_expect(pos[walk] >= len[walk], 0)) {
          flush_walk(walk, ev);
          len[walk] = 0;
          train_sen_num++;
        } else {
          const int P = pos[walk];
          if (P + w < len[walk]) {
            bool fresh;
            int v;
            const int s = enter_assign(walk, P + w, &fresh, &v);
            if (fresh) {
#pragma unroll
              for (int t = 0; t < DCH; t++) {
                const int q = lane + 32 * t;
                if (q < d4) ent[walk][t] = RowIO<S>::load_raw(p.wih, v, d, q);
              }
              ent_row[walk] = walk * NS + s;
              n_loads++;
            }
          }
          if (P - w - 1 >= 0) leave(walk, P - w - 1, ev);
        }
      }
    }
    if (train_sen_num >= 2) {
      change_neg = true;
      train_sen_num = 0;
    }
    step_id++;
  }

  // worker statistics
  if (kLoss) {
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(kFull, loss, o);
  }
  if (lane == 0) {
    atomicAdd(&p.ctr->pairs, n_pairs);
    atomicAdd(&p.ctr->steps, n_steps);
    atomicAdd(&p.ctr->outputs, n_outs);
    atomicAdd(&p.ctr->row_loads, n_loads);
    atomicAdd(&p.ctr->row_stores, n_stores);
    if (kLoss) atomicAdd(&p.ctr->loss, (double)loss);
    atomicSub(&p.ctr->active, 1);
  }
}

}  // namespace

size_t window_smem_bytes(int d, int window, int K, int lmax, int warps_per_cta) {
  const WinLayout L = win_layout(d, window, K, lmax);
  return sizeof(float) * ((size_t)kHdrWords + (size_t)warps_per_cta * L.words);
}

// hidden sizes with their own kernel (training without the loss); others read d at run time
constexpr int kFixedD[] = {64, 128, 256};
inline int fixed_d(int d) {
  for (int f : kFixedD)
    if (d == f) return f;
  return 0;
}

template <int S, int DCH, int OM, bool kLoss, int DFIX, int TILE>
static cudaError_t occupancy_d(int d, int w, int K, int lmax, int wpc, int* ctas) {
  const size_t smem = window_smem_bytes(d, w, K, lmax, wpc);
  cudaError_t e = cudaFuncSetAttribute(window_engine_kernel<S, DCH, OM, kLoss, DFIX, TILE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, window_engine_kernel<S, DCH, OM, kLoss, DFIX, TILE>,
                                                       32 * wpc, smem);
}
template <int S, int DCH, int OM, int DFIX>
static cudaError_t occupancy_tile(int d, int w, int K, int lmax, int wpc, int tile, int* ctas) {
  if constexpr (DCH == 1 && OM == 7)
    if (tile == 2) return occupancy_d<S, DCH, OM, false, DFIX, 2>(d, w, K, lmax, wpc, ctas);
  return occupancy_d<S, DCH, OM, false, DFIX, 1>(d, w, K, lmax, wpc, ctas);
}
template <int S, int DCH, int OM>
static cudaError_t occupancy_t(int d, int w, int K, int lmax, int wpc, int tile, int* ctas) {
  const int f = fixed_d(d);
  if constexpr (DCH == 1) {
    if (f == 64) return occupancy_tile<S, DCH, OM, 64>(d, w, K, lmax, wpc, tile, ctas);
    if (f == 128) return occupancy_tile<S, DCH, OM, 128>(d, w, K, lmax, wpc, tile, ctas);
  } else {
    if (f == 256) return occupancy_tile<S, DCH, OM, 256>(d, w, K, lmax, wpc, tile, ctas);
  }
  return occupancy_tile<S, DCH, OM, 0>(d, w, K, lmax, wpc, tile, ctas);
}

template <int S, int DCH, int OM, bool kLoss, int DFIX, int TILE, int NW = 2>
static cudaError_t launch_loss_t(const TrainParams& p, int wpc, cudaStream_t s) {
  const size_t smem = window_smem_bytes(p.d, p.window, p.K, p.lmax, wpc);
  cudaError_t e = cudaFuncSetAttribute(window_engine_kernel<S, DCH, OM, kLoss, DFIX, TILE, NW>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int blocks = (p.workers + wpc - 1) / wpc;
  window_engine_kernel<S, DCH, OM, kLoss, DFIX, TILE, NW><<<blocks, 32 * wpc, smem, s>>>(p);
  return cudaGetLastError();
}
template <int S, int DCH, int OM, bool kLoss, int DFIX>
static cudaError_t launch_tile_t(const TrainParams& p, int wpc, cudaStream_t s) {
  if constexpr (DCH == 1 && OM == 7)
    if (p.fwd_tile == 2) return launch_loss_t<S, DCH, OM, kLoss, DFIX, 2>(p, wpc, s);
  return launch_loss_t<S, DCH, OM, kLoss, DFIX, 1>(p, wpc, s);
}
template <int S, int DCH, int OM>
static cudaError_t launch_t(const TrainParams& p, int wpc, cudaStream_t s) {
  // single-window steps: the generic kernel (run-time d, one lane per input)
  if (p.windows == 1)
    return p.compute_loss ? launch_loss_t<S, DCH, OM, true, 0, 1, 1>(p, wpc, s)
                          : launch_loss_t<S, DCH, OM, false, 0, 1, 1>(p, wpc, s);
  if (p.compute_loss) return launch_tile_t<S, DCH, OM, true, 0>(p, wpc, s);
  const int f = fixed_d(p.d);
  if constexpr (DCH == 1) {
    if (f == 64) return launch_tile_t<S, DCH, OM, false, 64>(p, wpc, s);
    if (f == 128) return launch_tile_t<S, DCH, OM, false, 128>(p, wpc, s);
  } else {
    if (f == 256) return launch_tile_t<S, DCH, OM, false, 256>(p, wpc, s);
  }
  return launch_tile_t<S, DCH, OM, false, 0>(p, wpc, s);
}

// kernel variants: storage x column chunks per lane (d <= 128 or <= 256) x outputs per
// step (K <= 5 or K <= 10)
#define SGNS_WINDOW_DISPATCH(FN, ...)                                                         \
  do {                                                                                     \
    const bool wide_ = d > 128, small_ = K <= 5;                                           \
    if (storage == STORE_BF16) {                                                           \
      if (wide_) return small_ ? FN<STORE_BF16, 2, 7>(__VA_ARGS__) : FN<STORE_BF16, 2, kOMax>(__VA_ARGS__); \
      return small_ ? FN<STORE_BF16, 1, 7>(__VA_ARGS__) : FN<STORE_BF16, 1, kOMax>(__VA_ARGS__);            \
    }                                                                                      \
    if (wide_) return small_ ? FN<STORE_F32, 2, 7>(__VA_ARGS__) : FN<STORE_F32, 2, kOMax>(__VA_ARGS__);     \
    return small_ ? FN<STORE_F32, 1, 7>(__VA_ARGS__) : FN<STORE_F32, 1, kOMax>(__VA_ARGS__);                \
  } while (0)

cudaError_t window_engine_occupancy(int storage, int d, int w, int K, int lmax, int wpc, int tile, int* ctas) {
  SGNS_WINDOW_DISPATCH(occupancy_t, d, w, K, lmax, wpc, tile, ctas);
}

cudaError_t launch_window_engine(const TrainParams& p, int wpc, cudaStream_t s) {
  const int d = p.d, K = p.K, storage = p.storage;
  SGNS_WINDOW_DISPATCH(launch_t, p, wpc, s);
}

}  // namespace sgns
