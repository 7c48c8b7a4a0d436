// Tiny-node warp kernel, root construction, level scans and model emission.
#pragma once
#include "bag.cuh"
#include "fit_kernels.cuh"
#include "warp_rf.cuh"

namespace dml {

// ============================================================== tiny nodes
// Groups of G lanes (G = 8, 16 or 32) per node with at most G entries, 32/G
// nodes per warp: entries live in lanes.  RF sorts rank << 5 | lane keys with a
// register bitonic network, and the entropy numerator of every boundary comes
// from one group scan of each entry's own-class change.  Same
// candidate rules as the CTA kernels.  Every shuffle and ballot names only the
// group's lanes, so groups of one warp may hold nodes of different forests
// (RF and ERT, classification and regression) and run different try counts.
template <int G, class T>
__device__ __forceinline__ T grp_excl_scan(T v, int gl, unsigned gm) {
  T x = v;
#pragma unroll
  for (int o = 1; o < G; o <<= 1) {
    T y = __shfl_up_sync(gm, x, o, G);
    if (gl >= o) x += y;
  }
  return x - v;
}

template <int G, class T>
__device__ __forceinline__ T grp_sum(T v, unsigned gm) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gm, v, o, G);
  return v;
}

template <int CW, int G>
// Five resident CTAs per SM (51 registers, some spilled): the group scans and
// sorts wait on shuffle latency, and the extra warps hide it better than
// fewer at more registers (the group classes of the 1M x 128, 10-class fit
// took 135 / 115 / 106 ms at 3 / 4 / 5 CTAs per SM).  The node's class
// counts are read from global memory where the ERT gain needs them rather
// than held in registers.  Eight or more packed class words keep three CTAs
// (80 registers).
__global__ void __launch_bounds__(256, CW >= 8 ? 3 : 5) k_group_nodes(LevelArgs a) {
  constexpr int NPW = 32 / G;                 // nodes per warp
  constexpr int NS = (10 + G - 1) / G;        // ERT samples per lane
  const int lane = threadIdx.x & 31;
  const int gl = lane & (G - 1);
  const int gi = lane / G;
  const unsigned gm = G == 32 ? kFull : (((1u << G) - 1u) << (gi * G));
  const unsigned glt = ((1u << lane) - 1u) & gm;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nslots = (a.nwork + NPW - 1) / NPW;
  unsigned long long tries_done = 0, entries_done = 0;  // on group leaders
  for (int ws = gw; ws < nslots; ws += nwarps) {
    const int wi = ws * NPW + gi;
    if (wi >= a.nwork) continue;
    const int node = a.work[wi];
    const LNode nd = a.nodes[node];
    const ProbDesc& P = a.probs[nd.prob];
    const int C = P.C;
    const int m = nd.ecnt;
    const bool valid = gl < m;
    const int* rows = a.rowsA + nd.ebeg;
    const int* ncnt = a.cnt + (long long)node * a.Cmax;
    const int ml = max(1, P.min_leaf);
    const int row = valid ? __ldg(rows + gl) : 0;
    const int w = valid ? (a.wA ? __ldg(a.wA + nd.ebeg + gl) : 1) : 0;
    const int k = (valid && P.task == 0) ? __ldg(P.lab + row) : -1;
    const long long qv = (valid && P.task == 1) ? __ldg(P.q + row) : 0;
    long long prior = 0;
    if (P.task == 0) prior = entropy_prior(a.H, nd.n, C, [&](int c) { return (long long)ncnt[c]; });
    // RF classification: h(n), the class total of each lane's entry and the
    // bit planes of the group's largest weight, fixed across tries
    const long long Hn = P.task == 0 ? __ldg(a.H + nd.n) : 0;
    const int Nk = (P.task == 0 && valid) ? __ldg(ncnt + k) : 0;
    int wbits;
    {
      int wm = w;
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) wm = max(wm, __shfl_xor_sync(gm, wm, o, G));
      wbits = 32 - __clz(max(wm, 1));
    }
    Cand best;
    best.valid = 0;
    // RF classification with value ranks: a candidate carries the ranks on both
    // sides of its boundary (in suml, a regression field) and its threshold is
    // read from the value table once per node, after the try loop: tries of
    // one feature give one candidate, so the threshold never decides between
    // tries.  The entries' values are then never gathered during the search.
    const bool defer_thr = P.algo == 0 && P.task == 0 && P.rank != nullptr && P.N <= (1ll << 26);
    // the features of tries 0 .. 31, computed by the group's lanes at once
    constexpr int NT = 32 / G;
    const int ntry = P.n_mand + P.n_opt;
    int fpre[NT];
#pragma unroll
    for (int r = 0; r < NT; ++r) fpre[r] = gl + G * r < ntry ? feature_of_try(P, nd, gl + G * r) : 0;
    for (int t = 0;; ++t) {
      int f;
      if (t < 32) {
        int fr = fpre[0];
#pragma unroll
        for (int r = 1; r < NT; ++r)
          if (t / G == r) fr = fpre[r];
        f = __shfl_sync(gm, fr, t % G, G);
      } else {
        f = feature_of_try(P, nd, t);
      }
      const float* xf = P.X + (long long)f * P.N;
      // RF with value ranks: rank << 5 | group lane as one 32-bit sort key
      // (invalid lanes sort last with their own lane index)
      const bool r32 = P.algo == 0 && P.rank != nullptr && P.N <= (1ll << 26);
      const float xv = valid && !defer_thr ? __ldg(xf + row) : 0.0f;
      Cand cd;
      cd.f = f;
      if (P.algo == 1) {  // ERT: sample s is held by lane s % G, slot s / G
        float sv[NS];
#pragma unroll
        for (int r = 0; r < NS; ++r) {
          const int smp = gl + G * r;
          sv[r] = 0.0f;
          if (smp < 10) {
            U4 rr = keyed(P.seed, kTagSample, (uint32_t)nd.depth, (uint32_t)(nd.tree + P.tree_key0),
                          (uint32_t)nd.idx, (uint32_t)(t * 3 + smp / 4));
            uint32_t pos = pick(rr, smp & 3) % (uint32_t)m;
            sv[r] = __ldg(xf + __ldg(rows + pos));
          }
        }
        float acc = 0.0f;
#pragma unroll
        for (int smp = 0; smp < 10; ++smp)
          acc = __fadd_rn(acc, __shfl_sync(gm, sv[smp / G], smp % G, G));
        const float thr = __fdiv_rn(acc, 10.0f);
        const bool left = valid && goes_left(xv, thr);
        const unsigned lm = __ballot_sync(gm, left);
        const long long nl = __popc(lm);
        const long long nr = (long long)nd.n - nl;
        cd.thr = thr;
        cd.nl_e = (int)nl;
        cd.nl = (int)nl;
        cd.suml = 0;
        cd.valid = nl >= ml && nr >= ml;
        if (P.task == 0) {
          int Lc[2 * CW];
#pragma unroll
          for (int c = 0; c < 2 * CW; ++c)
            Lc[c] = c < C ? __popc(__ballot_sync(gm, k == c) & lm) : 0;
          cd.gain = cd.valid ? entropy_gain_u<2 * CW>(
                                   a.H, prior, C, nl, nr, [&](int c) { return (long long)Lc[c]; },
                                   [&](int c) { return (long long)__ldg(ncnt + c); })
                             : -FLT_MAX;
        } else {
          long long sl = grp_sum<G, long long>(left ? qv : 0, gm);
          cd.suml = sl;
          cd.gain = cd.valid ? variance_gain(nl, sl, nr, nd.sum - sl, P.S) : -FLT_MAX;
        }
      } else {  // RF: bitonic sort of (key, lane) over the group
        uint32_t key;
        int idx;
        if (r32) {
          uint32_t pk32 = valid ? (__ldg(P.rank + (long long)f * P.N + row) << 5) | (uint32_t)gl
                                : 0xFFFFFFE0u | (uint32_t)gl;
#pragma unroll
          for (int kk = 2; kk <= G; kk <<= 1) {
#pragma unroll
            for (int j = kk >> 1; j > 0; j >>= 1) {
              const uint32_t o = __shfl_xor_sync(gm, pk32, j, G);
              const bool up = (gl & kk) == 0;
              const bool lower = (gl & j) == 0;
              const uint32_t mn = min(pk32, o), mx = max(pk32, o);
              pk32 = (lower == up) ? mn : mx;
            }
          }
          key = gl < m ? pk32 >> 5 : 0xFFFFFFFFu;
          idx = (int)(pk32 & 31u);
        } else {
          key = valid ? orderable(xv) : 0xFFFFFFFFu;
          idx = gl;
#pragma unroll
          for (int kk = 2; kk <= G; kk <<= 1) {
#pragma unroll
            for (int j = kk >> 1; j > 0; j >>= 1) {
              uint32_t pk = __shfl_xor_sync(gm, key, j, G);
              int pi = __shfl_xor_sync(gm, idx, j, G);
              bool up = (gl & kk) == 0;
              bool lower = (gl & j) == 0;
              bool mine_smaller = key < pk || (key == pk && idx < pi);
              bool keep = (lower == up) ? mine_smaller : !mine_smaller;
              if (!keep) {
                key = pk;
                idx = pi;
              }
            }
          }
        }
        // group lane p now holds sorted position p, originally group lane idx
        const int ke = __shfl_sync(gm, k, idx, G);
        const int we = __shfl_sync(gm, w, idx, G);
        const long long qe = __shfl_sync(gm, qv, idx, G);
        const float xe = defer_thr ? 0.0f : __shfl_sync(gm, xv, idx, G);
        const uint32_t prevk = __shfl_up_sync(gm, key, 1, G);
        const float prevx = defer_thr ? 0.0f : __shfl_up_sync(gm, xe, 1, G);
        const long long nl = grp_excl_scan<G, long long>(we, gl, gm);
        const long long nr = (long long)nd.n - nl;
        bool bnd = gl > 0 && gl < m && prevk < key && nl >= ml && nr >= ml;
        float g = -FLT_MAX;
        long long sl = 0;
        if (P.task == 0) {
          // gain numerator P - Q = h(n) - h(nL) - h(nR) + sum over the positions q
          // left of the boundary of the change that moving q's entry to the left
          // makes to sum_c h(L_c) + h(N_c - L_c): only its own class c changes,
          // from L_c (the weight of class c at positions below q: the lanes
          // matching its class, summed over the weights' bit planes)
          const int Ne = __shfl_sync(gm, Nk, idx, G);
          const bool ve = gl < m;
          const unsigned below = __match_any_sync(gm, ve ? ke : -1) & glt;
          int Lo = 0;
          for (int b = 0; b < wbits; ++b)
            Lo += __popc(__ballot_sync(gm, (we >> b) & 1) & below) << b;
          long long dq = 0;
          if (ve) {
            const int R = Ne - Lo;
            dq = (__ldg(a.H + Lo + we) - __ldg(a.H + Lo)) + (__ldg(a.H + R - we) - __ldg(a.H + R));
          }
          const long long S = grp_excl_scan<G, long long>(dq, gl, gm);
          if (bnd) g = gain_from_numerator(Hn - __ldg(a.H + nl) - __ldg(a.H + nr) + S, nd.n);
        } else {
          sl = grp_excl_scan<G, long long>(qe * (long long)we, gl, gm);
          if (bnd) g = variance_gain(nl, sl, nr, nd.sum - sl, P.S);
        }
        // group argmax: valid, higher gain, lower position
        int bp = bnd ? gl : -1;
        float bg = g;
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
          float g2 = __shfl_xor_sync(gm, bg, o, G);
          int p2 = __shfl_xor_sync(gm, bp, o, G);
          bool take = p2 >= 0 && (bp < 0 || g2 > bg || (g2 == bg && p2 < bp));
          if (take) {
            bg = g2;
            bp = p2;
          }
        }
        const int src = bp >= 0 ? bp : 0;
        const long long nlb = __shfl_sync(gm, nl, src, G);
        const long long slb = __shfl_sync(gm, sl, src, G);
        float thr = 0.0f;
        long long ranks = 0;
        if (defer_thr) {
          ranks = ((long long)__shfl_sync(gm, prevk, src, G) << 32) |
                  (long long)__shfl_sync(gm, key, src, G);
        } else {
          const float xa = __shfl_sync(gm, prevx, src, G);
          const float xb = __shfl_sync(gm, xe, src, G);
          thr = midpoint_threshold(xa, xb);
        }
        if (bp >= 0) {
          cd.valid = 1;
          cd.gain = bg;
          cd.thr = thr;
          cd.nl_e = bp;
          cd.nl = (int)nlb;
          cd.suml = defer_thr ? ranks : slb;
        } else {
          cd.valid = 0;
          cd.gain = -FLT_MAX;
          cd.thr = 0.0f;
          cd.nl_e = cd.nl = 0;
          cd.suml = 0;
        }
      }
      // try-loop decision (uniform across the group)
      bool more;
      if (t < P.n_mand) {
        if (t == 0 || better(cd, best)) best = cd;
        more = (t + 1 < P.n_mand) || (P.n_opt > 0 && !(best.valid && best.gain >= kSensible));
      } else {
        if (better(cd, best)) best = cd;
        more = !(cd.valid && cd.gain >= kSensible) && (t + 1 < P.n_mand + P.n_opt);
      }
      if (!more) {
        if (gl == 0) {
          tries_done += (unsigned long long)(t + 1) * m;
          entries_done += m;
        }
        break;
      }
    }
    if (!best.valid) {
      if (gl == 0) write_leaf(a.res, node);
      continue;
    }
    if (defer_thr) {
      const float* vf = P.vals + (long long)best.f * P.N;
      best.thr = midpoint_threshold(__ldg(vf + (uint32_t)((unsigned long long)best.suml >> 32)),
                                    __ldg(vf + (uint32_t)best.suml));
      best.suml = 0;
    }
    if (gl == 0) write_result(a.res, a.res_cnt, a.Cmax, node, best, nullptr, 0);
    // stable partition with one ballot; the left class counts of the split
    const float xb = valid ? __ldg(P.X + (long long)best.f * P.N + row) : 0.0f;
    const bool left = valid && goes_left(xb, best.thr);
    const unsigned lm = __ballot_sync(gm, left);
    if (P.task == 0)
      for (int c = 0; c < C; ++c) {
        const int lc = grp_sum<G, int>(left && k == c ? w : 0, gm);
        if (gl == (c & (G - 1))) a.res_cnt[(long long)node * a.Cmax + c] = lc;
      }
    if (valid) {
      int pos = __popc(lm & glt);
      long long dst = nd.ebeg + (left ? pos : best.nl_e + (gl - pos));
      a.rowsB[dst] = row;
      if (a.wB) a.wB[dst] = w;
    }
  }
  tries_done = warp_sum<unsigned long long>(tries_done);
  entries_done = warp_sum<unsigned long long>(entries_done);
  if (lane == 0 && tries_done) {
    atomicAdd((unsigned long long*)&a.stats[2], tries_done);
    atomicAdd((unsigned long long*)&a.stats[3], entries_done);
  }
}

// ============================================================ work queues
// Node classes: tiny (<= 8, 16, 32 entries: lane groups), RF warp (up to 64,
// 128, 256, 512 entries), ERT warp (up to 256), ERT (CTA), RF small (CTA,
// shared-memory sort), RF big (per-try items, global sort).  Queue order does
// not affect results, only scheduling.
enum { kQWarp = 0, kQErt = 1, kQRfSmall = 2, kQRfBig = 3, kQRfW2 = 4, kQRfW4 = 5, kQRfW8 = 6,
       kQG16 = 7, kQG8 = 8, kQRfW16 = 9, kQErtW = 10, kNumQ = 11 };

struct Queues {
  int* list[kNumQ];
  int* count;  // [kNumQ]
  int rf_small_cap;  // RF nodes up to this many entries sort in shared memory
  int rf_warp_max;   // RF nodes up to this many entries (64, 128, 256 or 512) sort in a warp
};

// Warp-aggregated append of `node` to queue q (all lanes call; `want` selects).
__device__ __forceinline__ void enqueue(Queues Q, int q, int node, bool want) {
  for (int qq = 0; qq < kNumQ; ++qq) {
    bool mine = want && q == qq;
    unsigned m = __ballot_sync(kFull, mine);
    if (m == 0) continue;
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&Q.count[qq], __popc(m));
    base = __shfl_sync(kFull, base, leader);
    if (mine) Q.list[qq][base + __popc(m & ((1u << lane) - 1u))] = node;
  }
}

// The node class of a node with ecnt entries.  The RF thresholds come from
// the fit's tuning; every class computes the same split.
__device__ __forceinline__ int queue_of(const ProbDesc& P, int ecnt, const Queues& Q) {
  if (ecnt <= 8) return kQG8;
  if (ecnt <= 16) return kQG16;
  if (ecnt <= 32) return kQWarp;
  if (P.algo == 1) return ecnt <= 256 ? kQErtW : kQErt;
  if (ecnt <= 64 && Q.rf_warp_max >= 64) return kQRfW2;
  if (ecnt <= 128 && Q.rf_warp_max >= 128) return kQRfW4;
  if (ecnt <= 256 && Q.rf_warp_max >= 256) return kQRfW8;
  if (ecnt <= 512 && Q.rf_warp_max >= 512) return kQRfW16;
  return ecnt <= Q.rf_small_cap ? kQRfSmall : kQRfBig;
}

__device__ __forceinline__ bool preleaf(const ProbDesc& P, int n, int depth) {
  return n <= P.min_node_size || depth >= P.max_depth;
}

#ifndef DML_SEARCH_CW  // driver-only kernels (fit.cu)
// ============================================================ roots
// RF bootstrap multiplicities: row r of tree t is drawn w[r] times among the
// tree's bag draws (bag.cuh).
__global__ void k_boot_count(const ProbDesc* probs, const int* tree_prob, int* wcnt,
                             int chunk) {
  const int gt = blockIdx.y;
  const ProbDesc& P = probs[tree_prob[gt]];
  if (P.algo != 0) return;
  const int t = gt - P.tree0;
  long long slot0 = P.ent0 + (long long)t * P.N;
  long long beg = (long long)blockIdx.x * chunk;
  long long end = min(bag_draws(P), beg + chunk);
  for (long long i = beg + threadIdx.x; i < end; i += blockDim.x) {
    const long long row = bag_draw(P, t, i);
    if (row >= 0) atomicAdd(&wcnt[slot0 + row], 1);
  }
}

// One CTA per tree: compact the rows with non-zero weight (ascending) into
// the entry slots and build the root node.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_roots(const ProbDesc* probs, const int* tree_prob,
                                                 const int* wcnt, int* rows, int* wts,
                                                 LNode* nodes, int* cnt, int Cmax, NodeRes* res,
                                                 Queues Q, long long* stats) {
  __shared__ int sm[BLOCK / 32];
  __shared__ int s_cnt[kMaxClasses];
  __shared__ unsigned long long s_sum;
  __shared__ unsigned long long s_n;
  const int gt = blockIdx.x;
  const int pi = tree_prob[gt];
  const ProbDesc& P = probs[pi];
  const int t = gt - P.tree0;
  const long long slot0 = P.ent0 + (long long)t * P.N;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < kMaxClasses) s_cnt[threadIdx.x] = 0;
  if (threadIdx.x == 0) {
    s_sum = 0;
    s_n = 0;
  }
  __syncthreads();
  int out = 0;
  for (long long base = 0; base < P.N; base += BLOCK) {
    long long r = base + threadIdx.x;
    int w = 0;
    if (r < P.N) w = P.algo == 0 ? wcnt[slot0 + r] : 1;
    int tot;
    int pos = block_excl_scan<BLOCK, int>(w > 0 ? 1 : 0, &tot, sm);
    if (w > 0) {
      rows[slot0 + out + pos] = (int)r;
      if (wts) wts[slot0 + out + pos] = w;
    }
    out += tot;
    unsigned long long wn = warp_sum<unsigned long long>((unsigned long long)w);
    if (lane == 0) atomicAdd(&s_n, wn);
    if (P.task == 0) {
      int k = (w > 0) ? __ldg(P.lab + r) : -1;
      for (int c = 0; c < P.C; ++c) {
        int s = warp_sum<int>(k == c ? w : 0);
        if (lane == 0 && s) atomicAdd(&s_cnt[c], s);
      }
    } else {
      long long s = warp_sum<long long>(w > 0 ? __ldg(P.q + r) * (long long)w : 0);
      if (lane == 0 && s) atomicAdd(&s_sum, (unsigned long long)s);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    LNode nd;
    nd.prob = pi;
    nd.tree = t;
    nd.idx = 0;
    nd.depth = 0;
    nd.tstart = gt;
    nd.fstart = P.tree0;
    nd.fend = P.tree0 + P.n_trees;
    nd.ecnt = out;
    nd.ebeg = slot0;
    nd.n = (int)s_n;
    nd.pad = 0;
    nd.sum = (long long)s_sum;
    nodes[gt] = nd;
    write_leaf(res, gt);
  }
  if (threadIdx.x < Cmax) cnt[(long long)gt * Cmax + threadIdx.x] = threadIdx.x < P.C ? s_cnt[threadIdx.x] : 0;
  if (threadIdx.x < 32) {
    bool want = threadIdx.x == 0 && !preleaf(P, (int)s_n, 0);
    enqueue(Q, queue_of(P, out, Q), gt, want);
    if (want) {
      atomicAdd((unsigned long long*)&stats[0], (unsigned long long)out);
      atomicAdd((unsigned long long*)&stats[1], s_n);
    }
  }
}

// ============================================================ level scans
// Exclusive scans over the level of (2 if split) and (1 if leaf): child and
// leaf positions.  pos arrays have n+1 entries (the last holds the totals).
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;

__global__ void __launch_bounds__(kScanBlock) k_scan_part(const NodeRes* res, int n, int2* part) {
  __shared__ int sm[kScanBlock / 32];
  long long base = (long long)blockIdx.x * kScanBlock * kScanItems;
  int c = 0, l = 0;
  for (int it = 0; it < kScanItems; ++it) {
    long long j = base + (long long)it * kScanBlock + threadIdx.x;
    if (j < n) {
      int s = res[j].split;
      c += 2 * s;
      l += 1 - s;
    }
  }
  int tc, tl;
  block_excl_scan<kScanBlock, int>(c, &tc, sm);
  block_excl_scan<kScanBlock, int>(l, &tl, sm);
  if (threadIdx.x == 0) part[blockIdx.x] = make_int2(tc, tl);
}

__global__ void __launch_bounds__(kScanBlock) k_scan_top(int2* part, int nparts, int* childpos,
                                                         int* leafpos, int n, int* summary) {
  __shared__ int sm[kScanBlock / 32];
  int carry_c = 0, carry_l = 0;
  for (int base = 0; base < nparts; base += kScanBlock) {
    int i = base + threadIdx.x;
    int2 v = i < nparts ? part[i] : make_int2(0, 0);
    int tc, tl;
    int ec = block_excl_scan<kScanBlock, int>(v.x, &tc, sm);
    int el = block_excl_scan<kScanBlock, int>(v.y, &tl, sm);
    if (i < nparts) part[i] = make_int2(carry_c + ec, carry_l + el);
    carry_c += tc;
    carry_l += tl;
  }
  if (threadIdx.x == 0) {
    childpos[n] = carry_c;
    leafpos[n] = carry_l;
    summary[0] = carry_c;
    summary[1] = carry_l;
  }
}

__global__ void __launch_bounds__(kScanBlock) k_scan_apply(const NodeRes* res, int n,
                                                           const int2* part, int* childpos,
                                                           int* leafpos) {
  __shared__ int sm[kScanBlock / 32];
  const long long base = (long long)blockIdx.x * kScanBlock * kScanItems;
  int2 off = part[blockIdx.x];
  for (int it = 0; it < kScanItems; ++it) {
    long long j = base + (long long)it * kScanBlock + threadIdx.x;
    int s = j < n ? res[j].split : 0;
    int c = j < n ? 2 * s : 0, l = j < n ? 1 - s : 0;
    int tc, tl;
    int ec = block_excl_scan<kScanBlock, int>(c, &tc, sm);
    int el = block_excl_scan<kScanBlock, int>(l, &tl, sm);
    if (j < n) {
      childpos[j] = off.x + ec;
      leafpos[j] = off.y + el;
    }
    off.x += tc;
    off.y += tl;
  }
}

// ============================================================ emission
struct EmitArgs {
  const ProbDesc* probs;
  const LNode* cur;
  const int* cnt;
  const NodeRes* res;
  const int* res_cnt;
  const int* childpos;
  const int* leafpos;
  int n;
  int Cmax;
  long long log_base;    // node log position of this level's first node
  long long plog_base;   // first leaf rank of this level in the probability log
  ClassifyNode* node_log;
  float* gain_log;       // per node: the chosen split's FP32 gain, NaN for leaves (or null)
  float* prob_log;       // Cmax floats per leaf rank
  const long long* fbase_cur;
  const long long* lbase_cur;
  long long* fbase_next;
  long long* lbase_next;
  Seg* seg;              // [n_forests] for this level
  LNode* next;
  int* next_cnt;
  NodeRes* next_res;
  Queues Q;
  long long* stats;      // [0] entries of searched nodes, [1] their weighted rows
};

__global__ void __launch_bounds__(256) k_emit(EmitArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = j < a.n;
  int qL = 0, qR = 0, cpL = 0, cpR = 0;
  bool wantL = false, wantR = false;
  unsigned long long my_e = 0, my_w = 0;
  if (act) {
    const LNode nd = a.cur[j];
    const NodeRes r = a.res[j];
    const ProbDesc& P = a.probs[nd.prob];
    const int f = nd.prob;
    const int fs = nd.fstart, fe = nd.fend;
    const long long fb = a.fbase_cur[f], lb = a.lbase_cur[f];
    ClassifyNode cn;
    if (r.split) {
      const int cp = a.childpos[j];
      const int cfs = a.childpos[fs];
      cn.child_start = (int)(fb + (fe - fs) + (cp - cfs));
      cn.child_count = 2;
      cn.probability_start = -1;
      cn.attribute = r.f;
      cn.split_point = r.thr;
      LNode L, R;
      L.prob = R.prob = nd.prob;
      L.tree = R.tree = nd.tree;
      L.idx = cp - a.childpos[nd.tstart];
      R.idx = L.idx + 1;
      L.depth = R.depth = nd.depth + 1;
      L.tstart = R.tstart = a.childpos[nd.tstart];
      L.fstart = R.fstart = cfs;
      L.fend = R.fend = a.childpos[fe];
      L.ebeg = nd.ebeg;
      L.ecnt = r.nl_e;
      R.ebeg = nd.ebeg + r.nl_e;
      R.ecnt = nd.ecnt - r.nl_e;
      L.n = r.nl;
      R.n = nd.n - r.nl;
      L.pad = R.pad = 0;
      L.sum = r.suml;
      R.sum = nd.sum - r.suml;
      a.next[cp] = L;
      a.next[cp + 1] = R;
      for (int c = 0; c < a.Cmax; ++c) {
        int lc = (P.task == 0 && c < P.C) ? a.res_cnt[(long long)j * a.Cmax + c] : 0;
        int tc = (P.task == 0 && c < P.C) ? a.cnt[(long long)j * a.Cmax + c] : 0;
        a.next_cnt[(long long)cp * a.Cmax + c] = lc;
        a.next_cnt[(long long)(cp + 1) * a.Cmax + c] = tc - lc;
      }
      write_leaf(a.next_res, cp);
      write_leaf(a.next_res, cp + 1);
      cpL = cp;
      cpR = cp + 1;
      wantL = !preleaf(P, L.n, L.depth);
      wantR = !preleaf(P, R.n, R.depth);
      qL = queue_of(P, L.ecnt, a.Q);
      qR = queue_of(P, R.ecnt, a.Q);
    } else {
      const long long lr = lb + (a.leafpos[j] - a.leafpos[fs]);
      cn.child_start = -1;
      cn.child_count = 0;
      cn.probability_start = (int)(lr * (long long)P.C);
      cn.attribute = -1;
      cn.split_point = -1.0f;
      float* dst = a.prob_log + (a.plog_base + a.leafpos[j]) * (long long)a.Cmax;
      if (P.task == 0) {
        for (int c = 0; c < P.C; ++c) dst[c] = (float)a.cnt[(long long)j * a.Cmax + c];
      } else {
        double v = ((double)nd.sum * pow2d(-P.S)) / (double)nd.n;
        dst[0] = __double2float_rn(v);
      }
    }
    a.node_log[a.log_base + j] = cn;
    if (a.gain_log) a.gain_log[a.log_base + j] = r.split ? r.gain : __int_as_float(0x7FC00000);
    if (j == fs) {
      a.fbase_next[f] = fb + (fe - fs);
      a.lbase_next[f] = lb + (a.leafpos[fe] - a.leafpos[fs]);
      Seg s;
      s.node_pos = a.log_base + fs;
      s.node_cnt = fe - fs;
      s.pad = 0;
      s.leaf_rank = a.plog_base + a.leafpos[fs];
      s.leaf_cnt = a.leafpos[fe] - a.leafpos[fs];
      a.seg[f] = s;
    }
  }
  if (wantL) {
    my_e += (unsigned long long)a.next[cpL].ecnt;
    my_w += (unsigned long long)a.next[cpL].n;
  }
  if (wantR) {
    my_e += (unsigned long long)a.next[cpR].ecnt;
    my_w += (unsigned long long)a.next[cpR].n;
  }
  my_e = warp_sum<unsigned long long>(my_e);
  my_w = warp_sum<unsigned long long>(my_w);
  if ((threadIdx.x & 31) == 0 && my_e) {
    atomicAdd((unsigned long long*)&a.stats[0], my_e);
    atomicAdd((unsigned long long*)&a.stats[1], my_w);
  }
  enqueue(a.Q, qL, cpL, wantL);
  enqueue(a.Q, qR, cpR, wantR);
}

// ============================================================ data prep
// Checks the frame (finite features, integral labels in [0, C)) and gathers
// max |y| for the regression fixed-point scale.  err bits: 1 = non-finite
// feature, 2 = bad label, 4 = non-finite target.
__device__ void validate_range(const float* X, long long nX, const float* y, long long N,
                               int task, int C, int* err, unsigned* maxabs) {
  long long stride = (long long)gridDim.x * blockDim.x;
  int e = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nX; i += stride) {
    float x = X[i];
    if (!isfinite(x)) e |= 1;
  }
  unsigned mx = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
    float v = y[i];
    if (task == 0) {
      if (!(v >= 0.0f && v < (float)C && v == truncf(v))) e |= 2;
    } else {
      if (!isfinite(v)) e |= 4;
      mx = max(mx, __float_as_uint(fabsf(v)));
    }
  }
  if (e) atomicOr(err, e);
  if (task == 1) atomicMax(maxabs, mx);
}
__global__ void k_validate(const float* X, long long nX, const float* y, long long N, int task,
                           int C, int* err, unsigned* maxabs) {
  validate_range(X, nX, y, N, task, C, err, maxabs);
}

__device__ void prep_range(const float* y, long long N, int task, int S, int* lab, long long* q) {
  long long stride = (long long)gridDim.x * blockDim.x;
  const double sc = pow2d(S);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
    if (task == 0)
      lab[i] = (int)y[i];
    else
      q[i] = __double2ll_rn((double)y[i] * sc);
  }
}
__global__ void k_prep_targets(const float* y, long long N, int task, int S, int* lab,
                               long long* q) {
  prep_range(y, N, task, S, lab, q);
}

// The same for every problem of a fit in one launch each: problem blockIdx.y.
struct PrepJob {
  const float* X;
  long long nX;
  const float* y;
  long long N;
  int task, C, S;
  int* lab;
  long long* q;
};
__global__ void k_validate_all(const PrepJob* jobs, int* err, unsigned* maxabs) {
  const PrepJob j = jobs[blockIdx.y];
  validate_range(j.X, j.nX, j.y, j.N, j.task, j.C, err, maxabs + blockIdx.y);
}
__global__ void k_prep_all(const PrepJob* jobs) {
  const PrepJob j = jobs[blockIdx.y];
  prep_range(j.y, j.N, j.task, j.S, j.lab, j.q);
}

// One launch for every (level, forest) segment of a batch: nodes from the
// node log into the forest's array, leaf payloads from the strided
// probability log into the forest's packed array.
struct GatherSeg {
  long long node_pos, leaf_rank, leaf_cnt;
  ClassifyNode* node_dst;
  float* gain_dst;
  float* prob_dst;
  int node_cnt, C;
};

__global__ void k_gather_segments(const GatherSeg* segs, const ClassifyNode* log,
                                  const float* glog, const float* plog, int Cmax) {
  const GatherSeg g = segs[blockIdx.x];
  for (int i = threadIdx.x; i < g.node_cnt; i += blockDim.x) {
    g.node_dst[i] = log[g.node_pos + i];
    g.gain_dst[i] = glog[g.node_pos + i];
  }
  const long long tot = g.leaf_cnt * g.C;
  for (long long i = threadIdx.x; i < tot; i += blockDim.x) {
    const long long l = i / g.C;
    const int c = (int)(i % g.C);
    g.prob_dst[i] = plog[(g.leaf_rank + l) * Cmax + c];
  }
}

// Probabilities from the strided log into a forest's packed array, and the
// nodes of each (level, forest) segment into the forest's node array.
__global__ void k_gather_nodes(const ClassifyNode* log, long long pos, int cnt, ClassifyNode* dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    dst[i] = log[pos + i];
}
__global__ void k_gather_probs(const float* plog, long long rank0, long long cnt, int Cmax, int C,
                               float* dst) {
  long long total = cnt * C;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long l = i / C;
    int c = (int)(i % C);
    dst[i] = plog[(rank0 + l) * Cmax + c];
  }
}

// Predict layout from the Classify layout: the voted class of each leaf
// (first class with the strictly largest count, gpudte.cu:340-352) is
// precomputed; regression leaves carry their value.
__global__ void k_to_pnodes(const ClassifyNode* nodes, long long n, const float* probs, int C,
                            int task, PNode* out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    ClassifyNode cn = nodes[i];
    PNode p;
    p.pad = 0;
    if (cn.child_count > 0) {
      p.a = cn.child_start;
      p.b = cn.attribute;
      p.t = cn.split_point;
    } else {
      const float* pr = probs + cn.probability_start;
      p.a = -1;
      if (task == 0) {
        int sel = 0;
        float mx = 0.0f;
        for (int c = 0; c < C; ++c)
          if (pr[c] > mx) {
            mx = pr[c];
            sel = c;
          }
        p.b = sel;
        p.t = 0.0f;
      } else {
        p.b = 0;
        p.t = pr[0];
      }
    }
    out[i] = p;
  }
}

// The largest bootstrap multiplicity of the fit, for the big-node items'
// packed sort keys (rank, label and weight in one word).
__global__ void k_max_weight(const int* __restrict__ w, long long n, int* out) {
  int mx = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    mx = max(mx, w[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
  if ((threadIdx.x & 31) == 0 && mx > 0) atomicMax(out, mx);
}

// Compact predict layout (PNode8) from the 16-byte one; *bad is set when a
// child offset does not fit the bits above the feature field.
__global__ void k_to_pnodes8(const PNode* in, long long n, int fbits, PNode8* out, int* bad) {
  const uint32_t marker = (1u << fbits) - 1u;
  const long long lim = 1ll << (32 - fbits);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const PNode p = in[i];
    PNode8 q;
    q.t = p.t;
    if (p.a >= 0) {
      const long long off = (long long)p.a - i;
      if (off <= 0 || off >= lim) {
        atomicExch(bad, 1);
        q.w = 0;
      } else {
        q.w = ((uint32_t)off << fbits) | (uint32_t)p.b;
      }
    } else {
      q.w = ((uint32_t)p.b << fbits) | marker;
    }
    out[i] = q;
  }
}

#endif  // DML_SEARCH_CW

}  // namespace dml
