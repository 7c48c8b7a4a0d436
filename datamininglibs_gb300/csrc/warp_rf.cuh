// RF split search for nodes of 33 .. 32*E entries, one warp per node.
//
// The node's (key, entry) pairs are held striped in registers (element
// r*32 + lane in register r), sorted by a bitonic network (register
// compare-exchanges for distances >= 32, shuffles below) and written to shared
// memory.  Classification scans the sorted positions one round of 32 at a
// time: each entry's class weight below it (earlier rounds from a per-warp
// class histogram, its round from a match instruction and the weights' bit
// planes) gives the change its move to the left side makes to the entropy
// sum, and one warp scan of those changes gives every boundary's exact gain
// numerator.  Regression scans E consecutive positions per lane after one
// warp scan of counts and target sums.  No block barriers; a node per warp,
// eight warps a block (two for 512-entry nodes).  Same candidate rules as the CTA kernels
// (lib_ensembles/source/gpurf.cu:131-259, 618-917 restated).
#pragma once
#include "fit_kernels.cuh"

namespace dml {

template <int E, class T>
__device__ __forceinline__ void warp_bitonic_sort(T (&key)[E]) {
  const int lane = threadIdx.x & 31;
  constexpr int M = 32 * E;
#pragma unroll
  for (int k = 2; k <= M; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const int rj = j >> 5;
#pragma unroll
        for (int r = 0; r < E; ++r) {
          const int p = r ^ rj;
          if (p > r) {
            const int i = r * 32 + lane;
            const bool up = (i & k) == 0;
            T a = key[r], b = key[p];
            bool swap = up ? (a > b) : (a < b);
            key[r] = swap ? b : a;
            key[p] = swap ? a : b;
          }
        }
      } else {
#pragma unroll
        for (int r = 0; r < E; ++r) {
          const int i = r * 32 + lane;
          const bool up = (i & k) == 0;
          const bool lower = (lane & j) == 0;
          T o = __shfl_xor_sync(kFull, key[r], j);
          T mine = key[r];
          // the lower element keeps the min of an ascending pair
          bool take_min = (lower == up);
          T mn = mine < o ? mine : o, mx = mine < o ? o : mine;
          key[r] = take_min ? mn : mx;
        }
      }
    }
  }
}

template <int CW>
__device__ __forceinline__ long long packed_get(const unsigned long long (&L)[CW], int c) {
  unsigned long long x = L[0];
#pragma unroll
  for (int j = 1; j < CW; ++j)
    if ((c >> 1) == j) x = L[j];
  return (long long)((c & 1) ? (x >> 32) : (x & 0xFFFFFFFFull));
}

// Nt[c] for a class index known only at run time (a select chain over the
// registers instead of a local-memory array).
template <int CW>
__device__ __forceinline__ int Nt_of(const int (&Nt)[2 * CW], int c) {
  int x = Nt[0];
#pragma unroll
  for (int j = 1; j < 2 * CW; ++j)
    if (c == j) x = Nt[j];
  return x;
}

// Warps per block: 8, or 2 for 512-entry nodes (static shared memory per warp).
template <int E>
constexpr int warp_rf_wpb() {
  return E >= 16 ? 2 : 8;
}

// Resident blocks per SM the registers are sized for, by measurement on the
// 1M x 128 fit (class times at 16 / 24 / 32 warps per SM): E = 2 at 32 warps
// (64 registers; 61.4 / 47.7 / 43.8 ms), E = 4 at 24 (85; 45.4 / 38.6 /
// 38.7), E = 8 at 24 (85; 38.2 / 37.6 / 60.1), E = 16 at 16 (128; 58.1 /
// 76.3 / 82.3).  More warps hide the shuffle latency of the sorts and scans
// until the spills of the larger register sets cost more than they hide.
// Eight or more packed class words keep 16 warps (128 registers): their class
// counts alone take 16 or 32 registers.
template <int E, int CW>
constexpr int warp_rf_min_blocks() {
  return (CW >= 8 ? 16 : E == 2 ? 32 : E == 16 ? 16 : 24) / warp_rf_wpb<E>();
}

struct RegScan {
  float g;    // the lane's best gain, -FLT_MAX if none
  int p;      // its sorted position, -1 if none
  long long nl, sl;  // left weight and weighted target sum there
};

// Regression boundary scan of one sorted try of a warp kernel: lane l owns
// sorted positions p0 = l*E .. p0+E-1, its keys at sk[0 .. E-1] (key, entry
// index) and prevk the key before them; sw / sqw: the entries' weights and
// fixed-point targets.  One warp scan of the lanes' weights and target sums,
// then each lane walks its positions.  The float-float gain is evaluated only
// where variance_gain_bounds' upper bound reaches the largest lower bound over
// the warp: a boundary below it can neither be nor tie the warp's best.
// n, sum: the node's weight and weighted target sum; S: the target scale.
template <int E>
static __device__ __forceinline__ RegScan warp_reg_scan(const unsigned long long* sk,
                                                        uint32_t prevk, int p0, const int* sw,
                                                        const long long* sqw, long long n,
                                                        long long sum, int ml, int S) {
  const float rc = __frcp_rn(__ll2float_rn(n));
  const float p2 = pow2f(-2 * S);
  long long tn = 0, ts = 0;
  unsigned bnd = 0;  // bit j: position p0 + j starts a new key
#pragma unroll 1
  for (int j = 0; j < E; ++j) {
    const unsigned long long kv = sk[j];
    if (kv == ~0ull) break;
    const int e = (int)(kv & 0xFFFFFFFFull);
    const uint32_t kk = (uint32_t)(kv >> 32);
    if (p0 + j > 0 && prevk < kk) bnd |= 1u << j;
    prevk = kk;
    const int w = sw[e];
    tn += w;
    ts += sqw[e] * (long long)w;
  }
  const long long nl0 = warp_excl_scan<long long>(tn);
  const long long sl0 = warp_excl_scan<long long>(ts);
  float t = -FLT_MAX;
  {
    long long nl = nl0, sl = sl0;
#pragma unroll 1
    for (int j = 0; j < E && bnd >> j; ++j) {
      const int e = (int)(sk[j] & 0xFFFFFFFFull);
      const int w = sw[e];
      const long long nr = n - nl;
      if (((bnd >> j) & 1u) && nl >= ml && nr >= ml) {
        float lo, hi;
        variance_gain_bounds((int)nl, sl, (int)nr, sum - sl, rc, p2, lo, hi);
        t = fmaxf(t, lo);
      }
      sl += sqw[e] * (long long)w;
      nl += w;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(kFull, t, o));
  RegScan r{-FLT_MAX, -1, 0, 0};
  long long nl = nl0, sl = sl0;
#pragma unroll 1
  for (int j = 0; j < E && bnd >> j; ++j) {
    const int e = (int)(sk[j] & 0xFFFFFFFFull);
    const int w = sw[e];
    const long long nr = n - nl;
    if (((bnd >> j) & 1u) && nl >= ml && nr >= ml) {
      float lo, hi;
      variance_gain_bounds((int)nl, sl, (int)nr, sum - sl, rc, p2, lo, hi);
      if (hi >= t) {
        const float g = variance_gain(nl, sl, nr, sum - sl, S);
        if (r.p < 0 || g > r.g) {
          r.g = g;
          r.p = p0 + j;
          r.nl = nl;
          r.sl = sl;
        }
      }
    }
    sl += sqw[e] * (long long)w;
    nl += w;
  }
  return r;
}

template <int E, int CW>
__global__ void __launch_bounds__(32 * warp_rf_wpb<E>(), warp_rf_min_blocks<E, CW>())
    k_warp_rf(LevelArgs a) {
  constexpr int M = 32 * E;
  constexpr int WPB = warp_rf_wpb<E>();
  __shared__ int s_row[WPB][M];
  __shared__ int s_w[WPB][M];
  // labels (classification) or fixed-point targets (regression) of the entries
  __shared__ long long s_lq[WPB][M];
  int* const s_lab_w = reinterpret_cast<int*>(s_lq[threadIdx.x >> 5]);
  const long long* const s_q_w = s_lq[threadIdx.x >> 5];
  // sorted (key, entry) of the current try; sorted position p at p + p / E, so
  // that lane l's E consecutive positions are read without bank conflicts
  __shared__ unsigned long long s_key[WPB][M + 32];
  __shared__ int s_hist[WPB][kMaxClasses];  // round scan: class weights of earlier rounds
  const int lane = threadIdx.x & 31;
  const int wb = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int wi = gw; wi < a.nwork; wi += nwarps) {
    const int node = a.work[wi];
    const LNode nd = a.nodes[node];
    const ProbDesc& P = a.probs[nd.prob];
    const int C = P.C;
    const int m = nd.ecnt;
    const int* ncnt = a.cnt + (long long)node * a.Cmax;
    const int ml = max(1, P.min_leaf);
    // sort keys: rank << kIdxBits | entry when ranks and entries fit 31 bits
    constexpr int kIdxBits = E == 2 ? 6 : E == 4 ? 7 : E == 8 ? 8 : 9;
    static_assert((1 << kIdxBits) == M, "entry index bits");
    const bool r32 = P.rank != nullptr && (32 - __clz((int)max(1ll, P.N - 1))) + kIdxBits <= 31;
    int rowr[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int i = r * 32 + lane;
      rowr[r] = 0;
      if (i < m) {
        const int row = __ldg(a.rowsA + nd.ebeg + i);
        rowr[r] = row;
        s_row[wb][i] = row;
        s_w[wb][i] = a.wA ? __ldg(a.wA + nd.ebeg + i) : 1;
        if (P.task == 0)
          s_lab_w[i] = __ldg(P.lab + row);
        else
          s_lq[wb][i] = __ldg(P.q + row);
      }
    }
    __syncwarp();
    int Nt[2 * CW];
#pragma unroll
    for (int c = 0; c < 2 * CW; ++c) Nt[c] = (P.task == 0 && c < C) ? ncnt[c] : 0;
    const long long Hn = P.task == 0 ? __ldg(a.H + nd.n) : 0;
    int wbits;  // bit planes of the node's largest weight
    {
      int wm = 1;
#pragma unroll
      for (int r = 0; r < E; ++r)
        if (r * 32 + lane < m) wm = max(wm, s_w[wb][r * 32 + lane]);
      for (int o = 16; o > 0; o >>= 1) wm = max(wm, __shfl_xor_sync(kFull, wm, o));
      wbits = 32 - __clz(wm);
    }
    Cand best;
    best.valid = 0;
    // the features of tries 0 .. 31, one per lane
    const int fpre = lane < P.n_mand + P.n_opt ? feature_of_try(P, nd, lane) : 0;
    int t = 0;
    for (;; ++t) {
      const int f = t < 32 ? __shfl_sync(kFull, fpre, t) : feature_of_try(P, nd, t);
      const float* xf = P.X + (long long)f * P.N;
      if (r32) {
        // value ranks and entry indices packed in 32 bits: half the shuffles
        const uint32_t* rk = P.rank + (long long)f * P.N;
        uint32_t key[E];
#pragma unroll
        for (int r = 0; r < E; ++r) {
          const int i = r * 32 + lane;
          key[r] = i < m ? (__ldg(rk + rowr[r]) << kIdxBits) | (uint32_t)i : ~0u;
        }
        warp_bitonic_sort<E>(key);
#pragma unroll
        for (int r = 0; r < E; ++r)
          s_key[wb][r * 32 + lane + (r * 32 + lane) / E] =
              key[r] == ~0u ? ~0ull
                            : ((unsigned long long)(key[r] >> kIdxBits) << 32) |
                                  (key[r] & (uint32_t)(M - 1));
      } else {
        unsigned long long key[E];
#pragma unroll
        for (int r = 0; r < E; ++r) {
          const int i = r * 32 + lane;
          key[r] = i < m ? (((unsigned long long)orderable(__ldg(xf + rowr[r])) << 32) | (unsigned)i)
                         : ~0ull;
        }
        warp_bitonic_sort<E>(key);
#pragma unroll
        for (int r = 0; r < E; ++r) s_key[wb][r * 32 + lane + (r * 32 + lane) / E] = key[r];
      }
      __syncwarp();
      long long my_nl = 0, my_sl = 0;
      float bg = -FLT_MAX;
      int bp = -1;
      if (P.task == 0) {
        // classification, by rounds: sorted positions r*32 + lane,
        // one round at a time.  The gain numerator is h(n) - h(nL) - h(nR)
        // plus the scan of each entry's own-class change: its class weight
        // below it is that of the earlier rounds (s_hist) plus that of the
        // lanes below it in its round matching its class (match, bit planes)
        for (int c = lane; c < C; c += 32) s_hist[wb][c] = 0;
        __syncwarp();
        NumBest nb;
        nb.init();
        long long carry_n = 0, carry_s = 0;
        uint32_t lastk = 0;
#pragma unroll 1
        for (int r = 0; r < E; ++r) {
          const int pos = r * 32 + lane;
          const unsigned long long kv = s_key[wb][pos + pos / E];
          const bool ok = kv != ~0ull;
          const int e = (int)(kv & 0xFFFFFFFFull);
          const uint32_t kk = (uint32_t)(kv >> 32);
          const int w = ok ? s_w[wb][e] : 0;
          const int c = ok ? s_lab_w[e] : -1;
          const unsigned peers = __match_any_sync(kFull, c);
          int lw = 0, gw_c = 0;
          for (int b = 0; b < wbits; ++b) {
            const unsigned bb = __ballot_sync(kFull, (w >> b) & 1);
            lw += __popc(bb & peers & lt) << b;
            gw_c += __popc(bb & peers) << b;
          }
          long long dq = 0;
          if (ok) {
            const int L = s_hist[wb][c] + lw;
            const int R = Nt_of<CW>(Nt, c) - L;
            dq = (__ldg(a.H + L + w) - __ldg(a.H + L)) + (__ldg(a.H + R - w) - __ldg(a.H + R));
          }
          const long long xn = warp_excl_scan<long long>(w);
          const long long xs = warp_excl_scan<long long>(dq);
          const long long nl = carry_n + xn, S = carry_s + xs;
          uint32_t prevk = __shfl_up_sync(kFull, kk, 1);
          if (lane == 0) prevk = lastk;
          const long long nr = (long long)nd.n - nl;
          if (ok && pos > 0 && prevk < kk && nl >= ml && nr >= ml &&
              nb.offer(Hn - __ldg(a.H + nl) - __ldg(a.H + nr) + S, pos, nd.n))
            my_nl = nl;
          carry_n += __shfl_sync(kFull, xn + w, 31);
          carry_s += __shfl_sync(kFull, xs + dq, 31);
          lastk = __shfl_sync(kFull, kk, 31);
          __syncwarp();
          if (ok && (peers & lt) == 0) s_hist[wb][c] += gw_c;  // one lane per class
          __syncwarp();
        }
        bg = nb.gain(nd.n);
        bp = nb.p;
      } else {
        // regression: lane l owns sorted positions l*E .. l*E+E-1
        const int p0 = lane * E;
        const RegScan rs = warp_reg_scan<E>(
            &s_key[wb][p0 + lane], p0 > 0 ? (uint32_t)(s_key[wb][p0 - 1 + (p0 - 1) / E] >> 32) : 0u,
            p0, s_w[wb], s_q_w, nd.n, nd.sum, ml, P.S);
        bg = rs.g;
        bp = rs.p;
        my_nl = rs.nl;
        my_sl = rs.sl;
      }
      // warp argmax: higher gain, then lower position
      float wg = bg;
      int wp = bp;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        float g2 = __shfl_xor_sync(kFull, wg, o);
        int p2 = __shfl_xor_sync(kFull, wp, o);
        bool take = p2 >= 0 && (wp < 0 || g2 > wg || (g2 == wg && p2 < wp));
        if (take) {
          wg = g2;
          wp = p2;
        }
      }
      Cand cd;
      cd.f = f;
      if (wp >= 0) {
        const int src = __ffs(__ballot_sync(kFull, bp == wp)) - 1;
        cd.valid = 1;
        cd.gain = wg;
        // entries at sorted positions wp-1 and wp
        const unsigned long long ka = s_key[wb][wp - 1 + (wp - 1) / E],
                                 kb = s_key[wb][wp + wp / E];
        const float xa = __ldg(xf + s_row[wb][(int)(ka & 0xFFFFFFFFull)]);
        const float xb = __ldg(xf + s_row[wb][(int)(kb & 0xFFFFFFFFull)]);
        cd.thr = midpoint_threshold(xa, xb);
        cd.nl_e = wp;
        cd.nl = (int)__shfl_sync(kFull, my_nl, src);
        cd.suml = __shfl_sync(kFull, my_sl, src);
      } else {
        cd.valid = 0;
        cd.gain = -FLT_MAX;
        cd.thr = 0.0f;
        cd.nl_e = cd.nl = 0;
        cd.suml = 0;
      }
      bool more;
      if (t < P.n_mand) {
        if (t == 0 || better(cd, best)) best = cd;
        more = (t + 1 < P.n_mand) || (P.n_opt > 0 && !(best.valid && best.gain >= kSensible));
      } else {
        if (better(cd, best)) best = cd;
        more = !(cd.valid && cd.gain >= kSensible) && (t + 1 < P.n_mand + P.n_opt);
      }
      __syncwarp();
      if (!more) break;
    }
    if (lane == 0) {
      atomicAdd((unsigned long long*)&a.stats[2], (unsigned long long)(t + 1) * m);
      atomicAdd((unsigned long long*)&a.stats[3], (unsigned long long)m);
    }
    if (!best.valid) {
      if (lane == 0) write_leaf(a.res, node);
      __syncwarp();
      continue;
    }
    if (lane == 0) write_result(a.res, a.res_cnt, a.Cmax, node, best, nullptr, 0);
    // stable partition, 32 entries per round; the left class counts of the
    // split (packed two per word) from the entries that go left
    const float* xb = P.X + (long long)best.f * P.N;
    int offl = 0, offr = 0;
    unsigned long long lcnt[CW];
#pragma unroll
    for (int c = 0; c < CW; ++c) lcnt[c] = 0;
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int i = r * 32 + lane;
      const bool valid = i < m;
      const bool left = valid && goes_left(__ldg(xb + rowr[r]), best.thr);
      if (P.task == 0 && left) {
        const int k = s_lab_w[i];
        const unsigned long long w = (unsigned long long)s_w[wb][i];
#pragma unroll
        for (int c = 0; c < CW; ++c)
          lcnt[c] += (k == 2 * c ? w : 0ull) | (k == 2 * c + 1 ? (w << 32) : 0ull);
      }
      const unsigned lm = __ballot_sync(kFull, left);
      const unsigned vm = __ballot_sync(kFull, valid);
      if (valid) {
        const int pl = __popc(lm & lt);
        const long long dst =
            nd.ebeg + (left ? offl + pl : best.nl_e + offr + (__popc(vm & lt) - pl));
        a.rowsB[dst] = rowr[r];
        if (a.wB) a.wB[dst] = s_w[wb][i];
      }
      offl += __popc(lm);
      offr += __popc(vm) - __popc(lm);
    }
    if (P.task == 0) {
#pragma unroll
      for (int c = 0; c < CW; ++c) lcnt[c] = warp_sum<unsigned long long>(lcnt[c]);
      if (lane < C) a.res_cnt[(long long)node * a.Cmax + lane] = (int)packed_get<CW>(lcnt, lane);
    }
    __syncwarp();
  }
}

}  // namespace dml
