// RF split search for nodes of 33 .. 32*E entries, one warp per node.
//
// The node's (key, entry) pairs are held striped in registers (element
// r*32 + lane in register r), sorted by a bitonic network (register
// compare-exchanges for distances >= 32, shuffles below), then scanned 32
// consecutive elements at a time with warp scans of the packed class counts
// (two 32-bit counts per 64-bit word) or of the regression count / sum.  No
// block barriers; eight nodes per 256-thread block.  Same candidate rules as
// the CTA kernels (lib_ensembles/source/gpurf.cu:131-259, 618-917 restated).
#pragma once
#include "fit_kernels.cuh"

namespace dml {

template <int E>
__device__ __forceinline__ void warp_bitonic_sort(unsigned long long (&key)[E]) {
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
            unsigned long long a = key[r], b = key[p];
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
          unsigned long long o = __shfl_xor_sync(kFull, key[r], j);
          unsigned long long mine = key[r];
          // the lower element keeps the min of an ascending pair
          bool take_min = (lower == up);
          unsigned long long mn = mine < o ? mine : o, mx = mine < o ? o : mine;
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

// Warps per block: 8, or 4 for 512-entry nodes (shared memory per warp).
template <int E>
constexpr int warp_rf_wpb() {
  return E >= 16 ? 4 : 8;
}

template <int E, int CW>
__global__ void __launch_bounds__(32 * warp_rf_wpb<E>(), 2) k_warp_rf(LevelArgs a) {
  constexpr int M = 32 * E;
  constexpr int WPB = warp_rf_wpb<E>();
  __shared__ int s_row[WPB][M];
  __shared__ int s_w[WPB][M];
  __shared__ int s_lab[WPB][M];
  __shared__ long long s_q[WPB][M];
  __shared__ unsigned long long s_key[WPB][M];  // sorted (key, entry) of the current try
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
          s_lab[wb][i] = __ldg(P.lab + row);
        else
          s_q[wb][i] = __ldg(P.q + row);
      }
    }
    __syncwarp();
    long long prior = 0;
    int Nt[2 * CW];
#pragma unroll
    for (int c = 0; c < 2 * CW; ++c) Nt[c] = (P.task == 0 && c < C) ? ncnt[c] : 0;
    if (P.task == 0) prior = entropy_prior(a.H, nd.n, C, [&](int c) { return (long long)ncnt[c]; });
    Cand best;
    best.valid = 0;
    unsigned long long bestL[CW];
#pragma unroll
    for (int j = 0; j < CW; ++j) bestL[j] = 0;
    int t = 0;
    for (;; ++t) {
      const int f = feature_of_try(P, nd, t);
      const float* xf = P.X + (long long)f * P.N;
      unsigned long long key[E];
#pragma unroll
      for (int r = 0; r < E; ++r) {
        const int i = r * 32 + lane;
        key[r] = i < m ? (((unsigned long long)orderable(__ldg(xf + rowr[r])) << 32) | (unsigned)i)
                       : ~0ull;
      }
      warp_bitonic_sort<E>(key);
#pragma unroll
      for (int r = 0; r < E; ++r) s_key[wb][r * 32 + lane] = key[r];
      __syncwarp();
      // boundary scan, 32 sorted elements per round (a rolled loop: the
      // per-round class scans and gains are the bulk of the kernel's code)
      unsigned long long carryL[CW], L[CW], myL[CW];
#pragma unroll
      for (int j = 0; j < CW; ++j) {
        carryL[j] = 0;
        myL[j] = 0;
      }
      long long carry_n = 0, carry_s = 0, my_nl = 0, my_sl = 0;
      uint32_t lastk = 0;
      float bg = -FLT_MAX;
      int bp = -1;
#pragma unroll 1
      for (int r = 0; r < E; ++r) {
        const unsigned long long kv = s_key[wb][r * 32 + lane];
        const bool ok = kv != ~0ull;
        const int e = (int)(kv & 0xFFFFFFFFull);
        const uint32_t kk = (uint32_t)(kv >> 32);
        const int pos = r * 32 + lane;
        const int w = ok ? s_w[wb][e] : 0;
        long long nl, sl = 0;
        {
          long long ex = warp_excl_scan<long long>(w);
          nl = carry_n + ex;
          carry_n += __shfl_sync(kFull, ex + w, 31);
        }
        if (P.task == 0) {
          const int k = ok ? s_lab[wb][e] : -1;
#pragma unroll
          for (int j = 0; j < CW; ++j) {
            unsigned long long v = (k == 2 * j ? (unsigned long long)w : 0ull) |
                                   (k == 2 * j + 1 ? ((unsigned long long)w << 32) : 0ull);
            unsigned long long ex = warp_excl_scan<unsigned long long>(v);
            L[j] = carryL[j] + ex;
            carryL[j] += __shfl_sync(kFull, ex + v, 31);
          }
        } else {
          const long long qw = ok ? s_q[wb][e] * (long long)w : 0;
          long long ex = warp_excl_scan<long long>(qw);
          sl = carry_s + ex;
          carry_s += __shfl_sync(kFull, ex + qw, 31);
        }
        uint32_t prevk = __shfl_up_sync(kFull, kk, 1);
        if (lane == 0) prevk = lastk;
        lastk = __shfl_sync(kFull, kk, 31);
        const long long nr = (long long)nd.n - nl;
        const bool bnd = ok && pos > 0 && prevk < kk && nl >= ml && nr >= ml;
        if (bnd) {
          float g;
          if (P.task == 0)
            g = entropy_gain_u<2 * CW>(
                a.H, prior, C, nl, nr,
                [&](int c) {
                  return (long long)((c & 1) ? (L[c >> 1] >> 32) : (L[c >> 1] & 0xFFFFFFFFull));
                },
                [&](int c) { return (long long)Nt[c]; });
          else
            g = variance_gain(nl, sl, nr, nd.sum - sl, P.S);
          if (bp < 0 || g > bg) {
            bg = g;
            bp = pos;
            my_nl = nl;
            my_sl = sl;
#pragma unroll
            for (int j = 0; j < CW; ++j) myL[j] = L[j];
          }
        }
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
      unsigned long long candL[CW];
      if (wp >= 0) {
        const int src = __ffs(__ballot_sync(kFull, bp == wp)) - 1;
        cd.valid = 1;
        cd.gain = wg;
        // entries at sorted positions wp-1 and wp
        const unsigned long long ka = s_key[wb][wp - 1], kb = s_key[wb][wp];
        const float xa = __ldg(xf + s_row[wb][(int)(ka & 0xFFFFFFFFull)]);
        const float xb = __ldg(xf + s_row[wb][(int)(kb & 0xFFFFFFFFull)]);
        cd.thr = midpoint_threshold(xa, xb);
        cd.nl_e = wp;
        cd.nl = (int)__shfl_sync(kFull, my_nl, src);
        cd.suml = __shfl_sync(kFull, my_sl, src);
#pragma unroll
        for (int j = 0; j < CW; ++j) candL[j] = __shfl_sync(kFull, myL[j], src);
      } else {
        cd.valid = 0;
        cd.gain = -FLT_MAX;
        cd.thr = 0.0f;
        cd.nl_e = cd.nl = 0;
        cd.suml = 0;
#pragma unroll
        for (int j = 0; j < CW; ++j) candL[j] = 0;
      }
      bool more;
      bool take;
      if (t < P.n_mand) {
        take = (t == 0 || better(cd, best));
        if (take) best = cd;
        more = (t + 1 < P.n_mand) || (P.n_opt > 0 && !(best.valid && best.gain >= kSensible));
      } else {
        take = better(cd, best);
        if (take) best = cd;
        more = !(cd.valid && cd.gain >= kSensible) && (t + 1 < P.n_mand + P.n_opt);
      }
      if (take) {
#pragma unroll
        for (int j = 0; j < CW; ++j) bestL[j] = candL[j];
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
    if (P.task == 0 && lane < C) a.res_cnt[(long long)node * a.Cmax + lane] = (int)packed_get<CW>(bestL, lane);
    // stable partition, 32 entries per round
    const float* xb = P.X + (long long)best.f * P.N;
    int offl = 0, offr = 0;
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int i = r * 32 + lane;
      const bool valid = i < m;
      const bool left = valid && goes_left(__ldg(xb + rowr[r]), best.thr);
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
    __syncwarp();
  }
}

}  // namespace dml
