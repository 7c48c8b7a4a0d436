// ERT split search for nodes of 33 .. 32*E entries, one warp per node.
//
// The same tries as the CTA kernel (k_ert_cta; gpuert.cu:119-247, 275-381
// restated): try t draws a feature and a threshold, the mean of 10 node values
// summed in draw order.  Lane t computes try t's feature and threshold for all
// tries of the node at once (tries below 32).  Each try is one pass over the
// node's entries, E per lane: a ballot of the entries that go left per round,
// and lane c counts its class among them with the round's class mask (taken
// once per node), so the entropy needs one warp sum of the lanes' class terms.
// Counts are of entries, as in the CTA kernel.  Then the stable partition.
#pragma once
#include "fit_kernels.cuh"
#include "warp_rf.cuh"

namespace dml {

// Three resident blocks per SM (24 warps, 85 registers, some spilled): on the
// 256 uneven forests the class took 15.0 ms at two blocks, 11.8 at three and
// 11.9 at four.
template <int E>
__global__ void __launch_bounds__(256, 3) k_ert_warp(LevelArgs a) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int wi = gw; wi < a.nwork; wi += nwarps) {
    const int node = a.work[wi];
    const LNode nd = a.nodes[node];
    const ProbDesc& P = a.probs[nd.prob];
    const int C = P.C;
    const int m = nd.ecnt;
    const int* rows = a.rowsA + nd.ebeg;
    const int* ncnt = a.cnt + (long long)node * a.Cmax;
    const int ml = max(1, P.min_leaf);
    // row ids; for classification lane c keeps, per round, the mask of the
    // lanes whose entry is of class c (C <= 32)
    int rowr[E];
    unsigned cmr[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int i = r * 32 + lane;
      rowr[r] = i < m ? __ldg(rows + i) : 0;
      cmr[r] = 0;
      if (P.task == 0) {
        const int k = i < m ? __ldg(P.lab + rowr[r]) : -1;
        for (int c = 0; c < C; ++c) {
          const unsigned mc = __ballot_sync(kFull, k == c);
          if (lane == c) cmr[r] = mc;
        }
      }
    }
    const long long Nc = (P.task == 0 && lane < C) ? __ldg(ncnt + lane) : 0;
    const long long Hn = P.task == 0 ? __ldg(a.H + nd.n) : 0;
    // prior numerator h(n) - sum_c h(N_c)
    const long long prior =
        P.task == 0 ? Hn - warp_sum<long long>(lane < C ? __ldg(a.H + Nc) : 0) : 0;
    // features and thresholds of tries 0 .. 31, lane t computing try t
    const int ntry = P.n_mand + P.n_opt;
    int f_l = 0;
    float thr_l = 0.0f;
    if (lane < ntry) {
      f_l = feature_of_try(P, nd, lane);
      thr_l = ert_threshold(P, nd, lane, f_l, rows);
    }
    Cand best;
    best.valid = 0;
    int t = 0;
    for (;; ++t) {
      int f;
      float thr;
      if (t < 32) {
        f = __shfl_sync(kFull, f_l, t);
        thr = __shfl_sync(kFull, thr_l, t);
      } else {
        f = feature_of_try(P, nd, t);
        thr = ert_threshold(P, nd, t, f, rows);
      }
      const float* xf = P.X + (long long)f * P.N;
      int nl = 0, lc = 0;
      long long sl_l = 0;
#pragma unroll
      for (int r = 0; r < E; ++r) {
        const int i = r * 32 + lane;
        const bool left = i < m && goes_left(__ldg(xf + rowr[r]), thr);
        const unsigned lm = __ballot_sync(kFull, left);
        nl += __popc(lm);
        lc += __popc(lm & cmr[r]);
        if (P.task != 0 && left) sl_l += __ldg(P.q + rowr[r]);
      }
      const long long nr = (long long)nd.n - nl;
      Cand cd;
      cd.f = f;
      cd.thr = thr;
      cd.nl_e = nl;
      cd.nl = nl;
      cd.valid = nl >= ml && nr >= ml;
      if (P.task == 0) {
        // Q = h(nL) + h(nR) - sum_c (h(L_c) + h(N_c - L_c)), lane c's term summed
        const long long term = lane < C ? __ldg(a.H + lc) + __ldg(a.H + (Nc - lc)) : 0;
        const long long Q = __ldg(a.H + nl) + __ldg(a.H + nr) - warp_sum<long long>(term);
        cd.suml = 0;
        cd.gain = cd.valid ? gain_from_numerator(prior - Q, nd.n) : -FLT_MAX;
      } else {
        const long long sl = warp_sum<long long>(sl_l);
        cd.suml = sl;
        cd.gain = cd.valid ? variance_gain(nl, sl, nr, nd.sum - sl, P.S) : -FLT_MAX;
      }
      bool more;
      if (t < P.n_mand) {
        if (t == 0 || better(cd, best)) best = cd;
        more = (t + 1 < P.n_mand) || (P.n_opt > 0 && !(best.valid && best.gain >= kSensible));
      } else {
        if (better(cd, best)) best = cd;
        more = !(cd.valid && cd.gain >= kSensible) && (t + 1 < ntry);
      }
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
    // stable partition, 32 entries per round; lane c counts its class among
    // the entries that go left
    const float* xb = P.X + (long long)best.f * P.N;
    int offl = 0, offr = 0, lcnt = 0;
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int i = r * 32 + lane;
      const bool valid = i < m;
      const bool left = valid && goes_left(__ldg(xb + rowr[r]), best.thr);
      const unsigned lm = __ballot_sync(kFull, left);
      const unsigned vm = __ballot_sync(kFull, valid);
      lcnt += __popc(lm & cmr[r]);
      if (valid) {
        const int pl = __popc(lm & lt);
        const long long dst =
            nd.ebeg + (left ? offl + pl : best.nl_e + offr + (__popc(vm & lt) - pl));
        a.rowsB[dst] = rowr[r];
        if (a.wB) a.wB[dst] = a.wA ? __ldg(a.wA + nd.ebeg + i) : 1;
      }
      offl += __popc(lm);
      offr += __popc(vm) - __popc(lm);
    }
    if (P.task == 0 && lane < C) a.res_cnt[(long long)node * a.Cmax + lane] = lcnt;
    __syncwarp();
  }
}

}  // namespace dml
