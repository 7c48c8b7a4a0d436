// Fit kernels: root construction, per-level split search + stable partition
// (ERT and RF, classification and regression), level scans and model emission.
//
// Reference path restated (lib_ensembles/source):
//   gpurf.cu:58-129 / gpuert.cu:54-118   tree-batch init (bootstrap / identity)
//   gpuert.cu:119-247, 275-381           ERT node search
//   gpurf.cu:131-259, 440-917            RF node search (sort + boundary scan)
//   gpudte.cu:156-309                    node split: partition, children, leaf
//   gpudte_algorithm.cc:46-92            level-by-level node-array assembly
#pragma once
#include <cuda_runtime.h>

#include "dml_device.cuh"
#include "dml_internal.h"

namespace dml {

constexpr unsigned kFull = 0xFFFFFFFFu;

// -------------------------------------------------------------- block scans
template <int BLOCK, class T>
__device__ __forceinline__ T block_excl_scan(T v, T* total, T* sm) {
  constexpr int NW = BLOCK / 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[w] = x;
  __syncthreads();
  if (w == 0) {
    T t = lane < NW ? sm[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(kFull, t, o);
      if (lane >= o) t += y;
    }
    if (lane < NW) sm[lane] = t;
  }
  __syncthreads();
  T base = w ? sm[w - 1] : T(0);
  *total = sm[NW - 1];
  __syncthreads();
  return base + x - v;
}

// Exclusive block scans of NV 64-bit integers at once (one pair of barriers
// for all of them); tot[j] receives the block total of value j.  sm holds
// BLOCK/32 * NV words.  Integer sums, so the result is the same in any order.
template <int BLOCK, int NV>
__device__ __forceinline__ void block_excl_scan_n(unsigned long long (&v)[NV],
                                                  unsigned long long (&tot)[NV],
                                                  unsigned long long* sm) {
  constexpr int NW = BLOCK / 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long x[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    x[j] = v[j];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(kFull, x[j], o);
      if (lane >= o) x[j] += y;
    }
  }
  if (lane == 31)
#pragma unroll
    for (int j = 0; j < NV; ++j) sm[w * NV + j] = x[j];
  __syncthreads();
  if (w == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      unsigned long long t = lane < NW ? sm[lane * NV + j] : 0ull;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(kFull, t, o);
        if (lane >= o) t += y;
      }
      if (lane < NW) sm[lane * NV + j] = t;
    }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    const unsigned long long base = w ? sm[(w - 1) * NV + j] : 0ull;
    tot[j] = sm[(NW - 1) * NV + j];
    v[j] = base + x[j] - v[j];
  }
  __syncthreads();
}

// The block's best boundary: valid (p >= 0) first, then the higher gain, then
// the lower position -- a total order, so any reduction shape gives the same
// winner.  Warp shuffles, one exchange of the warps' winners through sg / sp
// (BLOCK/32 entries each), one barrier; every thread returns the position.
// Callers separate a later reuse of sg / sp by a barrier.
template <int BLOCK>
__device__ __forceinline__ int block_best_pos(float g, int p, float* sg, int* sp) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float g2 = __shfl_xor_sync(kFull, g, o);
    const int p2 = __shfl_xor_sync(kFull, p, o);
    if (p2 >= 0 && (p < 0 || g2 > g || (g2 == g && p2 < p))) {
      g = g2;
      p = p2;
    }
  }
  if (lane == 0) {
    sg[w] = g;
    sp[w] = p;
  }
  __syncthreads();
  float bg = sg[0];
  int bp = sp[0];
#pragma unroll
  for (int k = 1; k < BLOCK / 32; ++k) {
    const float g2 = sg[k];
    const int p2 = sp[k];
    if (p2 >= 0 && (bp < 0 || g2 > bg || (g2 == bg && p2 < bp))) {
      bg = g2;
      bp = p2;
    }
  }
  return bp;
}

template <class T>
__device__ __forceinline__ T warp_excl_scan(T v) {
  const int lane = threadIdx.x & 31;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  return x - v;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// ----------------------------------------------------------- candidates
struct Cand {
  int valid;
  float gain;
  int f;
  float thr;
  int nl_e, nl;
  long long suml;
};

__device__ __forceinline__ bool better(const Cand& a, const Cand& b) {
  return cand_better(a.valid != 0, a.gain, a.f, a.thr, b.valid != 0, b.gain, b.f, b.thr);
}

__device__ __forceinline__ int feature_of_try(const ProbDesc& P, const LNode& nd, int t) {
  U4 w = keyed(P.seed, kTagFeature, (uint32_t)nd.depth, (uint32_t)(nd.tree + P.tree_key0),
               (uint32_t)nd.idx,
               (uint32_t)t);
  return (int)(w.x % (uint32_t)P.F);
}

// ERT threshold: mean of 10 node values drawn with replacement, summed in
// draw order in FP32 (gpuert.cu:167-183 with a fixed order).
__device__ __forceinline__ float ert_threshold(const ProbDesc& P, const LNode& nd, int t, int f,
                                               const int* rows) {
  const float* xf = P.X + (long long)f * P.N;
  float v[10];
#pragma unroll
  for (int g = 0; g < 3; ++g) {
    U4 w = keyed(P.seed, kTagSample, (uint32_t)nd.depth, (uint32_t)(nd.tree + P.tree_key0),
                 (uint32_t)nd.idx,
                 (uint32_t)(t * 3 + g));
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      int j = g * 4 + s;
      if (j < 10) {
        uint32_t pos = pick(w, s) % (uint32_t)nd.ecnt;
        v[j] = __ldg(xf + __ldg(rows + pos));
      }
    }
  }
  float acc = 0.0f;
#pragma unroll
  for (int j = 0; j < 10; ++j) acc = __fadd_rn(acc, v[j]);
  return __fdiv_rn(acc, 10.0f);
}

// ------------------------------------------------------- stable partition
// Entries [ebeg, ebeg+m) of (rowsA, wA) into (rowsB, wB): left entries first
// in their order, then right entries in their order (gpudte.cu:205-232 made
// stable).  wA may be null (unit weights).
template <int BLOCK>
__device__ void cta_partition(const int* rowsA, const int* wA, int* rowsB, int* wB,
                              long long ebeg, int m, int nl_e, const float* xf, float thr,
                              int* sm) {
  int offl = 0, offr = 0;
  for (int base = 0; base < m; base += BLOCK) {
    int i = base + threadIdx.x;
    int row = 0, w = 1, left = 0;
    if (i < m) {
      row = rowsA[ebeg + i];
      if (wA) w = wA[ebeg + i];
      left = goes_left(__ldg(xf + row), thr) ? 1 : 0;
    }
    int tot;
    int pos = block_excl_scan<BLOCK, int>(left, &tot, sm);
    if (i < m) {
      long long dst = left ? ebeg + offl + pos : ebeg + nl_e + offr + (threadIdx.x - pos);
      rowsB[dst] = row;
      if (wB) wB[dst] = w;
    }
    offl += tot;
    offr += min(BLOCK, m - base) - tot;
  }
}

__device__ __forceinline__ void write_result(NodeRes* res, int* res_cnt, int Cmax, int node,
                                             const Cand& b, const int* Lc, int C) {
  NodeRes r;
  r.split = 1;
  r.f = b.f;
  r.thr = b.thr;
  r.gain = b.gain;
  r.nl_e = b.nl_e;
  r.nl = b.nl;
  r.suml = b.suml;
  res[node] = r;
  if (Lc)
    for (int c = 0; c < C; ++c) res_cnt[(long long)node * Cmax + c] = Lc[c];
}

__device__ __forceinline__ void write_leaf(NodeRes* res, int node) {
  NodeRes r;
  r.split = 0;
  r.f = -1;
  r.thr = 0.0f;
  r.gain = 0.0f;
  r.nl_e = 0;
  r.nl = 0;
  r.suml = 0;
  res[node] = r;
}

struct LevelArgs {
  const ProbDesc* probs;
  const LNode* nodes;
  const int* cnt;       // node class counts [node * Cmax]
  int Cmax;
  const int* work;      // node ids
  int nwork;
  NodeRes* res;
  int* res_cnt;         // left class counts of the chosen split [node * Cmax]
  const int* rowsA;
  const int* wA;        // null for unit weights (ERT)
  int* rowsB;
  int* wB;
  const long long* H;   // n*ln(n) table, fixed point 2^-28
  long long* stats;     // [2] += tries evaluated x node entries, [3] += node entries
  int smem_cap;         // entries per node of the shared-memory RF search's buffers
};

// ================================================================== ERT (CTA)
// One CTA per node: thresholds of a chunk of tries, one pass over the node's
// entries building every try's 2 x C histogram with warp ballots, gains,
// the try loop's decision, then the stable partition.
constexpr int kErtChunk = 16;

// Six resident CTAs per SM (40 registers, no spills): on the 256 uneven
// forests the class took 13.5 ms at the four CTAs that 64 registers allow,
// 11.5 at six and 12.5 at eight.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 6) k_ert_cta(LevelArgs a) {
  constexpr int NW = BLOCK / 32;
  __shared__ int s_f[kErtChunk];
  __shared__ float s_thr[kErtChunk];
  __shared__ int s_cntw[NW][kErtChunk][kMaxClasses];   // per-warp left class counts
  __shared__ long long s_sumw[NW][kErtChunk];          // per-warp left target sums
  __shared__ int s_nlw[NW][kErtChunk];                 // per-warp left counts (regression)
  __shared__ Cand s_cand[kErtChunk];
  __shared__ int s_L[kErtChunk][kMaxClasses];
  __shared__ int s_bestL[kMaxClasses];
  __shared__ Cand s_best;
  __shared__ int s_phase;  // 0 stop, 1 run optional chunk
  __shared__ int s_scan[NW];
  __shared__ long long s_prior;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int wi = blockIdx.x; wi < a.nwork; wi += gridDim.x) {
    const int node = a.work[wi];
    const LNode nd = a.nodes[node];
    const ProbDesc& P = a.probs[nd.prob];
    const int C = P.C;
    const int* rows = a.rowsA + nd.ebeg;
    const int* ncnt = a.cnt + (long long)node * a.Cmax;
    const int ml = max(1, P.min_leaf);
    if (threadIdx.x == 0 && P.task == 0)
      s_prior = entropy_prior(a.H, nd.n, C, [&](int c) { return (long long)ncnt[c]; });
    // chunks: mandatory tries [0, n_mand) in chunks, then one optional chunk
    int t0 = 0, tries_done = 0;
    bool optional = false;
    while (true) {
      const int tcount = optional ? P.n_opt : min(kErtChunk, P.n_mand - t0);
      tries_done += tcount;
      if (threadIdx.x < tcount) {
        int t = t0 + threadIdx.x;
        int f = feature_of_try(P, nd, t);
        s_f[threadIdx.x] = f;
        s_thr[threadIdx.x] = ert_threshold(P, nd, t, f, rows);
      }
      for (int i = threadIdx.x; i < NW * kErtChunk * kMaxClasses; i += BLOCK)
        (&s_cntw[0][0][0])[i] = 0;
      for (int i = threadIdx.x; i < NW * kErtChunk; i += BLOCK) {
        (&s_sumw[0][0])[i] = 0;
        (&s_nlw[0][0])[i] = 0;
      }
      __syncthreads();
      // one pass over the entries
      for (int base = warp * 32; base < nd.ecnt; base += BLOCK) {
        const int i = base + lane;
        const bool valid = i < nd.ecnt;
        const int row = valid ? __ldg(rows + i) : 0;
        if (P.task == 0) {
          const int k = valid ? __ldg(P.lab + row) : -1;
          unsigned my = 0;
          for (int c = 0; c < C; ++c) {
            unsigned mc = __ballot_sync(kFull, k == c);
            if (lane == c) my = mc;
          }
          for (int t = 0; t < tcount; ++t) {
            bool left = valid && goes_left(__ldg(P.X + (long long)s_f[t] * P.N + row), s_thr[t]);
            unsigned lm = __ballot_sync(kFull, left);
            if (lane < C) s_cntw[warp][t][lane] += __popc(lm & my);
          }
        } else {
          const long long qv = valid ? __ldg(P.q + row) : 0;
          for (int t = 0; t < tcount; ++t) {
            bool left = valid && goes_left(__ldg(P.X + (long long)s_f[t] * P.N + row), s_thr[t]);
            unsigned lm = __ballot_sync(kFull, left);
            long long s = warp_sum<long long>(left ? qv : 0);
            if (lane == 0) {
              s_nlw[warp][t] += __popc(lm);
              s_sumw[warp][t] += s;
            }
          }
        }
      }
      __syncthreads();
      // reduce warps, gains per try
      if (P.task == 0) {
        for (int i = threadIdx.x; i < tcount * C; i += BLOCK) {
          int t = i / C, c = i % C, s = 0;
          for (int w = 0; w < NW; ++w) s += s_cntw[w][t][c];
          s_L[t][c] = s;
        }
        __syncthreads();
        if (threadIdx.x < tcount) {
          const int t = threadIdx.x;
          long long nl = 0;
          for (int c = 0; c < C; ++c) nl += s_L[t][c];
          long long nr = (long long)nd.n - nl;
          Cand cd;
          cd.f = s_f[t];
          cd.thr = s_thr[t];
          cd.nl_e = (int)nl;
          cd.nl = (int)nl;
          cd.suml = 0;
          cd.valid = nl >= ml && nr >= ml;
          cd.gain = cd.valid ? entropy_gain(
                                   a.H, s_prior, C, nl, nr,
                                   [&](int c) { return (long long)s_L[t][c]; },
                                   [&](int c) { return (long long)ncnt[c]; })
                             : -FLT_MAX;
          s_cand[t] = cd;
        }
      } else {
        if (threadIdx.x < tcount) {
          const int t = threadIdx.x;
          long long nl = 0, sl = 0;
          for (int w = 0; w < NW; ++w) {
            nl += s_nlw[w][t];
            sl += s_sumw[w][t];
          }
          long long nr = (long long)nd.n - nl;
          Cand cd;
          cd.f = s_f[t];
          cd.thr = s_thr[t];
          cd.nl_e = (int)nl;
          cd.nl = (int)nl;
          cd.suml = sl;
          cd.valid = nl >= ml && nr >= ml;
          cd.gain = cd.valid ? variance_gain(nl, sl, nr, nd.sum - sl, P.S) : -FLT_MAX;
          s_cand[t] = cd;
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        int next = 0;
        if (!optional) {
          for (int t = 0; t < tcount; ++t) {
            if ((t0 + t == 0) || better(s_cand[t], s_best)) {
              s_best = s_cand[t];
              if (P.task == 0)
                for (int c = 0; c < C; ++c) s_bestL[c] = s_L[t][c];
            }
          }
          if (t0 + tcount < P.n_mand)
            next = 1;  // more mandatory tries
          else if (P.n_opt > 0 && !(s_best.valid && s_best.gain >= kSensible))
            next = 2;
        } else {
          for (int t = 0; t < tcount; ++t) {
            if (better(s_cand[t], s_best)) {
              s_best = s_cand[t];
              if (P.task == 0)
                for (int c = 0; c < C; ++c) s_bestL[c] = s_L[t][c];
            }
            if (s_cand[t].valid && s_cand[t].gain >= kSensible) break;
          }
        }
        s_phase = next;
      }
      __syncthreads();
      const int ph = s_phase;
      __syncthreads();
      if (ph == 0) break;
      if (ph == 1) t0 += tcount;
      if (ph == 2) {
        optional = true;
        t0 = P.n_mand;
      }
    }
    const Cand b = s_best;
    if (threadIdx.x == 0) {
      atomicAdd((unsigned long long*)&a.stats[2],
                (unsigned long long)tries_done * nd.ecnt);
      atomicAdd((unsigned long long*)&a.stats[3], (unsigned long long)nd.ecnt);
    }
    if (!b.valid) {
      if (threadIdx.x == 0) write_leaf(a.res, node);
    } else {
      if (threadIdx.x == 0)
        write_result(a.res, a.res_cnt, a.Cmax, node, b, P.task == 0 ? s_bestL : nullptr, C);
      cta_partition<BLOCK>(a.rowsA, a.wA, a.rowsB, a.wB, nd.ebeg, nd.ecnt, b.nl_e,
                           P.X + (long long)b.f * P.N, b.thr, s_scan);
    }
    __syncthreads();
  }
}

// ============================================================ RF (CTA, sorted)
// Radix sort (LSD, 8-bit digits) of (key, value) pairs held in shared memory.
// Stability comes from per-warp contiguous chunks and in-order ranking of
// equal digits within a warp (digit_peers).
// Lanes of `mask` whose digit equals this lane's.  Every lane of `mask` must
// call it.  (One match instruction measured faster on the big-node passes than
// eight ballots, one per digit bit.)
__device__ __forceinline__ unsigned digit_peers(unsigned mask, unsigned d) {
  return __match_any_sync(mask, d);
}

template <int BLOCK>
struct SortSmem {
  unsigned hist[BLOCK / 32][256];
  unsigned digit_base[256];
  unsigned scan_tmp[BLOCK / 32];
};

template <int BLOCK>
__device__ void radix_pass(const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                           uint32_t* vout, int m, int shift, SortSmem<BLOCK>& S) {
  static_assert(BLOCK == 256, "one thread per digit");
  constexpr int NW = BLOCK / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int chunk = ((m + NW - 1) / NW + 31) & ~31;
  const int beg = min(m, warp * chunk), end = min(m, beg + chunk);
  // each warp clears and fills its own histogram row
  for (int i = lane; i < 256; i += 32) S.hist[warp][i] = 0;
  __syncwarp();
  for (int i = beg + lane; i < end; i += 32) atomicAdd(&S.hist[warp][(kin[i] >> shift) & 255u], 1u);
  __syncthreads();
  // digit-major, warp-minor exclusive offsets; thread d owns digit d
  {
    const int d = threadIdx.x;
    unsigned h[NW];
    unsigned tot = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      h[w] = S.hist[w][d];
      tot += h[w];
    }
    unsigned x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) S.scan_tmp[warp] = x;
    __syncthreads();
    unsigned run = x - tot;
    for (int w = 0; w < warp; ++w) run += S.scan_tmp[w];
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      S.hist[w][d] = run;
      run += h[w];
    }
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  for (int b = beg; b < end; b += 32) {
    const int i = b + lane;
    const bool act = i < end;
    const unsigned mask = __ballot_sync(kFull, act);
    if (act) {
      uint32_t k = kin[i], v = vin[i];
      unsigned d = (k >> shift) & 255u;
      unsigned peers = digit_peers(mask, d);
      unsigned pos = S.hist[warp][d] + __popc(peers & lt);
      kout[pos] = k;
      vout[pos] = v;
      __syncwarp(mask);
      if ((peers & lt) == 0) S.hist[warp][d] += __popc(peers);
    }
    __syncwarp();
  }
  __syncthreads();
}

// Sorts pairs whose varying key bits are `diff` (OR ^ AND of all keys, which
// the caller reduced while writing them).  Passes whose digit is constant are
// skipped; returns true when the sorted pairs are in k2/v2, false when in k/v.
template <int BLOCK>
__device__ bool cta_radix_sort_diff(uint32_t* k, uint32_t* v, uint32_t* k2, uint32_t* v2, int m,
                                    unsigned diff, SortSmem<BLOCK>& S) {
  bool in_primary = true;
  for (int shift = 0; shift < 32; shift += 8) {
    if (((diff >> shift) & 255u) == 0) continue;
    if (in_primary)
      radix_pass<BLOCK>(k, v, k2, v2, m, shift, S);
    else
      radix_pass<BLOCK>(k2, v2, k, v, m, shift, S);
    in_primary = !in_primary;
  }
  return !in_primary;
}

}  // namespace dml
