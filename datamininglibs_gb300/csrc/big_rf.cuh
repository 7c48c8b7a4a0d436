// RF split search for large nodes (more entries than fit a shared-memory
// sort): one CTA per (node, try) work item on a persistent grid, each with its
// own global scratch.  The item gathers its keys (value ranks) and the node's
// packed (label, weight) values, counting the digit histograms of the keys'
// significant bytes on the way.  The sort is an LSD radix sort (8-bit digits)
// over tiles of 2048 pairs: each warp loads its 256-pair chunk with eight loads
// in flight, ranks digits stably within warps (digit_peers), and the tile is
// reordered in shared memory so that every digit's run is written to global
// memory as one contiguous stretch.  The boundary scan gives each thread 8
// consecutive sorted elements (one block scan of packed class counts per 2048
// elements) and keeps the entropy incrementally; a regression item's scan
// reads one packed (target, weight) word per element and evaluates the
// float-float variance gain only where its bound reaches the warp's best.
// Both scans run out of line from the sort.  A second kernel applies the try
// loop (gpurf.cu:177-245) per node and partitions its entries.  The
// shared-memory kernel for mid-size nodes (k_rf_smem) is at the end.
#pragma once
#include "fit_kernels.cuh"
#include "warp_rf.cuh"

namespace dml {

constexpr int kBigBlock = 256;
constexpr int kBigPer = 8;                       // elements per thread
constexpr int kBigTile = kBigBlock * kBigPer;    // 2048
constexpr int kBigWarps = kBigBlock / 32;
constexpr int kBigPerKeys = 16;                  // elements per thread of a keys-only pass

struct BigSmem {
  unsigned whist[kBigWarps][256];
  unsigned tstart[256];
  unsigned running[2][256];
  unsigned red[2 * kBigWarps];
  // a pass's tile: keys in [0, kBigTile), values after them; the class
  // columns of the classification scan once the sort is done
  uint32_t tile[2 * kBigTile];
  unsigned long long scan64[kBigWarps * (kMaxClasses / 2 + 1)];  // block_excl_scan_n, CW + 1 values
  unsigned scan32[kBigWarps];
  unsigned dh[4][256];  // per-digit histograms of the item's keys, counted while gathering
};

// Adds one warp-round of digits to a histogram: every lane of the warp calls,
// `act` lanes contribute.  A round whose active lanes share one digit (a
// constant byte) adds with one atomic instead of 32 on the same word.
__device__ __forceinline__ void hist_add_round(unsigned* h, unsigned dgt, bool act) {
  const unsigned mask = __ballot_sync(kFull, act);
  if (mask == 0) return;
  const int src = __ffs(mask) - 1;
  const unsigned d0 = __shfl_sync(kFull, dgt, src);
  if (__all_sync(kFull, !act || dgt == d0)) {
    if ((int)(threadIdx.x & 31) == src) atomicAdd(&h[d0], (unsigned)__popc(mask));
  } else if (act) {
    atomicAdd(&h[dgt], 1u);
  }
}

// The value of a sort key of feature f: a rank (looked up) or an orderable key.
// Equal to from_orderable of the value's key either way (-0 reads as +0).
__device__ __forceinline__ float key_value(const ProbDesc& P, int f, uint32_t k) {
  return P.rank ? __ldg(P.vals + (long long)f * P.N + k) : from_orderable(k);
}

// Exclusive scan over the 256 digits of per-digit totals (thread d owns digit
// d): warp shuffles, one exchange of warp sums, one barrier.  The caller
// separates a later reuse of sm (kBigWarps words) by a barrier.
static __device__ __forceinline__ unsigned digit_excl_scan(unsigned tot, unsigned* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned x = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[warp] = x;
  __syncthreads();
  unsigned ex = x - tot;
  for (int w = 0; w < warp; ++w) ex += sm[w];
  return ex;
}

// One LSD pass of pairs (kin, vin) -> (kout, vout) on the 8-bit digit at bit
// `shift`, whose histogram over all m keys is dh; a null vin stands for the
// values 0 .. m-1.  Without VALS the keys move alone (packed keys carry their
// values, and PER elements a thread fill the whole tile buffer).  Scratch
// written earlier in the same kernel is read with plain loads (never the
// read-only cache path).
template <bool VALS, int PER = kBigPer>
static __device__ void big_pass(const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                                uint32_t* vout, int m, int shift, const unsigned* dh,
                                BigSmem& S) {
  static_assert(kBigBlock == 256, "one thread per digit");
  constexpr int T = kBigBlock * PER;  // entries a tile
  static_assert(VALS ? T == kBigTile : T <= 2 * kBigTile, "the tile fits its buffer");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int dg = threadIdx.x;
  const unsigned lt = (1u << lane) - 1u;
  // each digit's first output position
  S.running[0][dg] = digit_excl_scan(dh[dg], S.scan32);
  __syncthreads();
  // tiles: stable local sort in shared memory, contiguous run writes; the
  // running positions are double-buffered (tile t reads running[cur] and
  // writes running[cur ^ 1] for tile t + 1)
  int cur = 0;
  for (int base = 0; base < m; base += T) {
    const int tn = min(T, m - base);
    const int wbeg = warp * 32 * PER;
    uint32_t k[PER], v[VALS ? PER : 1];
#pragma unroll
    for (int r = 0; r < PER; ++r) {
      const int i = wbeg + r * 32 + lane;
      k[r] = i < tn ? kin[base + i] : 0u;
      if (VALS) v[r] = i < tn ? (vin ? vin[base + i] : (uint32_t)(base + i)) : 0u;
    }
    for (int i = lane; i < 256; i += 32) S.whist[warp][i] = 0;
    __syncwarp();
    unsigned pr[PER];  // each element's equal-digit lanes, reused by the scatter
#pragma unroll
    for (int r = 0; r < PER; ++r) {
      const int i = wbeg + r * 32 + lane;
      const bool act = i < tn;
      const unsigned mask = __ballot_sync(kFull, act);
      pr[r] = 0;
      if (act) {
        const unsigned dgt = (k[r] >> shift) & 255u;
        const unsigned peers = digit_peers(mask, dgt);
        pr[r] = peers;
        if ((peers & lt) == 0) S.whist[warp][dgt] += __popc(peers);
      }
      __syncwarp();
    }
    __syncthreads();
    {
      unsigned h[kBigWarps];
      unsigned tot = 0;
#pragma unroll
      for (int w = 0; w < kBigWarps; ++w) {
        h[w] = S.whist[w][dg];
        tot += h[w];
      }
      const unsigned ex = digit_excl_scan(tot, S.scan32);
      S.tstart[dg] = ex;
      unsigned run = ex;
#pragma unroll
      for (int w = 0; w < kBigWarps; ++w) {
        S.whist[w][dg] = run;
        run += h[w];
      }
      S.running[cur ^ 1][dg] = S.running[cur][dg] + tot;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PER; ++r) {
      const int i = wbeg + r * 32 + lane;
      const bool act = i < tn;
      const unsigned mask = __ballot_sync(kFull, act);
      if (act) {
        const unsigned dgt = (k[r] >> shift) & 255u;
        const unsigned peers = pr[r];
        const unsigned pos = S.whist[warp][dgt] + __popc(peers & lt);
        S.tile[pos] = k[r];
        if (VALS) S.tile[kBigTile + pos] = v[r];
        __syncwarp(mask);
        if ((peers & lt) == 0) S.whist[warp][dgt] += __popc(peers);
      }
      __syncwarp();
    }
    __syncthreads();
    for (int j = threadIdx.x; j < tn; j += kBigBlock) {
      const uint32_t kk = S.tile[j];
      const unsigned dgt = (kk >> shift) & 255u;
      const unsigned pos = S.running[cur][dgt] + (j - S.tstart[dgt]);
      kout[pos] = kk;
      if (VALS) vout[pos] = S.tile[kBigTile + j];
    }
    __syncthreads();
    cur ^= 1;
  }
}

// Sorts the keys k of length m, whose varying bits are `diff` (not 0) and
// whose digit histograms are S.dh, with their values: the first pass reads
// the values from v0 (null: 0 .. m-1), later passes from the buffer the
// previous pass wrote.  Passes whose byte is the same in every key are
// skipped; returns true when the result is in (k2, v2), false when in (k, v).
static __device__ bool big_sort(uint32_t* k, uint32_t* v, uint32_t* k2, uint32_t* v2,
                                const uint32_t* v0, int m, unsigned diff, BigSmem& S) {
  bool primary = true, first = true;
  for (int d = 0; d < 4; ++d) {
    const int shift = 8 * d;
    if (((diff >> shift) & 255u) == 0) continue;
    if (primary)
      big_pass<true>(k, first ? v0 : v, k2, v2, m, shift, S.dh[d], S);
    else
      big_pass<true>(k2, v2, k, v, m, shift, S.dh[d], S);
    primary = !primary;
    first = false;
    __syncthreads();
  }
  return !primary;
}

// Sorts packed keys k (rank << pb | payload) of length m on their rank bits,
// whose varying bits are `diff` (of the ranks) and whose digit histograms are
// S.dh; returns true when the result is in k2, false when in k.
static __device__ bool big_sort_keys(uint32_t* k, uint32_t* k2, int m, unsigned diff, int pb,
                                     BigSmem& S) {
  bool primary = true;
  for (int d = 0; d < 4; ++d) {
    if (((diff >> (8 * d)) & 255u) == 0) continue;
    if (primary)
      big_pass<false, kBigPerKeys>(k, nullptr, k2, nullptr, m, pb + 8 * d, S.dh[d], S);
    else
      big_pass<false, kBigPerKeys>(k2, nullptr, k, nullptr, m, pb + 8 * d, S.dh[d], S);
    primary = !primary;
    __syncthreads();
  }
  return !primary;
}

struct BigArgs {
  LevelArgs L;
  const int* big;          // big node ids
  int nbig;
  const int* retry;        // nodes needing optional tries (phase 2)
  const int* nretry;       // device count
  int phase;               // 1 mandatory tries, 2 optional tries
  int tries_per_node;      // slots per node in this phase
  Cand* cand;              // [node slot][try slot]
  int* candL;              // [node slot][try slot][Cmax]
  uint32_t* slot;          // per-CTA scratch: 4 * slot_stride words
  long long slot_stride;   // >= the largest node's entry count
  Cand* partial;           // [big index] best of the mandatory tries
  int* partialL;           // [big index][Cmax]
  int* retry_out;          // append list of nodes (phase 1 decide)
  int* nretry_out;
  int* big_index;          // node id -> index in `big` (for phase 2)
  uint32_t* pv;            // classification: label << 27 | weight per entry slot of the big nodes
  long long* pq;           // regression: packed (target, weight) per entry slot of the big nodes
  int* item_ctr;           // [phase - 1]: items handed out so far, zero before the launch
  const int* maxw;         // the fit's largest entry weight
};

// Per-entry values of the big nodes, once per level instead of a gather by
// row per try: packed (label << 27 | weight) for classification, the packed
// (target, weight) word (qw_pack) for regression.
template <int CW>
__global__ void __launch_bounds__(kBigBlock) k_big_pack(BigArgs b) {
  const LevelArgs& a = b.L;
  for (int ni = blockIdx.x; ni < b.nbig; ni += gridDim.x) {
    const LNode nd = a.nodes[b.big[ni]];
    const ProbDesc& P = a.probs[nd.prob];
    if (P.task == 0 && b.pv) {
      for (int i = threadIdx.x; i < nd.ecnt; i += kBigBlock) {
        const long long e = nd.ebeg + i;
        b.pv[e] = ((uint32_t)__ldg(P.lab + __ldg(a.rowsA + e)) << 27) |
                  (uint32_t)(a.wA ? __ldg(a.wA + e) : 1);
      }
    } else if (P.task != 0 && b.pq) {
      const int wb = qw_bits(P.N);
      for (int i = threadIdx.x; i < nd.ecnt; i += kBigBlock) {
        const long long e = nd.ebeg + i;
        b.pq[e] = qw_pack(__ldg(P.q + __ldg(a.rowsA + e)), a.wA ? __ldg(a.wA + e) : 1, wb);
      }
    }
  }
}

// Boundary scan of a sorted classification item, whose values are the packed
// (label << 27 | weight) words: each thread owns `per` (1..8) consecutive
// elements of every tile of 256 * per.  INCR: each thread keeps its values in
// registers and Q incrementally along its elements (6 table terms an entry
// instead of 2C + 2 a boundary); worth it for 8 elements per thread.
template <int CW, bool INCR>
__device__ void big_boundary(const uint32_t* sk, const uint32_t* sv, int m, int per,
                             const LNode& nd, const ProbDesc& P, const int* ncnt,
                             const long long* H, long long prior, unsigned long long* scan64,
                             float* out_g, int* out_p, long long* out_nl,
                             unsigned long long (&outL)[CW]) {
  const int C = P.C;
  const int ml = max(1, P.min_leaf);
  int Nt[2 * CW];
#pragma unroll
  for (int c = 0; c < 2 * CW; ++c) Nt[c] = c < C ? ncnt[c] : 0;
  NumBest nb;
  nb.init();
  long long bnl = 0;
  unsigned long long bL[CW];
  unsigned long long carry[CW];
  long long carry_n = 0;
#pragma unroll
  for (int j = 0; j < CW; ++j) {
    bL[j] = 0;
    carry[j] = 0;
  }
  for (int base = 0; base < m; base += kBigBlock * per) {
    const int p0 = base + threadIdx.x * per;
    const uint32_t prevk0 = p0 > 0 && p0 - 1 < m ? sk[p0 - 1] : 0u;
    // per-thread totals from the packed values (which the scan below reads
    // again) and a bit mask of the key boundaries
    long long tn = 0;
    unsigned long long tl[CW];
#pragma unroll
    for (int c = 0; c < CW; ++c) tl[c] = 0;
    uint32_t vq[kBigPer];  // INCR: the packed values, consumed from vq[0]
    unsigned bnd = 0;  // bit j set when element j starts a new key
    {
      uint32_t prev = prevk0;
#pragma unroll
      for (int j = 0; j < kBigPer; ++j) {
        const int p = p0 + j;
        vq[j] = 0;
        if (j < per && p < m) {
          const uint32_t kj = sk[p];
          const uint32_t vv = sv[p];
          vq[j] = vv;
          if (p > 0 && prev < kj) bnd |= 1u << j;
          prev = kj;
          const int lj = (int)(vv >> 27);
          const int wj = (int)(vv & 0x7FFFFFFu);
          tn += wj;
#pragma unroll
          for (int c = 0; c < CW; ++c)
            tl[c] += (lj == 2 * c ? (unsigned long long)wj : 0ull) |
                     (lj == 2 * c + 1 ? ((unsigned long long)wj << 32) : 0ull);
        }
      }
    }
    // one block scan of the row count and the packed class counts of every
    // thread's elements
    unsigned long long sv_[CW + 1], tot[CW + 1];
    sv_[0] = (unsigned long long)tn;
#pragma unroll
    for (int c = 0; c < CW; ++c) sv_[1 + c] = tl[c];
    block_excl_scan_n<kBigBlock, CW + 1>(sv_, tot, scan64);
    long long run_n = carry_n + (long long)sv_[0];
    carry_n += (long long)tot[0];
    unsigned long long runL[CW];
#pragma unroll
    for (int c = 0; c < CW; ++c) {
      runL[c] = carry[c] + sv_[1 + c];
      carry[c] += tot[1 + c];
    }
    if (INCR) {
      // Q computed in full at the first boundary that meets min_leaf, then
      // moved entry by entry while boundaries remain (h(nL), h(nR) carried)
      long long Q = 0, hl = 0, hr = 0;
      bool haveQ = false;
#pragma unroll 1
      for (int j = 0; j < per; ++j) {
        const uint32_t vv = vq[0];
#pragma unroll
        for (int k = 0; k + 1 < kBigPer; ++k) vq[k] = vq[k + 1];
        const int p = p0 + j;
        const int labj = (int)(vv >> 27);
        const int wj = (int)(vv & 0x7FFFFFFu);
        const long long nr = (long long)nd.n - run_n;
        if (((bnd >> j) & 1u) && run_n >= ml && nr >= ml) {
          if (!haveQ) {
            Q = entropy_q_u<2 * CW>(
                H, C, run_n, nr,
                [&](int c) {
                  return (long long)((c & 1) ? (runL[c >> 1] >> 32) : (runL[c >> 1] & 0xFFFFFFFFull));
                },
                [&](int c) { return (long long)Nt[c]; });
            hl = __ldg(H + run_n);
            hr = __ldg(H + nr);
            haveQ = true;
          }
          if (nb.offer(prior - Q, p, nd.n)) {
            bnl = run_n;
#pragma unroll
            for (int c = 0; c < CW; ++c) bL[c] = runL[c];
          }
        }
        if (haveQ && (bnd >> (j + 1)) != 0u) {
          const long long lc = packed_get<CW>(runL, labj);
          const long long rc = (long long)Nt_of<CW>(Nt, labj) - lc;
          const long long hl1 = __ldg(H + run_n + wj), hr1 = __ldg(H + nr - wj);
          Q += (hl1 - hl) + (hr1 - hr) - (__ldg(H + lc + wj) - __ldg(H + lc)) -
               (__ldg(H + rc - wj) - __ldg(H + rc));
          hl = hl1;
          hr = hr1;
        }
        run_n += wj;
#pragma unroll
        for (int c = 0; c < CW; ++c)
          runL[c] += (labj == 2 * c ? (unsigned long long)wj : 0ull) |
                     (labj == 2 * c + 1 ? ((unsigned long long)wj << 32) : 0ull);
      }
    } else {
      // a rolled loop that re-reads each label|weight value
      // (the class terms unrolled eight times overflow the instruction cache);
      // boundaries are compared on their exact gain numerators P - Q
#pragma unroll 1
      for (int j = 0; j < per; ++j) {
        const int p = p0 + j;
        int wj = 0, labj = 0;
        if (p < m) {
          const uint32_t vv = sv[p];
          labj = (int)(vv >> 27);
          wj = (int)(vv & 0x7FFFFFFu);
        }
        const long long nr = (long long)nd.n - run_n;
        if (((bnd >> j) & 1u) && run_n >= ml && nr >= ml) {
          const long long Q = entropy_q_u<2 * CW>(
              H, C, run_n, nr,
              [&](int c) {
                return (long long)((c & 1) ? (runL[c >> 1] >> 32) : (runL[c >> 1] & 0xFFFFFFFFull));
              },
              [&](int c) { return (long long)Nt[c]; });
          if (nb.offer(prior - Q, p, nd.n)) {
            bnl = run_n;
#pragma unroll
            for (int c = 0; c < CW; ++c) bL[c] = runL[c];
          }
        }
        run_n += wj;
#pragma unroll
        for (int c = 0; c < CW; ++c)
          runL[c] += (labj == 2 * c ? (unsigned long long)wj : 0ull) |
                     (labj == 2 * c + 1 ? ((unsigned long long)wj << 32) : 0ull);
      }
    }
  }
  *out_g = nb.gain(nd.n);
  *out_p = nb.p;
  *out_nl = bnl;
#pragma unroll
  for (int c = 0; c < CW; ++c) outL[c] = bL[c];
}

// The big items' classification scan, out of line: the sort's registers and
// the scan's are allocated separately (the shared-memory kernel, whose sort
// state is smaller, is faster with the scan inlined).
template <int CW>
static __device__ __noinline__ void big_boundary_items(const uint32_t* sk, const uint32_t* sv,
                                                       int m, const LNode& nd, const ProbDesc& P,
                                                       const int* ncnt, const long long* H,
                                                       long long prior,
                                                       unsigned long long* scan64, float* out_g,
                                                       int* out_p, long long* out_nl,
                                                       unsigned long long (&outL)[CW]) {
  big_boundary<CW, true>(sk, sv, m, kBigPer, nd, P, ncnt, H, prior, scan64, out_g, out_p, out_nl,
                         outL);
}

// Per-thread class counts of the column scan below: column c of thread t at
// c * kColStride + t + t / 32 (one pad word per 32 threads, so that a lane
// reading eight consecutive threads' words and a thread reading its own word
// both meet 32 different banks).
constexpr int kColStride = kBigBlock + kBigBlock / 32;
__device__ __forceinline__ int col_of(int t) { return t + (t >> 5); }

// Classification boundary scan with the class counts in shared memory:
// column c < C holds each thread's count of class c, column C its row count.
// Per tile of 256 * per sorted elements (per = 1..8 consecutive elements a
// thread) each thread adds its elements' weights to its own words; one warp per column turns the words into exclusive prefixes
// (eight words a lane, a warp scan of the lane totals, the column's carry from
// the earlier tiles); the incremental scan then reads and moves the one count
// an element changes, where the register form selects among the packed words
// for every class on every element.  Results equal big_boundary<CW, INCR>.
// cols: (C + 1) * kColStride words and C + 1 carries after them; nt: the
// node's class counts (shared memory).  Two CTA barriers per tile.  PK: the
// keys are packed (rank << pb | label << wb | weight) and sv is not read.
template <int CW, bool PK>
static __device__ __noinline__ void big_boundary_cols(const uint32_t* sk, const uint32_t* sv,
                                                      int m, int per, const LNode& nd, int C,
                                                      int ml, int pb, int wb,
                                                      const long long* H, long long prior,
                                                      const int* nt, uint32_t* cols,
                                                      float* out_g, int* out_p, long long* out_nl,
                                                      unsigned long long (&outL)[CW]) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int me = col_of(tid);
  uint32_t* carry = cols + (C + 1) * kColStride;
  if (tid <= C) carry[tid] = 0;
  NumBest nb;
  nb.init();
  long long bnl = 0;
  unsigned long long bL[CW];
#pragma unroll
  for (int j = 0; j < CW; ++j) bL[j] = 0;
  for (int base = 0; base < m; base += kBigBlock * per) {
    const int p0 = base + tid * per;
    const uint32_t prevk0 =
        p0 > 0 && p0 - 1 < m ? (PK ? sk[p0 - 1] >> pb : sk[p0 - 1]) : 0u;
    for (int c = 0; c <= C; ++c) cols[c * kColStride + me] = 0;
    uint32_t vq[kBigPer];
    unsigned bnd = 0;
    uint32_t tn = 0;
    {
      uint32_t prev = prevk0;
#pragma unroll
      for (int j = 0; j < kBigPer; ++j) {
        const int p = p0 + j;
        vq[j] = 0;
        if (j < per && p < m) {
          const uint32_t raw = sk[p];
          const uint32_t kj = PK ? raw >> pb : raw;
          const uint32_t vv =
              PK ? (((raw >> wb) & ((1u << (pb - wb)) - 1u)) << 27) | (raw & ((1u << wb) - 1u))
                 : sv[p];
          vq[j] = vv;
          if (p > 0 && prev < kj) bnd |= 1u << j;
          prev = kj;
          const uint32_t wj = vv & 0x7FFFFFFu;
          cols[(int)(vv >> 27) * kColStride + me] += wj;
          tn += wj;
        }
      }
    }
    cols[C * kColStride + me] = tn;
    __syncthreads();
    for (int c = warp; c <= C; c += kBigWarps) {
      uint32_t* col = cols + c * kColStride + 8 * lane + (lane >> 2);
      uint32_t x[8];
      uint32_t run = 0;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        x[i] = run;
        run += col[i];
      }
      uint32_t inc = run;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, inc, o);
        if (lane >= o) inc += y;
      }
      const uint32_t base_c = carry[c] + inc - run;
#pragma unroll
      for (int i = 0; i < 8; ++i) col[i] = base_c + x[i];
      const uint32_t total = __shfl_sync(kFull, inc, 31);
      __syncwarp();
      if (lane == 0) carry[c] += total;
    }
    __syncthreads();
    long long run_n = (long long)cols[C * kColStride + me];
    long long Q = 0, hl = 0, hr = 0;
    bool haveQ = false;
#pragma unroll 1
    for (int j = 0; j < per; ++j) {
      const uint32_t vv = vq[0];
#pragma unroll
      for (int k = 0; k + 1 < kBigPer; ++k) vq[k] = vq[k + 1];
      const int labj = (int)(vv >> 27);
      const int wj = (int)(vv & 0x7FFFFFFu);
      const long long nr = (long long)nd.n - run_n;
      if (((bnd >> j) & 1u) && run_n >= ml && nr >= ml) {
        if (!haveQ) {
          Q = entropy_q_u<2 * CW>(
              H, C, run_n, nr, [&](int c) { return (long long)cols[c * kColStride + me]; },
              [&](int c) { return (long long)nt[c]; });
          hl = __ldg(H + run_n);
          hr = __ldg(H + nr);
          haveQ = true;
        }
        if (nb.offer(prior - Q, p0 + j, nd.n)) {
          bnl = run_n;
#pragma unroll
          for (int c = 0; c < CW; ++c) {
            const unsigned long long lo = 2 * c < C ? cols[2 * c * kColStride + me] : 0u;
            const unsigned long long hi = 2 * c + 1 < C ? cols[(2 * c + 1) * kColStride + me] : 0u;
            bL[c] = lo | (hi << 32);
          }
        }
      }
      uint32_t* cl = cols + labj * kColStride + me;
      const long long lc = (long long)*cl;
      if (haveQ && (bnd >> (j + 1)) != 0u) {
        const long long rc = (long long)nt[labj] - lc;
        const long long hl1 = __ldg(H + run_n + wj), hr1 = __ldg(H + nr - wj);
        Q += (hl1 - hl) + (hr1 - hr) - (__ldg(H + lc + wj) - __ldg(H + lc)) -
             (__ldg(H + rc - wj) - __ldg(H + rc));
        hl = hl1;
        hr = hr1;
      }
      *cl = (uint32_t)(lc + wj);
      run_n += wj;
    }
  }
  *out_g = nb.gain(nd.n);
  *out_p = nb.p;
  *out_nl = bnl;
#pragma unroll
  for (int c = 0; c < CW; ++c) outL[c] = bL[c];
}

// Boundary scan of a sorted regression item, whose values index eq, the
// entries' packed (target, weight) words; `per` (1..8) consecutive elements a
// thread per tile as above.  Out of line, so that its registers do not weigh
// on the classification scan of the same kernels.  The float-float gain is
// evaluated only at boundaries whose upper bound (variance_gain_bounds)
// reaches t, the largest over the warp of the lanes' best gains so far and of
// the lower bounds of their boundaries in the tile: a boundary below t can
// neither be nor tie the block's best.  n, sum: the node's weight and
// weighted target sum; S: the target scale; N: the problem's rows (the
// packing).
static __device__ __noinline__ void big_boundary_reg(const uint32_t* sk, const uint32_t* sv,
                                                     const long long* eq, int m, int per,
                                                     long long n, long long sum, int ml, int S,
                                                     long long N, unsigned long long* scan64,
                                                     float* out_g, int* out_p, long long* out_nl,
                                                     long long* out_sl) {
  const int wb = qw_bits(N);
  const float rc = __frcp_rn(__ll2float_rn(n));
  const float p2 = pow2f(-2 * S);
  float bg = -FLT_MAX;
  int bp = -1;
  long long bnl = 0, bsl = 0;
  long long carry_n = 0, carry_s = 0;
  for (int base = 0; base < m; base += kBigBlock * per) {
    const int p0 = base + threadIdx.x * per;
    // weights and weighted targets in registers, a bit mask of the key
    // boundaries
    int w[kBigPer];
    long long q[kBigPer];
    unsigned bnd = 0;
    long long tn = 0, ts = 0;
    uint32_t prev = p0 > 0 && p0 - 1 < m ? sk[p0 - 1] : 0u;
#pragma unroll
    for (int j = 0; j < kBigPer; ++j) {
      const int p = p0 + j;
      w[j] = 0;
      q[j] = 0;
      if (j < per && p < m) {
        const uint32_t kj = sk[p];
        if (p > 0 && prev < kj) bnd |= 1u << j;
        prev = kj;
        const long long x = eq[sv[p]];
        w[j] = qw_weight(x, wb);
        q[j] = qw_target(x, wb) * w[j];
      }
      tn += w[j];
      ts += q[j];
    }
    unsigned long long sv_[2] = {(unsigned long long)tn, (unsigned long long)ts}, tot[2];
    block_excl_scan_n<kBigBlock, 2>(sv_, tot, scan64);
    long long run_n = carry_n + (long long)sv_[0];
    long long run_s = carry_s + (long long)sv_[1];
    carry_n += (long long)tot[0];
    carry_s += (long long)tot[1];
    float hi[kBigPer];
    unsigned cand = 0;
    float t = bp < 0 ? -FLT_MAX : bg;
    {
      long long rn = run_n, rs = run_s;
#pragma unroll
      for (int j = 0; j < kBigPer; ++j) {
        hi[j] = 0.0f;
        const long long nr = n - rn;
        if (((bnd >> j) & 1u) && rn >= ml && nr >= ml) {
          float lo;
          variance_gain_bounds((int)rn, rs, (int)nr, sum - rs, rc, p2, lo, hi[j]);
          t = fmaxf(t, lo);
          cand |= 1u << j;
        }
        rn += w[j];
        rs += q[j];
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(kFull, t, o));
#pragma unroll
    for (int j = 0; j < kBigPer; ++j) {
      if (((cand >> j) & 1u) && hi[j] >= t) {
        const float g = variance_gain(run_n, run_s, n - run_n, sum - run_s, S);
        if (bp < 0 || g > bg) {
          bg = g;
          bp = p0 + j;
          bnl = run_n;
          bsl = run_s;
        }
      }
      run_n += w[j];
      run_s += q[j];
    }
  }
  *out_g = bg;
  *out_p = bp;
  *out_nl = bnl;
  *out_sl = bsl;
}

template <int CW>
__global__ void __launch_bounds__(kBigBlock, big_ctas_per_sm(CW)) k_rf_big_items(BigArgs b) {
  __shared__ BigSmem S;
  __shared__ float s_g[kBigWarps];
  __shared__ int s_p[kBigWarps];
  __shared__ long long s_prior;
  __shared__ int s_item[2];
  __shared__ int s_nt[kMaxClasses];
  const LevelArgs& a = b.L;
  const int nnodes = b.phase == 1 ? b.nbig : *b.nretry;
  const int nitems = nnodes * b.tries_per_node;
  uint32_t* k1 = b.slot + (long long)blockIdx.x * 4 * b.slot_stride;
  uint32_t* v1 = k1 + b.slot_stride;
  uint32_t* k2 = v1 + b.slot_stride;
  uint32_t* v2 = k2 + b.slot_stride;
  int* ctr = b.item_ctr + (b.phase - 1);
  // Items are handed out one at a time as CTAs become free: nodes differ in
  // size, and a fixed stride over the items left some CTAs with several times
  // the work of others.  The item number alternates between two words, so
  // the next fetch never overwrites a word that a thread may still read.
  for (int round = 0;; ++round) {
    if (threadIdx.x == 0) s_item[round & 1] = atomicAdd(ctr, 1);
    __syncthreads();
    const int it = s_item[round & 1];
    if (it >= nitems) break;
    const int ni = it / b.tries_per_node;
    const int ts = it % b.tries_per_node;
    const int node = b.phase == 1 ? b.big[ni] : b.retry[ni];
    const LNode nd = a.nodes[node];
    const ProbDesc& P = a.probs[nd.prob];
    const int t = b.phase == 1 ? ts : P.n_mand + ts;
    const int slot_node = b.phase == 1 ? ni : b.big_index[node];
    Cand* cout = b.cand + (long long)slot_node * kMaxTries + t;
    if ((b.phase == 1 && ts >= P.n_mand) || (b.phase == 2 && ts >= P.n_opt)) continue;
    const int m = nd.ecnt;
    const int* rows = a.rowsA + nd.ebeg;
    const int* ncnt = a.cnt + (long long)node * a.Cmax;
    const int f = feature_of_try(P, nd, t);
    const float* xf = P.X + (long long)f * P.N;
    if (threadIdx.x == 0 && P.task == 0)
      s_prior = entropy_prior(a.H, nd.n, P.C, [&](int c) { return (long long)ncnt[c]; });
    if (P.task == 0 && threadIdx.x < P.C) s_nt[threadIdx.x] = ncnt[threadIdx.x];
    // keys (and, for classification, the packed label | weight values) with
    // eight gathers in flight per thread; the keys' OR / AND and the digit
    // histograms of their significant bytes on the way
    const bool packed = P.task == 0;
    const uint32_t* pv = b.pv ? b.pv + nd.ebeg : nullptr;
    const uint32_t* rk = P.rank ? P.rank + (long long)f * P.N : nullptr;
    const int nbytes = rk ? (32 - __clz(max(1ll, P.N - 1)) + 7) >> 3 : 4;
    // packed keys (rank << pb | label << wb | weight) when the three fit one
    // word: the sort then moves one word per entry instead of a key and a
    // value, and the scan reads one
    int wb = 0, pb = 0;
    bool pk = false;
    if constexpr (CW >= 2 && CW <= 5) {
      if (packed && rk && pv) {
        wb = 32 - __clz(max(1, *b.maxw));
        pb = wb + (32 - __clz(max(1, P.C - 1)));
        pk = (32 - __clz((int)max(1ll, P.N - 1))) + pb <= 32;
      }
    }
    for (int i = threadIdx.x; i < 4 * 256; i += kBigBlock) (&S.dh[0][0])[i] = 0;
    __syncthreads();
    unsigned o = 0, an = 0xFFFFFFFFu;
    for (int base = 0; base < m; base += kBigTile) {
      int rr[kBigPer];
#pragma unroll
      for (int j = 0; j < kBigPer; ++j) {
        const int i = base + j * kBigBlock + threadIdx.x;
        rr[j] = i < m ? __ldg(rows + i) : 0;
      }
#pragma unroll
      for (int j = 0; j < kBigPer; ++j) {
        const int i = base + j * kBigBlock + threadIdx.x;
        const bool act = i < m;
        uint32_t k = 0;
        if (act) {
          k = rk ? __ldg(rk + rr[j]) : orderable(__ldg(xf + rr[j]));
          if (pk) {
            const uint32_t pvi = __ldg(pv + i);
            k1[i] = (k << pb) | ((pvi >> 27) << wb) | (pvi & 0x7FFFFFFu);
          } else {
            k1[i] = k;
          }
          o |= k;
          an &= k;
        }
        // lower bytes vary across the node's keys: plain atomics; the top byte
        // may be one value for the whole round (one atomic for the round)
        for (int d = 0; d + 1 < nbytes; ++d)
          if (act) atomicAdd(&S.dh[d][(k >> (8 * d)) & 255u], 1u);
        hist_add_round(S.dh[nbytes - 1], (k >> (8 * (nbytes - 1))) & 255u, act);
      }
    }
#pragma unroll
    for (int sh = 16; sh > 0; sh >>= 1) {
      o |= __shfl_xor_sync(kFull, o, sh);
      an &= __shfl_xor_sync(kFull, an, sh);
    }
    if ((threadIdx.x & 31) == 0) {
      S.red[2 * (threadIdx.x >> 5)] = o;
      S.red[2 * (threadIdx.x >> 5) + 1] = an;
    }
    __syncthreads();
    unsigned diff;
    {
      unsigned oo = 0, aa = 0xFFFFFFFFu;
#pragma unroll
      for (int w = 0; w < kBigWarps; ++w) {
        oo |= S.red[2 * w];
        aa &= S.red[2 * w + 1];
      }
      diff = oo ^ aa;
    }
    // S.red is written again only after the sort's and the scan's barriers.
    // The values (packed label and weight, or the entry index for regression)
    // enter with the first pass; keys that are all equal need no pass and
    // have their values copied.
    bool in2 = false;
    if (pk) {
      if (diff != 0) in2 = big_sort_keys(k1, k2, m, diff, pb, S);
    } else if (diff != 0) {
      in2 = big_sort(k1, v1, k2, v2, packed ? pv : nullptr, m, diff, S);
    } else {
      for (int i = threadIdx.x; i < m; i += kBigBlock) v1[i] = packed ? pv[i] : (uint32_t)i;
      __syncthreads();
    }
    const uint32_t* sk = in2 ? k2 : k1;
    const uint32_t* sv = in2 ? v2 : v1;
    float g;
    int p;
    long long nl, sl = 0;
    unsigned long long L[CW];
    if (packed) {
      if constexpr (CW >= 2 && CW <= 5) {
        static_assert((2 * CW + 1) * (kColStride + 1) <= 2 * kBigTile, "columns fit the tiles");
        if (pk)
          big_boundary_cols<CW, true>(sk, sv, m, kBigPer, nd, P.C, max(1, P.min_leaf), pb, wb,
                                      a.H, s_prior, s_nt, S.tile, &g, &p, &nl, L);
        else
          big_boundary_cols<CW, false>(sk, sv, m, kBigPer, nd, P.C, max(1, P.min_leaf), 0, 0,
                                       a.H, s_prior, s_nt, S.tile, &g, &p, &nl, L);
      } else {
        big_boundary_items<CW>(sk, sv, m, nd, P, ncnt, a.H, s_prior, S.scan64, &g, &p, &nl, L);
      }
    } else {
      big_boundary_reg(sk, sv, b.pq + nd.ebeg, m, kBigPer, nd.n, nd.sum, max(1, P.min_leaf), P.S,
                       P.N, S.scan64, &g, &p, &nl, &sl);
#pragma unroll
      for (int c = 0; c < CW; ++c) L[c] = 0;
    }
    const int bp = block_best_pos<kBigBlock>(g, p, s_g, s_p);
    if (bp >= 0 && p == bp) {
      Cand c;
      c.valid = 1;
      c.gain = g;
      c.f = f;
      // the values on both sides of the boundary (-0 reads back as +0, which
      // gives the same threshold)
      const uint32_t ka = pk ? sk[bp - 1] >> pb : sk[bp - 1];
      const uint32_t kb = pk ? sk[bp] >> pb : sk[bp];
      const float xa = packed ? key_value(P, f, ka) : __ldg(xf + __ldg(rows + sv[bp - 1]));
      const float xb = packed ? key_value(P, f, kb) : __ldg(xf + __ldg(rows + sv[bp]));
      c.thr = midpoint_threshold(xa, xb);
      c.nl_e = bp;
      c.nl = (int)nl;
      c.suml = sl;
      *cout = c;
      if (P.task == 0) {
        int* lo = b.candL + ((long long)slot_node * kMaxTries + t) * a.Cmax;
        for (int cc = 0; cc < P.C; ++cc) lo[cc] = (int)packed_get<CW>(L, cc);
      }
    }
    if (bp < 0 && threadIdx.x == 0) {
      Cand c;
      c.valid = 0;
      c.gain = -FLT_MAX;
      c.f = f;
      c.thr = 0.0f;
      c.nl_e = c.nl = 0;
      c.suml = 0;
      *cout = c;
    }
    if (threadIdx.x == 0) {
      atomicAdd((unsigned long long*)&a.stats[2], (unsigned long long)m);
      if (b.phase == 1 && ts == 0) atomicAdd((unsigned long long*)&a.stats[3], (unsigned long long)m);
    }
    __syncthreads();
  }
}

// Try loop per big node.  Phase 1: best of the mandatory tries; nodes whose
// best is not sensible (and that have optional tries) go to the retry list,
// the others are decided.  Phase 2: optional tries in order until one is
// sensible.  Decided nodes write their result and partition their entries.
template <int CW>
__global__ void __launch_bounds__(kBigBlock) k_rf_big_decide(BigArgs b) {
  __shared__ Cand s_best;
  __shared__ int s_bestL[kMaxClasses];
  __shared__ int s_act;
  __shared__ int s_scan[kBigWarps];
  const LevelArgs& a = b.L;
  const int nnodes = b.phase == 1 ? b.nbig : *b.nretry;
  for (int ni = blockIdx.x; ni < nnodes; ni += gridDim.x) {
    const int node = b.phase == 1 ? b.big[ni] : b.retry[ni];
    const int bi = b.phase == 1 ? ni : b.big_index[node];
    const LNode nd = a.nodes[node];
    const ProbDesc& P = a.probs[nd.prob];
    const Cand* cs = b.cand + (long long)bi * kMaxTries;
    const int* cL = b.candL + (long long)bi * kMaxTries * a.Cmax;
    if (threadIdx.x == 0) {
      int from = -1;
      if (b.phase == 1) {
        Cand best = cs[0];
        from = 0;
        for (int t = 1; t < P.n_mand; ++t)
          if (better(cs[t], best)) {
            best = cs[t];
            from = t;
          }
        b.big_index[node] = ni;
        if (P.n_opt > 0 && !(best.valid && best.gain >= kSensible)) {
          b.partial[ni] = best;
          for (int c = 0; c < P.C; ++c)
            b.partialL[(long long)ni * a.Cmax + c] = P.task == 0 ? cL[from * a.Cmax + c] : 0;
          b.retry_out[atomicAdd(b.nretry_out, 1)] = node;
          s_act = 0;
        } else {
          s_best = best;
          if (P.task == 0)
            for (int c = 0; c < P.C; ++c) s_bestL[c] = cL[from * a.Cmax + c];
          s_act = 1;
        }
      } else {
        Cand best = b.partial[bi];
        const int* pl = b.partialL + (long long)bi * a.Cmax;
        int bestL_src = -1;
        for (int j = 0; j < P.n_opt; ++j) {
          const Cand& c = cs[P.n_mand + j];
          if (better(c, best)) {
            best = c;
            bestL_src = P.n_mand + j;
          }
          if (c.valid && c.gain >= kSensible) break;
        }
        s_best = best;
        if (P.task == 0)
          for (int c = 0; c < P.C; ++c)
            s_bestL[c] = bestL_src < 0 ? pl[c] : cL[bestL_src * a.Cmax + c];
        s_act = 1;
      }
    }
    __syncthreads();
    if (s_act) {
      const Cand bb = s_best;
      if (!bb.valid) {
        if (threadIdx.x == 0) write_leaf(a.res, node);
      } else {
        if (threadIdx.x == 0)
          write_result(a.res, a.res_cnt, a.Cmax, node, bb, P.task == 0 ? s_bestL : nullptr, P.C);
        cta_partition<kBigBlock>(a.rowsA, a.wA, a.rowsB, a.wB, nd.ebeg, nd.ecnt, bb.nl_e,
                                 P.X + (long long)bb.f * P.N, bb.thr, s_scan);
      }
    }
    __syncthreads();
  }
}

// RF node of 257 .. a.smem_cap (<= SMEM_CAP) entries in one CTA.  The node's
// row ids and packed (label << 27 | weight) values are read into shared memory
// once per node; each try gathers the feature's keys (reducing their varying
// bits on the way), sorts the (key, value) pairs in shared memory and scans
// the boundaries with ceil(m / 256) consecutive elements per thread.
// Dynamic shared memory, 24 bytes per entry of a.smem_cap:
//   classification: k1 v1 k2 v2 (sort buffers), row ids, packed values;
//   regression:     k1 v1 k2 v2, packed (target, weight) words (8 bytes).
template <int CW, int SMEM_CAP>
__global__ void __launch_bounds__(kBigBlock, smem_ctas_per_sm(CW)) k_rf_smem(LevelArgs a) {
  __shared__ SortSmem<kBigBlock> SS;
  __shared__ unsigned red[2 * kBigWarps];
  __shared__ unsigned long long scan64[kBigWarps * (CW + 1)];
  __shared__ float s_g[kBigWarps];
  __shared__ int s_p[kBigWarps];
  __shared__ Cand s_cand, s_best;
  __shared__ int s_candL[kMaxClasses], s_bestL[kMaxClasses];
  __shared__ long long s_prior;
  __shared__ int s_scan[kBigWarps];
  __shared__ int s_next;
  __shared__ int s_nt[kMaxClasses];
  extern __shared__ __align__(16) unsigned char dsm[];
  const int cap = a.smem_cap;
  uint32_t* k1 = (uint32_t*)dsm;
  uint32_t* v1 = k1 + cap;
  uint32_t* k2 = k1 + 2 * cap;
  uint32_t* v2 = k1 + 3 * cap;
  int* s_rows = (int*)(k1 + 4 * cap);
  uint32_t* s_pv = k1 + 5 * cap;
  long long* q_e = (long long*)(k1 + 4 * cap);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int wi = blockIdx.x; wi < a.nwork; wi += gridDim.x) {
    const int node = a.work[wi];
    const LNode nd = a.nodes[node];
    const ProbDesc& P = a.probs[nd.prob];
    const int C = P.C;
    const int m = nd.ecnt;
    const int per = min(kBigPer, (m + kBigBlock - 1) / kBigBlock);
    const int* rows = a.rowsA + nd.ebeg;
    const int* wts = a.wA ? a.wA + nd.ebeg : nullptr;
    const int* ncnt = a.cnt + (long long)node * a.Cmax;
    const bool packed = P.task == 0;
    if (packed) {
      for (int i = threadIdx.x; i < m; i += kBigBlock) {
        const int row = __ldg(rows + i);
        s_rows[i] = row;
        s_pv[i] = ((uint32_t)__ldg(P.lab + row) << 27) | (uint32_t)(wts ? __ldg(wts + i) : 1);
      }
    } else {
      const int wb = qw_bits(P.N);
      for (int i = threadIdx.x; i < m; i += kBigBlock)
        q_e[i] = qw_pack(__ldg(P.q + __ldg(rows + i)), wts ? __ldg(wts + i) : 1, wb);
    }
    if (threadIdx.x == 0 && packed)
      s_prior = entropy_prior(a.H, nd.n, C, [&](int c) { return (long long)ncnt[c]; });
    if (packed && threadIdx.x < C) s_nt[threadIdx.x] = ncnt[threadIdx.x];
    __syncthreads();
    int t = 0;
    while (true) {
      const int f = feature_of_try(P, nd, t);
      const float* xf = P.X + (long long)f * P.N;
      const uint32_t* rk = P.rank ? P.rank + (long long)f * P.N : nullptr;
      unsigned o = 0, an = 0xFFFFFFFFu;
      if (packed) {
        for (int i = threadIdx.x; i < m; i += kBigBlock) {
          const int row = s_rows[i];
          const uint32_t k = rk ? __ldg(rk + row) : orderable(__ldg(xf + row));
          k1[i] = k;
          v1[i] = s_pv[i];
          o |= k;
          an &= k;
        }
      } else {
        for (int i = threadIdx.x; i < m; i += kBigBlock) {
          const int row = __ldg(rows + i);
          const uint32_t k = rk ? __ldg(rk + row) : orderable(__ldg(xf + row));
          k1[i] = k;
          v1[i] = (uint32_t)i;
          o |= k;
          an &= k;
        }
      }
#pragma unroll
      for (int sh = 16; sh > 0; sh >>= 1) {
        o |= __shfl_xor_sync(kFull, o, sh);
        an &= __shfl_xor_sync(kFull, an, sh);
      }
      if (lane == 0) {
        red[2 * warp] = o;
        red[2 * warp + 1] = an;
      }
      __syncthreads();
      unsigned diff;
      {
        unsigned oo = 0, aa = 0xFFFFFFFFu;
#pragma unroll
        for (int w = 0; w < kBigWarps; ++w) {
          oo |= red[2 * w];
          aa &= red[2 * w + 1];
        }
        diff = oo ^ aa;
      }
      // red is written again only after the sort's and the scan's barriers
      const bool in2 = cta_radix_sort_diff<kBigBlock>(k1, v1, k2, v2, m, diff, SS);
      const uint32_t* sk = in2 ? k2 : k1;
      const uint32_t* sv = in2 ? v2 : v1;
      float g;
      int p;
      long long nl, sl = 0;
      unsigned long long L[CW];
      bool cols_scan = false;
      if constexpr (CW >= 2 && CW <= 5) cols_scan = (C + 1) * (kColStride + 1) <= 2 * cap;
      if (packed && cols_scan) {
        // the class columns in the sort buffers the sorted pairs are not in
        big_boundary_cols<CW, false>(sk, sv, m, per, nd, C, max(1, P.min_leaf), 0, 0, a.H,
                                     s_prior, s_nt, in2 ? k1 : k2, &g, &p, &nl, L);
      } else if (packed) {
        big_boundary<CW, false>(sk, sv, m, per, nd, P, ncnt, a.H, s_prior, scan64, &g, &p, &nl, L);
      } else {
        big_boundary_reg(sk, sv, q_e, m, per, nd.n, nd.sum, max(1, P.min_leaf), P.S, P.N, scan64,
                         &g, &p, &nl, &sl);
#pragma unroll
        for (int c = 0; c < CW; ++c) L[c] = 0;
      }
      const int bp = block_best_pos<kBigBlock>(g, p, s_g, s_p);
      if (bp >= 0 && p == bp) {
        Cand c;
        c.valid = 1;
        c.gain = g;
        c.f = f;
        const float xa = packed ? key_value(P, f, sk[bp - 1]) : __ldg(xf + __ldg(rows + sv[bp - 1]));
        const float xb = packed ? key_value(P, f, sk[bp]) : __ldg(xf + __ldg(rows + sv[bp]));
        c.thr = midpoint_threshold(xa, xb);
        c.nl_e = bp;
        c.nl = (int)nl;
        c.suml = sl;
        s_cand = c;
        if (packed)
          for (int cc = 0; cc < C; ++cc) s_candL[cc] = (int)packed_get<CW>(L, cc);
      }
      if (bp < 0 && threadIdx.x == 0) {
        Cand c;
        c.valid = 0;
        c.gain = -FLT_MAX;
        c.f = f;
        c.thr = 0.0f;
        c.nl_e = c.nl = 0;
        c.suml = 0;
        s_cand = c;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        bool next;
        if (t < P.n_mand) {
          if (t == 0 || better(s_cand, s_best)) {
            s_best = s_cand;
            if (packed)
              for (int c = 0; c < C; ++c) s_bestL[c] = s_candL[c];
          }
          next = (t + 1 < P.n_mand) || (P.n_opt > 0 && !(s_best.valid && s_best.gain >= kSensible));
        } else {
          if (better(s_cand, s_best)) {
            s_best = s_cand;
            if (packed)
              for (int c = 0; c < C; ++c) s_bestL[c] = s_candL[c];
          }
          next = !(s_cand.valid && s_cand.gain >= kSensible) && (t + 1 < P.n_mand + P.n_opt);
        }
        s_next = next ? 1 : 0;
      }
      __syncthreads();
      const bool stop = s_next == 0;
      __syncthreads();
      ++t;
      if (stop) break;
    }
    const Cand b = s_best;
    if (threadIdx.x == 0) {
      atomicAdd((unsigned long long*)&a.stats[2], (unsigned long long)t * m);
      atomicAdd((unsigned long long*)&a.stats[3], (unsigned long long)m);
    }
    if (!b.valid) {
      if (threadIdx.x == 0) write_leaf(a.res, node);
    } else {
      if (threadIdx.x == 0)
        write_result(a.res, a.res_cnt, a.Cmax, node, b, packed ? s_bestL : nullptr, C);
      cta_partition<kBigBlock>(a.rowsA, a.wA, a.rowsB, a.wB, nd.ebeg, m, b.nl_e,
                               P.X + (long long)b.f * P.N, b.thr, s_scan);
    }
    __syncthreads();
  }
}

}  // namespace dml
