// The bag of each RF tree: bootstrap draws shared by the fit (multiplicities
// become entry weights) and the out-of-bag estimate (rows never drawn).
//
// Plain bootstrap (gpurf.cu:101-113 with keyed draws): draw i of tree t picks
// row (word i&3 of Philox(seed; i>>2, i>>34, t, kTagBoot)) % N, i in [0, N).
// Balanced bootstrap, the reference's easy ensemble (gpurf.cu:73-100, whose
// class ranges target_starts are never filled there): for every class c with
// n_c > 0 rows, N / C draws pick rows of that class uniformly with
// replacement: draw i = c * (N / C) + j takes row class_rows[off_c + word % n_c]
// of Philox(seed; i>>2, i>>34, t, kTagBalanced); empty classes draw nothing.
#pragma once
#include "dml_device.cuh"
#include "dml_internal.h"

namespace dml {

__device__ __forceinline__ long long bag_draws(const ProbDesc& P) {
  return P.balanced ? (long long)P.C * P.bal_m : P.N;
}

// Row of draw i of tree t (tree index within the forest), or -1 (no row).
__device__ __forceinline__ long long bag_draw(const ProbDesc& P, int t, long long i) {
  const uint32_t tree = (uint32_t)(t + P.tree_key0);
  if (!P.balanced) {
    U4 r = keyed(P.seed, kTagBoot, 0, tree, (uint32_t)(i >> 2), (uint32_t)(i >> 34));
    return pick(r, (int)(i & 3)) % (uint32_t)P.N;
  }
  const long long c = i / P.bal_m;
  const long long beg = P.class_off[c], nc = P.class_off[c + 1] - beg;
  if (nc == 0) return -1;
  U4 r = keyed(P.seed, kTagBalanced, 0, tree, (uint32_t)(i >> 2), (uint32_t)(i >> 34));
  return P.class_rows[beg + pick(r, (int)(i & 3)) % (uint32_t)nc];
}

// err |= 1 unless every target is an integer class in [0, C).
static __global__ void k_check_labels(const float* __restrict__ y, long long N, int C, int* err) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = y[i];
    if (!(v >= 0.0f && v < (float)C && v == floorf(v))) atomicOr(err, 1);
  }
}

// Per-class row lists of a classification target vector (class index as float,
// checked by k_check_labels or the fit's validation first).
static __global__ void k_class_count(const float* __restrict__ y, long long N, long long* counts) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x)
    atomicAdd((unsigned long long*)&counts[(int)y[i]], 1ull);
}

// counts[0..C) -> exclusive offsets off[0..C] (in place, one thread)
static __global__ void k_class_offsets(long long* off, int C) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  long long acc = 0;
  for (int c = 0; c < C; ++c) {
    long long n = off[c];
    off[c] = acc;
    acc += n;
  }
  off[C] = acc;
}

// One block per class: a stable compaction of the rows of class blockIdx.x.
static __global__ void __launch_bounds__(1024) k_class_rows(const float* __restrict__ y,
                                                            long long N,
                                                            const long long* __restrict__ off,
                                                            int* __restrict__ rows) {
  __shared__ int wsum[32];
  const int c = blockIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long base = off[c];
  for (long long i0 = 0; i0 < N; i0 += 1024) {
    const long long i = i0 + threadIdx.x;
    const bool mine = i < N && (int)y[i] == c;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, mine);
    if (lane == 0) wsum[w] = __popc(m);
    __syncthreads();
    int before = 0, total = 0;
    for (int k = 0; k < 32; ++k) {
      const int v = wsum[k];
      if (k < w) before += v;
      total += v;
    }
    if (mine) rows[base + before + __popc(m & ((1u << lane) - 1u))] = (int)i;
    base += total;
    __syncthreads();
  }
}

}  // namespace dml
