// Dense ranks of every feature's values, computed once per RF fit.
//
// rank[f * N + i] is the number of distinct values of feature f below x[f][i]
// (values compared as orderable keys, so -0 and +0 share a rank) and
// vals[f * N + r] is the value of rank r.  Sorting a node's entries by rank is
// sorting them by value, but a rank has only ceil(log2(distinct)) significant
// bits, so the split-search radix sorts skip the constant upper digits: three
// 8-bit passes instead of four for a million distinct values, one for a
// feature of 16 integer values.  The threshold of a boundary is read back from
// vals.  One device radix sort (CUB, run once per fit, not on the search path)
// orders (feature, key) pairs; one block per feature then scans its run.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>

#include "dml_device.cuh"
#include "engine.h"

namespace dml {

namespace {

__global__ void k_rank_keys(const float* __restrict__ X, long long N, long long n,
                            unsigned long long* __restrict__ keys, int* __restrict__ rows) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long f = i / N;
    keys[i] = ((unsigned long long)f << 32) | orderable(X[i]);
    rows[i] = (int)(i - f * N);
  }
}

// One block per feature: distinct-value flags, running inclusive scan.
__global__ void __launch_bounds__(1024) k_rank_scan(const unsigned long long* __restrict__ keys,
                                                    const int* __restrict__ rows, long long N,
                                                    uint32_t* __restrict__ rank,
                                                    float* __restrict__ vals) {
  __shared__ int wsum[32];
  const long long base = (long long)blockIdx.x * N;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long running = 0;  // distinct values before this chunk
  for (long long c0 = 0; c0 < N; c0 += 1024) {
    const long long i = c0 + threadIdx.x;
    const bool in = i < N;
    const uint32_t k = in ? (uint32_t)keys[base + i] : 0u;
    const int flag = in && (i == 0 || (uint32_t)keys[base + i - 1] != k) ? 1 : 0;
    int x = flag;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    int before = 0, total = 0;
    for (int k2 = 0; k2 < 32; ++k2) {
      const int v = wsum[k2];
      if (k2 < w) before += v;
      total += v;
    }
    if (in) {
      const long long r = running + before + x - 1;  // rank of element i
      rank[base + rows[base + i]] = (uint32_t)r;
      if (flag) vals[base + r] = from_orderable(k);
    }
    running += total;
    __syncthreads();
  }
}

}  // namespace

// Fills rank / vals ([F * N] each) on stream s; false if the temporary
// memory could not be had (the caller then sorts raw keys).
bool compute_ranks(const float* X, long long N, int F, uint32_t* rank, float* vals,
                   cudaStream_t s) {
  const long long n = N * F;
  if (n >= (1ll << 31)) return false;
  int fbits = 1;
  while ((1ll << fbits) < F) ++fbits;
  unsigned long long *k_in = nullptr, *k_out = nullptr;
  int *r_in = nullptr, *r_out = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, k_in, k_out, r_in, r_out, (int)n, 0,
                                  32 + fbits, s);
  bool ok = true;
  try {
    k_in = (unsigned long long*)dev_alloc(sizeof(unsigned long long) * n, s);
    k_out = (unsigned long long*)dev_alloc(sizeof(unsigned long long) * n, s);
    r_in = (int*)dev_alloc(sizeof(int) * n, s);
    r_out = (int*)dev_alloc(sizeof(int) * n, s);
    tmp = dev_alloc(tmp_bytes, s);
  } catch (const CudaError&) {
    ok = false;
  }
  if (ok) {
    const int grid = (int)std::min<long long>(8192, (n + 255) / 256);
    k_rank_keys<<<grid, 256, 0, s>>>(X, N, n, k_in, r_in);
    ok = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, r_in, r_out, (int)n, 0,
                                         32 + fbits, s) == cudaSuccess;
    if (ok) k_rank_scan<<<F, 1024, 0, s>>>(k_out, r_out, N, rank, vals);
    ok = ok && cudaGetLastError() == cudaSuccess;
  }
  dev_free(k_in, s);
  dev_free(k_out, s);
  dev_free(r_in, s);
  dev_free(r_out, s);
  dev_free(tmp, s);
  return ok;
}

}  // namespace dml
