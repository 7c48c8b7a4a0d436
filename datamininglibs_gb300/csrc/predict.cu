// Forest prediction and the forest handle entry points.
//
// Replaces GpuDteAlgorithm<T>::Predict (lib_ensembles/source/gpudte_algorithm.cc:
// 270-331) and gpudte_predict (lib_ensembles/source/gpudte.cu:311-359): the
// reference launches one thread per (tree, row), in chunks of 65,536 with a
// device sync each, and adds every vote to global memory with an atomic.  Here
// a thread owns a row for all trees: it walks each tree over the 16-byte
// predict layout (leaf votes precomputed), counts votes in shared memory and
// writes its row once.  Tree order is fixed, so regression sums are
// deterministic.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "dml_device.cuh"
#include "engine.h"

namespace dml {

const char* last_error_str();
void clear_error();
void init_pool_once();

constexpr int kPredBlock = 128;
constexpr int kWalk = 4;  // trees walked in lockstep per thread

// Rows are walked through all trees, four at a time; a tile of the row's
// features is not staged because each row reads only the features on its
// paths.
template <int TASK>
__global__ void __launch_bounds__(kPredBlock) k_predict(const PNode* __restrict__ nodes,
                                                        int n_trees, int C,
                                                        const float* __restrict__ X, long long N,
                                                        float* __restrict__ out) {
  extern __shared__ int votes[];  // [kPredBlock][C]
  const long long row = (long long)blockIdx.x * kPredBlock + threadIdx.x;
  const bool act = row < N;
  int* my = votes + threadIdx.x * C;
  if (TASK == 0)
    for (int c = 0; c < C; ++c) my[c] = 0;
  float acc = 0.0f;
  if (act) {
    auto xr = [&](int f) { return __ldg(X + (long long)f * N + row); };
    // kWalk trees in lockstep (kWalk loads in flight), then the rest one by
    // one; leaves are consumed in tree order, so regression sums keep it
    int t = 0;
    for (; t + kWalk <= n_trees; t += kWalk) {
      int4 lf[kWalk];
      walk_trees<kWalk>(nodes, t, xr, lf);
#pragma unroll
      for (int k = 0; k < kWalk; ++k) {
        if (TASK == 0)
          my[lf[k].y] += 1;
        else
          acc = __fadd_rn(acc, __int_as_float(lf[k].z));
      }
    }
    for (; t < n_trees; ++t) {
      int4 lf[1];
      walk_trees<1>(nodes, t, xr, lf);
      if (TASK == 0)
        my[lf[0].y] += 1;
      else
        acc = __fadd_rn(acc, __int_as_float(lf[0].z));
    }
    if (TASK == 0) {
      for (int c = 0; c < C; ++c) out[row * C + c] = (float)my[c];
    } else {
      out[row] = acc;
    }
  }
}

// Bulk predict in passes over blocks of trees.  A forest larger than L2 (the
// 128-tree, 1M-row forest is 692 MB) walked by many row tiles at once touches
// every tree's nodes at the same time, so almost every visit of a deep node is
// a DRAM miss.  In passes, every CTA of a launch walks the same block of trees,
// sized to sit well inside L2; node loads carry an L2 evict-last policy and
// the streamed rows evict-first, so a pass's nodes come from DRAM about once.
__device__ __forceinline__ unsigned long long l2_policy_evict_last() {
  unsigned long long p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ unsigned long long l2_policy_evict_first() {
  unsigned long long p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ int4 ld_node(const int4* p, unsigned long long pol) {
  int4 v;
  asm("ld.global.nc.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
      : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ float ld_stream(const float* p, unsigned long long pol) {
  float v;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}

// Rows in tiles of 16, their features staged in shared memory (a row reads
// one feature per node on its paths: from global memory those reads scatter
// over the whole sample matrix), 8 threads per row walking trees g, g + 8, ...
// four in lockstep.  Votes meet in shared memory (integer counts, order-free);
// regression keeps each tree's leaf value and one thread sums them in tree
// order, as k_predict does.
constexpr int kPSplit = 8;
constexpr int kPRows = kPredBlock / kPSplit;  // 16
// a feature's 16 rows, padded to 17 floats: lanes reading different features
// of one row meet different banks
constexpr int kPStride = kPRows + 1;

template <int TASK>
__global__ void __launch_bounds__(kPredBlock) k_predict_split(const PNode* __restrict__ nodes,
                                                              int t0, int t1, int first, int C,
                                                              int F, const float* __restrict__ X,
                                                              long long N, float* __restrict__ out) {
  extern __shared__ float psm[];  // xs [F][kPStride], then votes [kPRows][C] or values [kPRows][t1 - t0]
  const long long row0 = (long long)blockIdx.x * kPRows;
  const int rows = N - row0 < kPRows ? (int)(N - row0) : kPRows;
  const int g = threadIdx.x % kPSplit;
  const int r = threadIdx.x / kPSplit;
  const int nt = t1 - t0;
  const unsigned long long keep = l2_policy_evict_last();
  const unsigned long long stream = l2_policy_evict_first();
  float* xs = psm;
  for (int e = threadIdx.x; e < F * kPRows; e += kPredBlock) {
    const int f = e / kPRows, rr = e % kPRows;
    xs[f * kPStride + rr] = rr < rows ? ld_stream(X + (long long)f * N + row0 + rr, stream) : 0.0f;
  }
  int* votes = reinterpret_cast<int*>(psm + F * kPStride);
  float* vals = psm + F * kPStride + r * nt;
  if (TASK == 0)
    for (int i = threadIdx.x; i < kPRows * C; i += kPredBlock) votes[i] = 0;
  __syncthreads();
  if (r < rows) {
    const int4* nd = reinterpret_cast<const int4*>(nodes);
    // trees k, k + 8, k + 16, k + 24 in lockstep (four node loads in flight)
    for (int k0 = t0 + g; k0 < t1; k0 += 4 * kPSplit) {
      int4 lf[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = k0 + j * kPSplit;
        lf[j] = k < t1 ? ld_node(nd + k, keep) : make_int4(-1, 0, 0, 0);
      }
      bool more = true;
      while (more) {
        more = false;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (lf[j].x >= 0) {
            lf[j] = ld_node(nd + (goes_left(xs[lf[j].y * kPStride + r], __int_as_float(lf[j].z))
                                      ? lf[j].x
                                      : lf[j].x + 1),
                            keep);
            more = more || lf[j].x >= 0;
          }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = k0 + j * kPSplit;
        if (k < t1) {
          if (TASK == 0)
            atomicAdd(&votes[r * C + lf[j].y], 1);
          else
            vals[k - t0] = __int_as_float(lf[j].z);
        }
      }
    }
  }
  __syncthreads();
  if (r < rows) {
    const long long row = row0 + r;
    if (TASK == 0) {
      for (int c = g; c < C; c += kPSplit) {
        const float v = (float)votes[r * C + c];
        out[row * C + c] = first ? v : __fadd_rn(out[row * C + c], v);
      }
    } else if (g == 0) {
      // the pass's trees added one at a time in tree order onto the sum of
      // the earlier passes: the same float additions as one pass
      float sum = first ? 0.0f : out[row];
      for (int t = 0; t < nt; ++t) sum = __fadd_rn(sum, vals[t]);
      out[row] = sum;
    }
  }
}

// k_predict_split over the compact 8-byte layout (PNode8): the same walk,
// tiles and vote order, half the bytes per node load.
__device__ __forceinline__ uint2 ld_node8(const uint2* p, unsigned long long pol) {
  uint2 v;
  asm("ld.global.nc.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(v.x), "=r"(v.y) : "l"(p), "l"(pol));
  return v;
}

template <int TASK>
__global__ void __launch_bounds__(kPredBlock) k_predict_split8(const PNode8* __restrict__ nodes,
                                                               int fbits, int t0, int t1, int first,
                                                               int C, int F,
                                                               const float* __restrict__ X,
                                                               long long N, float* __restrict__ out) {
  extern __shared__ float psm[];  // as k_predict_split
  const long long row0 = (long long)blockIdx.x * kPRows;
  const int rows = N - row0 < kPRows ? (int)(N - row0) : kPRows;
  const int g = threadIdx.x % kPSplit;
  const int r = threadIdx.x / kPSplit;
  const int nt = t1 - t0;
  const uint32_t fmask = (1u << fbits) - 1u;
  const unsigned long long keep = l2_policy_evict_last();
  const unsigned long long stream = l2_policy_evict_first();
  float* xs = psm;
  for (int e = threadIdx.x; e < F * kPRows; e += kPredBlock) {
    const int f = e / kPRows, rr = e % kPRows;
    xs[f * kPStride + rr] = rr < rows ? ld_stream(X + (long long)f * N + row0 + rr, stream) : 0.0f;
  }
  int* votes = reinterpret_cast<int*>(psm + F * kPStride);
  float* vals = psm + F * kPStride + r * nt;
  if (TASK == 0)
    for (int i = threadIdx.x; i < kPRows * C; i += kPredBlock) votes[i] = 0;
  __syncthreads();
  if (r < rows) {
    const uint2* nd = reinterpret_cast<const uint2*>(nodes);
    for (int k0 = t0 + g; k0 < t1; k0 += 4 * kPSplit) {
      uint2 lf[4];
      long long at[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = k0 + j * kPSplit;
        at[j] = k;
        lf[j] = k < t1 ? ld_node8(nd + k, keep) : make_uint2(fmask, 0u);
      }
      bool more = true;
      while (more) {
        more = false;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if ((lf[j].x & fmask) != fmask) {
            const bool left =
                goes_left(xs[(lf[j].x & fmask) * kPStride + r], __uint_as_float(lf[j].y));
            at[j] += (long long)(lf[j].x >> fbits) + (left ? 0 : 1);
            lf[j] = ld_node8(nd + at[j], keep);
            more = more || (lf[j].x & fmask) != fmask;
          }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = k0 + j * kPSplit;
        if (k < t1) {
          if (TASK == 0)
            atomicAdd(&votes[r * C + (int)(lf[j].x >> fbits)], 1);
          else
            vals[k - t0] = __uint_as_float(lf[j].y);
        }
      }
    }
  }
  __syncthreads();
  if (r < rows) {
    const long long row = row0 + r;
    if (TASK == 0) {
      for (int c = g; c < C; c += kPSplit) {
        const float v = (float)votes[r * C + c];
        out[row * C + c] = first ? v : __fadd_rn(out[row * C + c], v);
      }
    } else if (g == 0) {
      float sum = first ? 0.0f : out[row];
      for (int t = 0; t < nt; ++t) sum = __fadd_rn(sum, vals[t]);
      out[row] = sum;
    }
  }
}

// Trees per pass: the pass's share of the predict nodes within kPassNodes
// nodes (or DML_PREDICT_PASS_MB megabytes of them).  On the 128-tree forest
// of the 1M x 128, 10-class fit (43 M nodes, predicting its 1M rows) 16
// trees a pass (5.4 M nodes) were fastest with either layout: 8
// trees 105.8, 16 trees 116.6, 24 trees 106.7 M rows/s with 16-byte nodes;
// 16 trees 144.2, 32 trees 127.8, 64 trees 130.1 M rows/s with 8-byte ones.
constexpr long long kPassNodes = 6ll << 20;
int predict_pass_trees(const dml_forest* f, long long node_bytes) {
  const char* e = getenv("DML_PREDICT_PASS_MB");
  const long long budget = e && atoll(e) > 0 ? (atoll(e) << 20) : kPassNodes * node_bytes;
  const long long per_tree = std::max<long long>(1, f->n_nodes * node_bytes /
                                                        std::max(1, f->n_trees));
  long long k = budget / per_tree;
  k = std::max<long long>(kPSplit, (k / kPSplit) * kPSplit);
  return (int)std::min<long long>(k, f->n_trees);
}

// The reference's predict structure (gpudte.cu:311-359): one thread per
// (tree, row) of one tree; votes are added to the output (a launch holds each
// row once, so plain adds keep tree order).
template <int TASK>
__global__ void k_predict_plain(const PNode* __restrict__ nodes, int tree, int C,
                                const float* __restrict__ X, long long N, long long row0,
                                long long rows, float* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  const long long row = row0 + i;
  int4 p = __ldg(reinterpret_cast<const int4*>(nodes) + tree);
  while (p.x >= 0) {
    float x = __ldg(X + (long long)p.y * N + row);
    int nx = goes_left(x, __int_as_float(p.z)) ? p.x : p.x + 1;
    p = __ldg(reinterpret_cast<const int4*>(nodes) + nx);
  }
  if (TASK == 0)
    out[row * C + p.y] = __fadd_rn(out[row * C + p.y], 1.0f);
  else
    out[row] = __fadd_rn(out[row], __int_as_float(p.z));
}

// Rows predicted in passes over blocks of trees from this many rows on (below
// it, one pass over every tree).
constexpr long long kPassMinRows = 1 << 16;

dml_status predict_device(const dml_forest* f, const float* dX, long long n_rows, float* dout,
                          cudaStream_t s) {
  if (n_rows <= 0) return DML_OK;
  const bool cls = f->task == DML_CLASSIFICATION;
  // bulk prediction walks the compact layout (built by the first one) unless
  // DML_PREDICT_NODE16 is set
  const char* n16 = getenv("DML_PREDICT_NODE16");
  const bool compact = n_rows >= kPassMinRows && !(n16 && atoi(n16) != 0);
  if (compact && !f->p8_ready.load(std::memory_order_acquire)) forest_build_pnodes8(f, s);
  const bool use8 = compact && f->pnodes8 != nullptr;
  const int per = n_rows >= kPassMinRows
                      ? predict_pass_trees(f, use8 ? (long long)sizeof(PNode8) : (long long)sizeof(PNode))
                      : f->n_trees;
  // staged rows when the tile (features, votes or per-tree values) fits 48 KB
  const size_t split_sm =
      sizeof(float) * ((size_t)kPStride * f->n_features +
                       (size_t)kPRows * (cls ? f->n_classes : std::min(per, f->n_trees)));
  if (split_sm <= 48 * 1024) {
    const long long tiles = (n_rows + kPRows - 1) / kPRows;
    for (int t0 = 0; t0 < f->n_trees; t0 += per) {
      const int t1 = std::min(f->n_trees, t0 + per);
      if (use8 && cls)
        k_predict_split8<0><<<(unsigned)tiles, kPredBlock, split_sm, s>>>(
            f->pnodes8, f->p8_bits, t0, t1, t0 == 0, f->n_classes, f->n_features, dX, n_rows, dout);
      else if (use8)
        k_predict_split8<1><<<(unsigned)tiles, kPredBlock, split_sm, s>>>(
            f->pnodes8, f->p8_bits, t0, t1, t0 == 0, 1, f->n_features, dX, n_rows, dout);
      else if (cls)
        k_predict_split<0><<<(unsigned)tiles, kPredBlock, split_sm, s>>>(
            f->pnodes, t0, t1, t0 == 0, f->n_classes, f->n_features, dX, n_rows, dout);
      else
        k_predict_split<1><<<(unsigned)tiles, kPredBlock, split_sm, s>>>(
            f->pnodes, t0, t1, t0 == 0, 1, f->n_features, dX, n_rows, dout);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) {
        set_error("predict launch failed: %s", cudaGetErrorString(e));
        return DML_ERR_CUDA;
      }
    }
    return DML_OK;
  }
  const long long blocks = (n_rows + kPredBlock - 1) / kPredBlock;
  if (f->task == DML_CLASSIFICATION) {
    size_t sm = sizeof(int) * kPredBlock * f->n_classes;
    k_predict<0><<<(unsigned)blocks, kPredBlock, sm, s>>>(f->pnodes, f->n_trees, f->n_classes, dX,
                                                          n_rows, dout);
  } else {
    k_predict<1><<<(unsigned)blocks, kPredBlock, 0, s>>>(f->pnodes, f->n_trees, 1, dX, n_rows,
                                                         dout);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("predict launch failed: %s", cudaGetErrorString(e));
    return DML_ERR_CUDA;
  }
  return DML_OK;
}

}  // namespace dml

using namespace dml;

extern "C" {

dml_status dml_predict(const dml_forest* f, const float* samples, int64_t n_rows, float* out,
                       int32_t memory, void* stream) {
  clear_error();
  if (!f || (!samples && n_rows > 0) || (!out && n_rows > 0) || n_rows < 0 ||
      (memory != DML_HOST && memory != DML_DEVICE)) {
    set_error("invalid predict arguments");
    return DML_ERR_INVALID_ARG;
  }
  if (n_rows == 0) return DML_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const long long width = f->task == DML_CLASSIFICATION ? f->n_classes : 1;
  if (memory == DML_DEVICE) {
    dml_status st = predict_device(f, samples, n_rows, out, s);
    return st;
  }
  init_pool_once();
  float* dX = nullptr;
  float* dout = nullptr;
  size_t xb = sizeof(float) * (size_t)n_rows * f->n_features;
  size_t ob = sizeof(float) * (size_t)n_rows * width;
  if (cudaMallocAsync(&dX, xb, s) != cudaSuccess || cudaMallocAsync(&dout, ob, s) != cudaSuccess) {
    cudaGetLastError();
    if (dX) cudaFreeAsync(dX, s);
    set_error("device allocation failed for a predict of %lld rows", (long long)n_rows);
    return DML_ERR_OOM;
  }
  dml_status st = DML_OK;
  if (copy_host_device(dX, samples, xb, true, s) != cudaSuccess) {
    set_error("host to device copy failed");
    st = DML_ERR_CUDA;
  }
  if (st == DML_OK) st = predict_device(f, dX, n_rows, dout, s);
  if (st == DML_OK && copy_host_device(out, dout, ob, false, s) != cudaSuccess) {
    set_error("device to host copy failed");
    st = DML_ERR_CUDA;
  }
  cudaFreeAsync(dX, s);
  cudaFreeAsync(dout, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (st == DML_OK && e != cudaSuccess) {
    set_error("predict failed: %s", cudaGetErrorString(e));
    st = DML_ERR_CUDA;
  }
  return st;
}

dml_status dml_predict_plain(const dml_forest* f, const float* samples, int64_t n_rows,
                             float* out, int32_t memory, void* stream) {
  clear_error();
  if (!f || (!samples && n_rows > 0) || (!out && n_rows > 0) || n_rows < 0 ||
      (memory != DML_HOST && memory != DML_DEVICE)) {
    set_error("invalid predict arguments");
    return DML_ERR_INVALID_ARG;
  }
  if (n_rows == 0) return DML_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const long long width = f->task == DML_CLASSIFICATION ? f->n_classes : 1;
  const size_t xb = sizeof(float) * (size_t)n_rows * f->n_features;
  const size_t ob = sizeof(float) * (size_t)n_rows * width;
  init_pool_once();
  const float* dX = samples;
  float* dout = out;
  float* tX = nullptr;
  float* tout = nullptr;
  if (memory == DML_HOST) {  // AllocatePredict's uploads (gpudte_algorithm.cc:639-673)
    if (cudaMallocAsync(&tX, xb, s) != cudaSuccess || cudaMallocAsync(&tout, ob, s) != cudaSuccess) {
      cudaGetLastError();
      if (tX) cudaFreeAsync(tX, s);
      set_error("device allocation failed for a predict of %lld rows", (long long)n_rows);
      return DML_ERR_OOM;
    }
    cudaMemcpyAsync(tX, samples, xb, cudaMemcpyHostToDevice, s);
    dX = tX;
    dout = tout;
  }
  dml_status st = DML_OK;
  cudaMemsetAsync(dout, 0, ob, s);
  // at most 65,536 (tree, row) threads per launch, a sync after each
  // (gpudte_algorithm.cc:292-311)
  constexpr long long kChunk = 65536;
  for (int t = 0; t < f->n_trees && st == DML_OK; ++t)
    for (long long r0 = 0; r0 < n_rows && st == DML_OK; r0 += kChunk) {
      const long long rows = std::min<long long>(kChunk, n_rows - r0);
      const unsigned blocks = (unsigned)((rows + 63) / 64);
      if (f->task == DML_CLASSIFICATION)
        k_predict_plain<0><<<blocks, 64, 0, s>>>(f->pnodes, t, f->n_classes, dX, n_rows, r0, rows,
                                                 dout);
      else
        k_predict_plain<1><<<blocks, 64, 0, s>>>(f->pnodes, t, 1, dX, n_rows, r0, rows, dout);
      cudaError_t e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) {
        set_error("predict failed: %s", cudaGetErrorString(e));
        st = DML_ERR_CUDA;
      }
    }
  if (memory == DML_HOST) {
    if (st == DML_OK && cudaMemcpyAsync(out, tout, ob, cudaMemcpyDeviceToHost, s) != cudaSuccess) {
      set_error("device to host copy failed");
      st = DML_ERR_CUDA;
    }
    cudaFreeAsync(tX, s);
    cudaFreeAsync(tout, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && st == DML_OK) st = DML_ERR_CUDA;
  }
  return st;
}

dml_status dml_forest_info_get(const dml_forest* f, dml_forest_info* info) {
  if (!f || !info) {
    set_error("null argument");
    return DML_ERR_INVALID_ARG;
  }
  std::memset(info, 0, sizeof(*info));
  info->task = f->task;
  info->n_trees = f->n_trees;
  info->n_classes = f->n_classes;
  info->n_features = f->n_features;
  info->n_nodes = f->n_nodes;
  info->n_probs = f->n_probs;
  info->max_depth = f->max_depth;
  info->fit_ms = f->fit_ms;
  return DML_OK;
}

dml_status dml_forest_export(const dml_forest* f, void* node_array, float* probs) {
  clear_error();
  if (!f || (!node_array && f->n_nodes) || (!probs && f->n_probs)) {
    set_error("null argument");
    return DML_ERR_INVALID_ARG;
  }
  if (copy_host_device(node_array, f->nodes, sizeof(ClassifyNode) * f->n_nodes, false, 0) !=
          cudaSuccess ||
      copy_host_device(probs, f->probs, sizeof(float) * f->n_probs, false, 0) != cudaSuccess ||
      cudaStreamSynchronize(0) != cudaSuccess) {
    cudaGetLastError();
    set_error("device to host copy failed");
    return DML_ERR_CUDA;
  }
  return DML_OK;
}

dml_status dml_forest_gains(const dml_forest* f, float* gains, int32_t memory, void* stream) {
  clear_error();
  if (!f || (!gains && f->n_nodes) || (memory != DML_HOST && memory != DML_DEVICE)) {
    set_error("null argument or bad memory kind");
    return DML_ERR_INVALID_ARG;
  }
  if (!f->gains) {
    set_error("the forest holds no split gains (it was imported or loaded, not fitted)");
    return DML_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(gains, f->gains, sizeof(float) * f->n_nodes,
                      memory == DML_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                      s) != cudaSuccess ||
      (memory == DML_HOST && cudaStreamSynchronize(s) != cudaSuccess)) {
    cudaGetLastError();
    set_error("copy of the split gains failed");
    return DML_ERR_CUDA;
  }
  return DML_OK;
}

dml_status dml_forest_import(int32_t task, int32_t n_trees, int32_t n_classes, int32_t n_features,
                             const void* node_array, int64_t n_nodes, const float* probs,
                             int64_t n_probs, dml_forest** out) {
  clear_error();
  if (!out || !node_array || !probs || n_trees <= 0 || n_nodes < n_trees || n_features <= 0 ||
      (task != DML_CLASSIFICATION && task != DML_REGRESSION) ||
      (task == DML_CLASSIFICATION && (n_classes < 1 || n_classes > kMaxClasses))) {
    set_error("invalid forest import arguments");
    return DML_ERR_INVALID_ARG;
  }
  const int C = task == DML_CLASSIFICATION ? n_classes : 1;
  // structural checks (the reference's "Faulty gpu node" check, gpudte_algorithm.cc:60-63)
  const ClassifyNode* nodes = (const ClassifyNode*)node_array;
  for (long long i = 0; i < n_nodes; ++i) {
    const ClassifyNode& n = nodes[i];
    if (n.child_count > 0) {
      if (n.child_count != 2 || n.child_start <= i || n.child_start + 1 >= n_nodes ||
          n.attribute < 0 || n.attribute >= n_features) {
        set_error("node %lld is malformed", i);
        return DML_ERR_INVALID_ARG;
      }
    } else if (n.probability_start < 0 || n.probability_start + C > n_probs) {
      set_error("leaf %lld points outside the probability array", i);
      return DML_ERR_INVALID_ARG;
    }
  }
  dml_forest* f = new dml_forest();
  f->task = task;
  f->n_trees = n_trees;
  f->n_classes = C;
  f->n_features = n_features;
  f->n_nodes = n_nodes;
  f->n_probs = n_probs;
  cudaGetDevice(&f->device);
  if (cudaMalloc(&f->nodes, sizeof(ClassifyNode) * n_nodes) != cudaSuccess ||
      cudaMalloc(&f->probs, sizeof(float) * std::max<int64_t>(1, n_probs)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(f->nodes);
    delete f;
    set_error("device allocation failed");
    return DML_ERR_OOM;
  }
  cudaMemcpy(f->nodes, node_array, sizeof(ClassifyNode) * n_nodes, cudaMemcpyHostToDevice);
  cudaMemcpy(f->probs, probs, sizeof(float) * n_probs, cudaMemcpyHostToDevice);
  dml_status st = forest_build_pnodes(f, 0);
  if (st == DML_OK && cudaDeviceSynchronize() != cudaSuccess) st = DML_ERR_CUDA;
  if (st != DML_OK) {
    dml_forest_free(f);
    return st;
  }
  *out = f;
  return DML_OK;
}

namespace {
constexpr char kMagic[4] = {'D', 'M', 'L', 'F'};
constexpr uint32_t kVersion = 1;

uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}
}  // namespace

dml_status dml_forest_save(const dml_forest* f, const char* path) {
  clear_error();
  if (!f || !path) {
    set_error("null argument");
    return DML_ERR_INVALID_ARG;
  }
  std::vector<ClassifyNode> nodes((size_t)f->n_nodes);
  std::vector<float> probs((size_t)f->n_probs);
  dml_status st = dml_forest_export(f, nodes.data(), probs.data());
  if (st != DML_OK) return st;
  const int32_t hdr[4] = {f->task, f->n_trees, f->n_classes, f->n_features};
  const int64_t sizes[2] = {f->n_nodes, f->n_probs};
  FILE* fp = std::fopen(path, "wb");
  if (!fp) {
    set_error("cannot open %s for writing", path);
    return DML_ERR_INVALID_ARG;
  }
  uint64_t h = 14695981039346656037ull;
  auto put = [&](const void* p, size_t n) {
    h = fnv1a(h, p, n);
    return std::fwrite(p, 1, n, fp) == n;
  };
  bool ok = put(kMagic, 4) && put(&kVersion, 4) && put(hdr, sizeof(hdr)) &&
            put(sizes, sizeof(sizes)) && put(nodes.data(), sizeof(ClassifyNode) * nodes.size()) &&
            put(probs.data(), sizeof(float) * probs.size());
  ok = ok && std::fwrite(&h, 1, 8, fp) == 8;
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) {
    set_error("write to %s failed", path);
    return DML_ERR_INVALID_ARG;
  }
  return DML_OK;
}

dml_status dml_forest_load(const char* path, dml_forest** out) {
  clear_error();
  if (!path || !out) {
    set_error("null argument");
    return DML_ERR_INVALID_ARG;
  }
  FILE* fp = std::fopen(path, "rb");
  if (!fp) {
    set_error("cannot open %s", path);
    return DML_ERR_INVALID_ARG;
  }
  uint64_t h = 14695981039346656037ull;
  auto get = [&](void* p, size_t n) {
    if (std::fread(p, 1, n, fp) != n) return false;
    h = fnv1a(h, p, n);
    return true;
  };
  char magic[4];
  uint32_t version = 0;
  int32_t hdr[4];
  int64_t sizes[2];
  std::vector<ClassifyNode> nodes;
  std::vector<float> probs;
  bool ok = get(magic, 4) && std::memcmp(magic, kMagic, 4) == 0 && get(&version, 4) &&
            version == kVersion && get(hdr, sizeof(hdr)) && get(sizes, sizeof(sizes));
  // sizes must be plausible before allocating: at least a root per tree, and
  // no more records than the file holds
  if (ok) {
    std::fseek(fp, 0, SEEK_END);
    const long long file_bytes = std::ftell(fp);
    std::fseek(fp, 4 + 4 + sizeof(hdr) + sizeof(sizes), SEEK_SET);
    ok = sizes[0] >= 1 && sizes[1] >= 0 &&
         sizes[0] <= file_bytes / (long long)sizeof(ClassifyNode) &&
         sizes[1] <= file_bytes / 4 &&
         (long long)sizeof(ClassifyNode) * sizes[0] + 4 * sizes[1] + 8 + 40 == file_bytes;
  }
  if (ok) {
    nodes.resize((size_t)sizes[0]);
    probs.resize((size_t)sizes[1]);
    ok = get(nodes.data(), sizeof(ClassifyNode) * nodes.size()) &&
         get(probs.data(), sizeof(float) * probs.size());
  }
  uint64_t stored = 0;
  const uint64_t computed = h;
  ok = ok && std::fread(&stored, 1, 8, fp) == 8 && stored == computed;
  std::fclose(fp);
  if (!ok) {
    set_error("%s is not a valid forest file", path);
    return DML_ERR_INVALID_ARG;
  }
  return dml_forest_import(hdr[0], hdr[1], hdr[2], hdr[3], nodes.data(), sizes[0], probs.data(),
                           sizes[1], out);
}

dml_status dml_device_count(int32_t* count) {
  if (!count) return DML_ERR_INVALID_ARG;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *count = 0;
    set_error("no CUDA device: %s", cudaGetErrorString(e));
    return DML_ERR_CUDA;
  }
  *count = n;
  return DML_OK;
}

dml_status dml_set_device(int32_t device) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("cannot select device %d: %s", device, cudaGetErrorString(e));
    return DML_ERR_CUDA;
  }
  return DML_OK;
}

void dml_forest_free(dml_forest* f) {
  if (!f) return;
  if (f->block) {
    if (f->block->refs.fetch_sub(1) == 1) {
      cudaFree(f->block->base);
      delete f->block;
    }
  } else {
    cudaFree(f->nodes);
    cudaFree(f->probs);
    cudaFree(f->pnodes);
  }
  cudaFree(f->pnodes8);
  delete f;
}

}  // extern "C"
