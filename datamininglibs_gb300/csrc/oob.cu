// Out-of-bag estimate and permutation importance of an RF forest.
//
// Replaces the reference's kOobEstimate and kFeatureImp kernels
// (gpurf.cu:290-438), which nothing launches there.  The reference walks one
// tree per (tree, row) thread, counts right and wrong votes of out-of-bag pairs
// with atomics, and for regression adds the raw leaf value to "mse"; here a
// thread owns a row: it walks every tree whose bag misses the row, counts its
// pairs, keeps the row's out-of-bag votes (or output sum) for the ensemble
// estimate, and writes four per-row values that a fixed-shape reduction sums,
// so the doubles do not depend on scheduling.  Regression errors are squared
// errors.  The bags come from the fit's own draws (bag.cuh).
#include <algorithm>
#include <cstring>
#include <vector>

#include "bag.cuh"
#include "engine.h"

namespace dml {

void clear_error();
void init_pool_once();

namespace {

constexpr int kOobBlock = 128;
constexpr int kRedBlock = 256;
constexpr int kRedItems = 16;  // rows per thread in the first reduction pass

// Multiplicities of every tree's bag: wcnt[t * N + row].
__global__ void k_oob_bag(const ProbDesc* __restrict__ Pp, int* __restrict__ wcnt, int chunk) {
  const ProbDesc& P = *Pp;
  const int t = blockIdx.y;
  const long long beg = (long long)blockIdx.x * chunk;
  const long long end = min(bag_draws(P), beg + chunk);
  for (long long i = beg + threadIdx.x; i < end; i += blockDim.x) {
    const long long row = bag_draw(P, t, i);
    if (row >= 0) atomicAdd(&wcnt[(long long)t * P.N + row], 1);
  }
}

// Per row: acc[0] pairs, acc[1] correct pairs or squared error of pairs,
// acc[2] 1 if the row is out of some bag, acc[3] ensemble correct or squared
// error of the mean out-of-bag output.
template <int TASK>
__global__ void __launch_bounds__(kOobBlock) k_oob_rows(const PNode* __restrict__ nodes,
                                                        const ProbDesc* __restrict__ Pp,
                                                        const float* __restrict__ y,
                                                        const int* __restrict__ wcnt,
                                                        int perm_feature,
                                                        double* __restrict__ acc) {
  extern __shared__ int votes[];  // [kOobBlock][C]
  const ProbDesc& P = *Pp;
  const long long N = P.N;
  const long long row = (long long)blockIdx.x * kOobBlock + threadIdx.x;
  if (row >= N) return;
  int* my = votes + threadIdx.x * P.C;
  if (TASK == 0)
    for (int c = 0; c < P.C; ++c) my[c] = 0;
  const float target = y[row];
  long long pairs = 0, correct = 0;
  double se = 0.0, vsum = 0.0;
  for (int t = 0; t < P.n_trees; ++t) {
    if (wcnt[(long long)t * N + row] > 0) continue;
    long long prow = row;
    if (perm_feature >= 0) {
      U4 r = keyed(P.seed, kTagPermute, (uint32_t)perm_feature, (uint32_t)(t + P.tree_key0),
                   (uint32_t)row, (uint32_t)(row >> 32));
      prow = r.x % (uint32_t)N;
    }
    int4 p = __ldg(reinterpret_cast<const int4*>(nodes) + t);
    while (p.x >= 0) {
      const long long r = p.y == perm_feature ? prow : row;
      const float x = __ldg(P.X + (long long)p.y * N + r);
      p = __ldg(reinterpret_cast<const int4*>(nodes) + (goes_left(x, __int_as_float(p.z)) ? p.x
                                                                                         : p.x + 1));
    }
    ++pairs;
    if (TASK == 0) {
      correct += p.y == (int)target;
      my[p.y] += 1;
    } else {
      const double v = (double)__int_as_float(p.z);
      const double d = __dsub_rn((double)target, v);
      se = __dadd_rn(se, __dmul_rn(d, d));
      vsum = __dadd_rn(vsum, v);
    }
  }
  acc[row] = (double)pairs;
  acc[N + row] = TASK == 0 ? (double)correct : se;
  acc[2 * N + row] = pairs > 0 ? 1.0 : 0.0;
  double ens = 0.0;
  if (pairs > 0) {
    if (TASK == 0) {  // the first class with the strictly largest vote count
      int sel = 0, mx = 0;
      for (int c = 0; c < P.C; ++c)
        if (my[c] > mx) {
          mx = my[c];
          sel = c;
        }
      ens = sel == (int)target ? 1.0 : 0.0;
    } else {
      const double d = __dsub_rn((double)target, __ddiv_rn(vsum, (double)pairs));
      ens = __dmul_rn(d, d);
    }
  }
  acc[3 * N + row] = ens;
}

// Fixed-shape sum of v[0..n): block b sums [b * 4096, (b+1) * 4096), thread j
// adding items j, j + 256, ... in order, then a halving tree over the block.
__device__ double block_tree_sum(double s, double* sm) {
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = kRedBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] = __dadd_rn(sm[threadIdx.x], sm[threadIdx.x + w]);
    __syncthreads();
  }
  return sm[0];
}

__global__ void __launch_bounds__(kRedBlock) k_sum_pass1(const double* __restrict__ v, long long n,
                                                         double* __restrict__ part, int nblk) {
  __shared__ double sm[kRedBlock];
  const double* col = v + (long long)blockIdx.y * n;
  const long long base = (long long)blockIdx.x * kRedBlock * kRedItems;
  double s = 0.0;
  for (int k = 0; k < kRedItems; ++k) {
    const long long i = base + threadIdx.x + (long long)k * kRedBlock;
    if (i < n) s = __dadd_rn(s, col[i]);
  }
  const double r = block_tree_sum(s, sm);
  if (threadIdx.x == 0) part[(long long)blockIdx.y * nblk + blockIdx.x] = r;
}

__global__ void __launch_bounds__(kRedBlock) k_sum_pass2(const double* __restrict__ part, int nblk,
                                                         double* __restrict__ out) {
  __shared__ double sm[kRedBlock];
  const double* col = part + (long long)blockIdx.x * nblk;
  double s = 0.0;
  for (int i = threadIdx.x; i < nblk; i += kRedBlock) s = __dadd_rn(s, col[i]);
  const double r = block_tree_sum(s, sm);
  if (threadIdx.x == 0) out[blockIdx.x] = r;
}

}  // namespace
}  // namespace dml

using namespace dml;

extern "C" dml_status dml_oob_estimate(const dml_forest* f, const dml_fit_desc* desc,
                                       int32_t permuted_feature, dml_oob_stats* out,
                                       void* stream) {
  clear_error();
  if (!f || !desc || !out) {
    set_error("null argument");
    return DML_ERR_INVALID_ARG;
  }
  const dml_fit_desc& d = *desc;
  if (d.algo != DML_ALGO_RF) {
    set_error("out-of-bag rows exist only for bootstrapped (RF) forests");
    return DML_ERR_INVALID_ARG;
  }
  if (d.task != f->task || d.n_features != f->n_features || d.n_trees != f->n_trees ||
      d.n_rows <= 0 || d.n_rows >= (1ll << 31) || !d.samples || !d.targets ||
      (d.task == DML_CLASSIFICATION && d.n_classes != f->n_classes) || d.tree_offset < 0 ||
      (d.memory != DML_HOST && d.memory != DML_DEVICE) || (d.balanced != 0 && d.balanced != 1) ||
      (d.balanced && d.task != DML_CLASSIFICATION) || permuted_feature < -1 ||
      permuted_feature >= f->n_features) {
    set_error("the descriptor does not match the forest, or the feature is out of range");
    return DML_ERR_INVALID_ARG;
  }
  std::memset(out, 0, sizeof(*out));
  init_pool_once();
  alloc_fault_arm();
  cudaStream_t s = (cudaStream_t)stream;
  const long long N = d.n_rows;
  const int C = f->task == DML_CLASSIFICATION ? f->n_classes : 1;
  std::vector<void*> owned;
  auto alloc = [&](size_t b) {
    void* p = dev_alloc(b, s);
    owned.push_back(p);
    return p;
  };
  dml_status st = DML_OK;
  try {
    const float* X = d.samples;
    const float* y = d.targets;
    if (d.memory == DML_HOST) {
      float* dx = (float*)alloc(sizeof(float) * N * d.n_features);
      float* dy = (float*)alloc(sizeof(float) * N);
      DML_CK(cudaMemcpyAsync(dx, d.samples, sizeof(float) * N * d.n_features,
                             cudaMemcpyHostToDevice, s));
      DML_CK(cudaMemcpyAsync(dy, d.targets, sizeof(float) * N, cudaMemcpyHostToDevice, s));
      X = dx;
      y = dy;
    }
    const int grid = (int)std::min<long long>(4096, (N + 255) / 256);
    ProbDesc P;
    std::memset(&P, 0, sizeof(P));
    P.X = X;
    P.N = N;
    P.F = d.n_features;
    P.C = C;
    P.seed = d.seed;
    P.n_trees = d.n_trees;
    P.tree_key0 = d.tree_offset;
    P.algo = DML_ALGO_RF;
    P.task = d.task;
    if (d.task == DML_CLASSIFICATION) {
      int* err = (int*)alloc(sizeof(int));
      DML_CK(cudaMemsetAsync(err, 0, sizeof(int), s));
      k_check_labels<<<grid, 256, 0, s>>>(y, N, C, err);
      int h_err = 0;
      DML_CK(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
      DML_CK(cudaStreamSynchronize(s));
      if (h_err) {
        set_error("classification targets must be integers in [0, n_classes)");
        throw InvalidArg{};
      }
    }
    if (d.balanced) {
      long long* off = (long long*)alloc(sizeof(long long) * (C + 1));
      int* rows = (int*)alloc(sizeof(int) * N);
      DML_CK(cudaMemsetAsync(off, 0, sizeof(long long) * (C + 1), s));
      k_class_count<<<grid, 256, 0, s>>>(y, N, off);
      k_class_offsets<<<1, 32, 0, s>>>(off, C);
      k_class_rows<<<C, 1024, 0, s>>>(y, N, off, rows);
      P.balanced = 1;
      P.bal_m = N / C;
      P.class_rows = rows;
      P.class_off = off;
    }
    ProbDesc* dP = (ProbDesc*)alloc(sizeof(ProbDesc));
    DML_CK(cudaMemcpyAsync(dP, &P, sizeof(ProbDesc), cudaMemcpyHostToDevice, s));
    int* wcnt = (int*)alloc(sizeof(int) * N * d.n_trees);
    DML_CK(cudaMemsetAsync(wcnt, 0, sizeof(int) * N * d.n_trees, s));
    const int chunk = 1 << 16;
    k_oob_bag<<<dim3((unsigned)((N + chunk - 1) / chunk), (unsigned)d.n_trees), 256, 0, s>>>(
        dP, wcnt, chunk);
    double* acc = (double*)alloc(sizeof(double) * 4 * N);
    const unsigned rb = (unsigned)((N + kOobBlock - 1) / kOobBlock);
    if (d.task == DML_CLASSIFICATION)
      k_oob_rows<0><<<rb, kOobBlock, sizeof(int) * kOobBlock * C, s>>>(f->pnodes, dP, y, wcnt,
                                                                       permuted_feature, acc);
    else
      k_oob_rows<1><<<rb, kOobBlock, 0, s>>>(f->pnodes, dP, y, wcnt, permuted_feature, acc);
    const int nblk = (int)((N + kRedBlock * kRedItems - 1) / (kRedBlock * kRedItems));
    double* part = (double*)alloc(sizeof(double) * 4 * nblk);
    double* sums = (double*)alloc(sizeof(double) * 4);
    k_sum_pass1<<<dim3((unsigned)nblk, 4), kRedBlock, 0, s>>>(acc, N, part, nblk);
    k_sum_pass2<<<4, kRedBlock, 0, s>>>(part, nblk, sums);
    DML_CK(cudaGetLastError());
    double h[4];
    DML_CK(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, s));
    DML_CK(cudaStreamSynchronize(s));
    out->pairs = (int64_t)h[0];
    out->rows = (int64_t)h[2];
    if (d.task == DML_CLASSIFICATION) {
      out->pairs_correct = (int64_t)h[1];
      out->rows_correct = (int64_t)h[3];
    } else {
      out->pairs_sq_err = h[1];
      out->rows_sq_err = h[3];
    }
  } catch (const CudaError& e) {
    st = e.e == cudaErrorMemoryAllocation ? DML_ERR_OOM : DML_ERR_CUDA;
  } catch (const InvalidArg&) {
    st = DML_ERR_INVALID_ARG;
  }
  for (void* p : owned) dev_free(p, s);
  if (st == DML_ERR_CUDA) cudaGetLastError();
  return st;
}
