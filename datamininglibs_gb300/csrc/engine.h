// Host-side engine internals shared by the fit driver, predict and server.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/dml.h"
#include "dml_internal.h"

namespace dml {
// One device allocation holding the models of every forest of a fit; each
// forest holds a reference, the last free releases it.
struct ForestBlock {
  void* base = nullptr;
  std::atomic<int> refs{0};
};
}  // namespace dml

struct dml_forest {
  int task = 0, n_trees = 0, n_classes = 1, n_features = 0;
  dml::ClassifyNode* nodes = nullptr;  // device, reference layout
  long long n_nodes = 0;
  float* probs = nullptr;              // device
  long long n_probs = 0;
  dml::PNode* pnodes = nullptr;        // device, predict layout
  // device, compact predict layout (null when it does not fit or before the
  // first bulk prediction, which builds it) and its feature bits.  p8_ready is
  // set (release) once both are final and the layout's kernel has completed;
  // a reader that sees it false builds under p8_mu, which waits for a build
  // another thread has started.
  mutable dml::PNode8* pnodes8 = nullptr;
  mutable int p8_bits = 0;
  mutable std::atomic<bool> p8_ready{false};
  mutable std::mutex p8_mu;
  float* gains = nullptr;              // device, FP32 gain per node (NaN for leaves); null
                                       // for forests not fitted by this engine
  dml::ForestBlock* block = nullptr;   // set when the three arrays live in a shared block
  int max_depth = 0;
  double fit_ms = 0.0;
  int device = 0;
};

namespace dml {

void set_error(const char* fmt, ...);

struct CudaError {
  cudaError_t e;
};

#define DML_CK(call)                                                                    \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      ::dml::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      throw ::dml::CudaError{e_};                                                       \
    }                                                                                   \
  } while (0)

struct InvalidArg {};

// n*ln(n) table recipe (host, IEEE double, fixed order) -> int64 fixed point 2^-28.
void build_nlogn_table(long long nmax, long long* out);
// Fixed-point scale of regression targets from max |y| and the row count.
int quant_scale_from_max(float maxabs, long long n);

dml_status forest_build_pnodes(dml_forest* f, cudaStream_t s);
// Copies `bytes` between a host buffer and device memory on stream s: with
// SM loads and stores through the host buffer's mapped device pointer when both
// ends are 16-byte aligned and the buffer is mapped (a device-to-host copy of
// 16 MB or more only into page-locked memory), else by cudaMemcpyAsync.
cudaError_t copy_host_device(void* dst, const void* src, size_t bytes, bool to_device,
                             cudaStream_t s);
void forest_build_pnodes8(const dml_forest* f, cudaStream_t s);

// Largest RF node (entries) the shared-memory search kernel can hold, and the
// default: with buffers of 2048 entries (48 KB) three CTAs fit an SM.
constexpr int kSearchSmemCap = 4096;
constexpr int kDefaultSmemCap = 2048;

// Scheduling of a fit (tuning.cu): RF nodes of up to warp_max entries (64, 128,
// 256 or 512) are searched by a warp, up to smem_cap by a CTA in shared memory,
// larger ones as per-try items on big_ctas persistent CTAs per SM.
struct Tuning {
  int warp_max, smem_cap, big_ctas;
};
int class_width(int n_classes);  // packed class-count words of the search kernels
bool valid_tuning(const Tuning& t);
Tuning default_tuning(int class_width);
Tuning tuning_for(const dml_fit_desc* descs, int nprob, int class_width);

// Stream-ordered device allocations from the device's memory pool.
void* dev_alloc(size_t bytes, cudaStream_t s);
void dev_free(void* p, cudaStream_t s);

// Forced allocation failure, for failure-detection tests (host side only, no
// device fault): with DML_FAIL_ALLOC=k in the environment, the k-th device
// allocation made by one call of an entry point on the calling thread fails as
// out of memory.  alloc_fault_arm() starts the count (each entry point calls
// it); alloc_fault_fire() is true for the allocation that must fail.
void alloc_fault_arm();
bool alloc_fault_fire();
// ": out of memory (injected by DML_FAIL_ALLOC)" once this call's injected
// failure has fired, else "" (appended to allocation error messages).
const char* alloc_fault_note();

}  // namespace dml
