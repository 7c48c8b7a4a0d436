// Fit driver: the level-wise build of all trees of all forests of a batch.
//
// Replaces GpuDteAlgorithm<T>::Fit (lib_ensembles/source/gpudte_algorithm.cc:
// 15-267).  Where the reference launches find-split / perform-split per chunk
// of <= 512 nodes with four host syncs per chunk and streams level overflow
// through host memory, this driver keeps every level on the device and issues
// one launch set per level for every open node of every tree of every forest,
// with one small summary read per level.  dml_fit_plain keeps the reference's
// chunked launch structure on the same kernels.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "engine.h"
#include "level_kernels.cuh"
#include "search_launch.cuh"

static_assert(dml::kNumQ == DML_NUM_QUEUES && dml::kQWarp == DML_Q_WARP32 &&
                  dml::kQErt == DML_Q_ERT && dml::kQRfSmall == DML_Q_RF_SMEM &&
                  dml::kQRfBig == DML_Q_RF_BIG && dml::kQRfW2 == DML_Q_RF_W64 &&
                  dml::kQRfW4 == DML_Q_RF_W128 && dml::kQRfW8 == DML_Q_RF_W256 &&
                  dml::kQG16 == DML_Q_GROUP16 && dml::kQG8 == DML_Q_GROUP8 &&
                  dml::kQRfW16 == DML_Q_RF_W512 && dml::kQErtW == DML_Q_ERT_W256,
              "node classes of the engine and of include/dml.h agree");

namespace dml {

namespace {
thread_local std::string g_last_error;
thread_local dml_fit_stats g_last_stats;
}  // namespace

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

const char* last_error_str() { return g_last_error.c_str(); }
void clear_error() { g_last_error.clear(); }

// ------------------------------------------------------------ host numerics
// Same recipe as the oracle's table: ln(x) = 2*atanh((m-1)/(m+1)) + e*ln2
// with x = m*2^e, m in [sqrt(1/2), sqrt(2)); compiled with
// -ffp-contract=off so every operation rounds separately.
static double table_ln(double x) {
  int e = 0;
  double m = std::frexp(x, &e);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e = e - 1;
  }
  double z = (m - 1.0) / (m + 1.0);
  double z2 = z * z;
  double term = z;
  double sum = 0.0;
  for (int k = 0; k < 13; ++k) {
    sum = sum + term / (double)(2 * k + 1);
    term = term * z2;
  }
  return 2.0 * sum + (double)e * 0.6931471805599453094;
}

// H[n] = round(n ln n * 2^28) (ldexp is exact; llrint rounds to nearest even).
void build_nlogn_table(long long nmax, long long* out) {
  for (long long n = 0; n <= nmax; ++n)
    out[n] = n < 2 ? 0 : std::llrint(std::ldexp((double)n * table_ln((double)n), 28));
}

int quant_scale_from_max(float mx, long long n) {
  if (mx == 0.0f) return 0;
  int ey = std::ilogb(mx) + 1;
  int en = 0;
  while (((long long)1 << en) < n) ++en;
  int S = 61 - ey - en;
  if (S > 62) S = 62;
  if (S < -60) S = -60;
  return S;
}

namespace {
thread_local long long t_alloc_count = 0;
thread_local long long t_alloc_fail_at = 0;
}  // namespace

void alloc_fault_arm() {
  t_alloc_count = 0;
  const char* e = getenv("DML_FAIL_ALLOC");
  t_alloc_fail_at = e ? std::atoll(e) : 0;
}

bool alloc_fault_fire() { return t_alloc_fail_at > 0 && ++t_alloc_count == t_alloc_fail_at; }

const char* alloc_fault_note() {
  return t_alloc_fail_at > 0 && t_alloc_count >= t_alloc_fail_at
             ? ": out of memory (injected by DML_FAIL_ALLOC)"
             : "";
}

void* dev_alloc(size_t bytes, cudaStream_t s) {
  if (bytes == 0) bytes = 16;
  if (alloc_fault_fire()) {
    set_error("device allocation of %zu bytes failed: out of memory (injected by DML_FAIL_ALLOC)",
              bytes);
    throw CudaError{cudaErrorMemoryAllocation};
  }
  void* p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes, s);
  if (e != cudaSuccess) {
    set_error("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    cudaGetLastError();
    throw CudaError{e};
  }
  return p;
}
void dev_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

// Host <-> device copies of pinned buffers by SMs.  On GB300 hosts shared
// with other jobs the copy engines' rate between pinned host memory and the
// device has varied over time; in one probe it fell from 193-211 to
// 26-54 GB/s while SM copies through the same buffers' mapped pointers still
// ran at 104-193 GB/s, and on an unloaded link both ran at 193-210 GB/s.
__global__ void k_copy16(const int4* __restrict__ src, int4* __restrict__ dst, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

cudaError_t copy_host_device(void* dst, const void* src, size_t bytes, bool to_device,
                             cudaStream_t s) {
  if (bytes == 0) return cudaSuccess;
  const void* host = to_device ? src : dst;
  void* mapped = nullptr;
  const size_t body = bytes & ~(size_t)15;
  const bool aligned = ((uintptr_t)dst % 16 == 0) && ((uintptr_t)src % 16 == 0);
  // Where the GPU reaches pageable memory through the host's page tables
  // (Grace), cudaHostGetDevicePointer maps pageable memory too.  SM loads from
  // it are fast.  SM stores into pages not yet touched fault them in one by
  // one, about 0.28 ms per MB (a 433 MB export into fresh arrays: 117-130 ms),
  // while cudaMemcpyAsync into fresh pageable memory costs a few milliseconds
  // per call plus about 0.03 ms per MB (16-18 ms for the same export, 7-9 ms
  // for an 8 MB predict output that SMs wrote in about 2.3 ms).  So copies to
  // the host take SMs into page-locked memory (cudaHostAlloc /
  // cudaHostRegister) and into pageable memory below kSmPageableStore bytes.
  // The callers synchronise before they return, so pageable sources are read
  // before the caller can reuse them.
  constexpr size_t kSmPageableStore = 16u << 20;
  bool sm = body != 0 && aligned &&
            cudaHostGetDevicePointer(&mapped, const_cast<void*>(host), 0) == cudaSuccess;
  if (sm && !to_device && bytes >= kSmPageableStore) {
    cudaPointerAttributes at{};
    sm = cudaPointerGetAttributes(&at, host) == cudaSuccess && at.type == cudaMemoryTypeHost;
  }
  if (!sm) {
    cudaGetLastError();  // not mapped, or a pageable destination: the copy engines
    return cudaMemcpyAsync(dst, src, bytes,
                           to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, s);
  }
  const int4* from = (const int4*)(to_device ? mapped : src);
  int4* to = (int4*)(to_device ? dst : mapped);
  int sms = 148, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long n = (long long)(body / 16);
  const long long grid = std::min<long long>((long long)sms * 4, (n + 511) / 512);
  k_copy16<<<(unsigned)grid, 512, 0, s>>>(from, to, n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || body == bytes) return e;
  return cudaMemcpyAsync((char*)dst + body, (const char*)src + body, bytes - body,
                         to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, s);
}

// Keeps freed pool memory cached in this process so that repeated fits and
// predictions reuse device buffers instead of returning to the driver.  The
// release threshold is an attribute of each device's own pool, so it is set
// once per device (the first fit on it).
void init_pool_once() {
  constexpr int kMaxDev = 64;
  static std::once_flag once[kMaxDev];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) {
    cudaGetLastError();
    return;
  }
  std::call_once(once[dev], [dev] {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  });
}

// A device buffer that grows (contents preserved) on the stream.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t cap = 0;
  void reserve(size_t n, cudaStream_t s, bool keep = true) {
    if (n <= cap) return;
    size_t nc = std::max(n, cap + cap / 2);
    T* q = (T*)dev_alloc(nc * sizeof(T), s);
    if (keep && p && cap)
      DML_CK(cudaMemcpyAsync(q, p, cap * sizeof(T), cudaMemcpyDeviceToDevice, s));
    dev_free(p, s);
    p = q;
    cap = nc;
  }
  void release(cudaStream_t s) {
    dev_free(p, s);
    p = nullptr;
    cap = 0;
  }
};

constexpr int kPlainChunk = 512;  // reference: max_blocks_ / max_nominal_ nodes per launch

// n*ln(n) table cached on the device across fits (grow-only).
struct TableCache {
  long long* H = nullptr;
  long long n = -1;
  std::mutex mu;
};
static TableCache g_table;

static const long long* nlogn_table(long long nmax, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_table.mu);
  if (g_table.n >= nmax) return g_table.H;
  long long n = std::max(nmax, (long long)1024);
  std::vector<long long> h((size_t)n + 1);
  build_nlogn_table(n, h.data());
  long long* d = nullptr;
  DML_CK(cudaMalloc(&d, sizeof(long long) * (n + 1)));
  DML_CK(cudaMemcpyAsync(d, h.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, s));
  DML_CK(cudaStreamSynchronize(s));
  if (g_table.H) cudaFree(g_table.H);
  g_table.H = d;
  g_table.n = n;
  return d;
}

template <int CW>
void launch_search_cw(int q, const LevelArgs& a, int count, cudaStream_t s);
extern template void launch_search_cw<1>(int, const LevelArgs&, int, cudaStream_t);
extern template void launch_search_cw<2>(int, const LevelArgs&, int, cudaStream_t);
extern template void launch_search_cw<4>(int, const LevelArgs&, int, cudaStream_t);
extern template void launch_search_cw<5>(int, const LevelArgs&, int, cudaStream_t);
extern template void launch_search_cw<8>(int, const LevelArgs&, int, cudaStream_t);
extern template void launch_search_cw<16>(int, const LevelArgs&, int, cudaStream_t);
template <int CW>
void launch_big_cw(BigArgs b, int phase, int grid, int decide_grid, int tries, cudaStream_t s);

static void launch_big(int CW, const BigArgs& b, int phase, int grid, int dgrid, int tries,
                       cudaStream_t s) {
  switch (CW) {
    case 1: launch_big_cw<1>(b, phase, grid, dgrid, tries, s); break;
    case 2: launch_big_cw<2>(b, phase, grid, dgrid, tries, s); break;
    case 4: launch_big_cw<4>(b, phase, grid, dgrid, tries, s); break;
    case 5: launch_big_cw<5>(b, phase, grid, dgrid, tries, s); break;
    case 8: launch_big_cw<8>(b, phase, grid, dgrid, tries, s); break;
    default: launch_big_cw<16>(b, phase, grid, dgrid, tries, s); break;
  }
}

static void launch_search(int CW, int q, const LevelArgs& a, int count, cudaStream_t s) {
  switch (CW) {
    case 1: launch_search_cw<1>(q, a, count, s); break;
    case 2: launch_search_cw<2>(q, a, count, s); break;
    case 4: launch_search_cw<4>(q, a, count, s); break;
    case 5: launch_search_cw<5>(q, a, count, s); break;
    case 8: launch_search_cw<8>(q, a, count, s); break;
    default: launch_search_cw<16>(q, a, count, s); break;
  }
}

struct Summary {
  int children, leaves;
  int qcount[kNumQ];
};

struct ProbHost {
  const float* X = nullptr;  // device
  const float* y = nullptr;  // device
  int* lab = nullptr;
  long long* q = nullptr;
};

static void finish_stats(dml_fit_stats& st) { g_last_stats = st; }

bool compute_ranks(const float* X, long long N, int F, uint32_t* rank, float* vals,
                   cudaStream_t s);

// NVTX ranges (no-ops unless a profiler is attached): one per fit, one per
// level, one per node class's launches.
struct NvtxRange {
  explicit NvtxRange(const char* fmt, ...) {
    char buf[96];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    nvtxRangePushA(buf);
  }
  ~NvtxRange() { nvtxRangePop(); }
};

static const char* const kQueueNames[kNumQ] = {
    "group32", "ert_cta", "rf_smem", "rf_big", "rf_warp64", "rf_warp128",
    "rf_warp256", "group16", "group8", "rf_warp512", "ert_warp256"};

// Fits of at most this many entries (rows drawn into all trees) overlap their
// node classes' launches.
constexpr long long kConcurrentClassEntries = 16ll << 20;

static std::vector<dml_forest*> run_fit(const dml_fit_desc* descs, int nprob, bool plain,
                                        cudaStream_t s) {
  NvtxRange fit_range("dml fit: %d forest(s)%s", nprob, plain ? ", plain" : "");
  init_pool_once();
  // ------------------------------------------------------------ checks
  std::vector<ProbDesc> hp(nprob);
  std::vector<ProbHost> ph(nprob);
  int Cmax = 1;
  long long total_slots = 0;
  int total_trees = 0;
  bool any_weights = false;
  long long H_n = 0;
  for (int i = 0; i < nprob; ++i) {
    const dml_fit_desc& d = descs[i];
    if (d.algo != DML_ALGO_RF && d.algo != DML_ALGO_ERT) {
      set_error("forest %d: algo must be RF (0) or ERT (1)", i);
      throw InvalidArg{};
    }
    if (d.task != DML_CLASSIFICATION && d.task != DML_REGRESSION) {
      set_error("forest %d: task must be classification (0) or regression (1)", i);
      throw InvalidArg{};
    }
    if (d.n_trees <= 0 || d.n_rows <= 0 || d.n_features <= 0 || !d.samples || !d.targets) {
      set_error("forest %d: n_trees, n_rows and n_features must be positive, data non-null", i);
      throw InvalidArg{};
    }
    // RF classification packs (label, bootstrap weight <= n_rows) into 32 bits
    if (d.n_rows >= (1ll << 27) || (long long)d.n_rows * d.n_features >= (1ll << 40)) {
      set_error("forest %d: too many rows", i);
      throw InvalidArg{};
    }
    if (d.task == DML_CLASSIFICATION && (d.n_classes < 1 || d.n_classes > kMaxClasses)) {
      set_error("forest %d: n_classes must be in [1, %d]", i, kMaxClasses);
      throw InvalidArg{};
    }
    if (d.max_depth < 0 || d.min_node_size < 0 || d.n_features_try < 0 || d.tree_offset < 0 ||
        (d.memory != DML_HOST && d.memory != DML_DEVICE)) {
      set_error("forest %d: max_depth, min_node_size, n_features_try must be >= 0", i);
      throw InvalidArg{};
    }
    if (d.balanced != 0 && (d.balanced != 1 || d.algo != DML_ALGO_RF ||
                            d.task != DML_CLASSIFICATION)) {
      set_error("forest %d: balanced sampling is for RF classification only", i);
      throw InvalidArg{};
    }
    ProbDesc& P = hp[i];
    std::memset(&P, 0, sizeof(P));
    P.N = d.n_rows;
    P.F = d.n_features;
    P.C = d.task == DML_CLASSIFICATION ? d.n_classes : 1;
    // kNrFeatures = 0 -> round(ln F) + 1 (gpudte_algorithm.cc:579-580)
    P.K = d.n_features_try > 0 ? d.n_features_try
                               : (int)std::round(std::log((double)d.n_features)) + 1;
    // try loop bounds (gpuert.cu:144-149): K mandatory tries (F if K > F), then
    // up to min(F - K, 10) more while the best gain stays <= 1e-3
    P.n_mand = std::min(P.K, P.F);
    P.n_opt = P.K < P.F ? std::min(P.F - P.K, 10) : 0;
    if (P.n_mand + P.n_opt > kMaxTries) {
      set_error("forest %d: at most %d tries per node", i, kMaxTries);
      throw InvalidArg{};
    }
    P.max_depth = d.max_depth;
    P.min_node_size = d.min_node_size;
    P.min_leaf = std::max(1, d.min_leaf);
    P.algo = d.algo;
    P.task = d.task;
    P.seed = d.seed;
    P.n_trees = d.n_trees;
    P.tree_key0 = d.tree_offset;
    P.tree0 = total_trees;
    P.ent0 = total_slots;
    total_trees += d.n_trees;
    total_slots += (long long)d.n_trees * d.n_rows;
    Cmax = std::max(Cmax, P.C);
    if (d.algo == DML_ALGO_RF) any_weights = true;
    if (d.task == DML_CLASSIFICATION) H_n = std::max(H_n, (long long)d.n_rows);
  }
  const int CW = class_width(Cmax);
  const Tuning tune = tuning_for(descs, nprob, CW);
  dml_fit_stats st;
  std::memset(&st, 0, sizeof(st));

  std::vector<void*> owned;
  auto alloc = [&](size_t bytes) {
    void* p = dev_alloc(bytes, s);
    owned.push_back(p);
    return p;
  };
  DBuf<LNode> cur, nxt;
  DBuf<int> cnt_cur, cnt_nxt, res_cnt, childpos, leafpos;
  DBuf<NodeRes> res_cur, res_nxt;
  DBuf<int2> parts;
  DBuf<int> qlist[kNumQ];
  DBuf<ClassifyNode> node_log;
  DBuf<float> gain_log;
  DBuf<float> prob_log;
  DBuf<Seg> segs;
  DBuf<Cand> big_cand, big_partial;
  DBuf<int> big_candL, big_partialL, big_retry, big_index;
  std::vector<dml_forest*> forests;
  auto release_all = [&]() {
    for (void* p : owned) dev_free(p, s);
    owned.clear();
    cur.release(s);
    nxt.release(s);
    cnt_cur.release(s);
    cnt_nxt.release(s);
    res_cnt.release(s);
    childpos.release(s);
    leafpos.release(s);
    res_cur.release(s);
    res_nxt.release(s);
    parts.release(s);
    for (auto& q : qlist) q.release(s);
    node_log.release(s);
    gain_log.release(s);
    prob_log.release(s);
    segs.release(s);
    big_cand.release(s);
    big_partial.release(s);
    big_candL.release(s);
    big_partialL.release(s);
    big_retry.release(s);
    big_index.release(s);
  };
  try {
    // ---------------------------------------------------- data to device
    int* d_err = (int*)alloc(sizeof(int) * 4);
    unsigned* d_max = (unsigned*)alloc(sizeof(unsigned) * nprob);
    DML_CK(cudaMemsetAsync(d_err, 0, sizeof(int) * 4, s));
    DML_CK(cudaMemsetAsync(d_max, 0, sizeof(unsigned) * nprob, s));
    std::vector<PrepJob> jobs(nprob);
    long long sum_nx = 0;
    for (int i = 0; i < nprob; ++i) {
      const dml_fit_desc& d = descs[i];
      ProbDesc& P = hp[i];
      ProbHost& H = ph[i];
      H.X = d.samples;
      H.y = d.targets;
      if (d.memory == DML_HOST) {
        float* dx = (float*)alloc(sizeof(float) * P.N * P.F);
        float* dy = (float*)alloc(sizeof(float) * P.N);
        DML_CK(copy_host_device(dx, d.samples, sizeof(float) * P.N * P.F, true, s));
        DML_CK(copy_host_device(dy, d.targets, sizeof(float) * P.N, true, s));
        H.X = dx;
        H.y = dy;
      }
      P.X = H.X;
      if (P.task == 0)
        H.lab = (int*)alloc(sizeof(int) * P.N);
      else
        H.q = (long long*)alloc(sizeof(long long) * P.N);
      P.lab = H.lab;
      P.q = H.q;
      jobs[i] = PrepJob{H.X, P.N * P.F, H.y, P.N, P.task, P.C, 0, H.lab, H.q};
      sum_nx += P.N * P.F;
    }
    // one launch validates every problem (about 64 values a thread overall),
    // one prepares the targets once the regression scales are known
    const unsigned prep_x = (unsigned)std::max<long long>(
        16, std::min<long long>(4096, sum_nx / (256 * 64) / nprob));
    PrepJob* d_jobs = (PrepJob*)alloc(sizeof(PrepJob) * nprob);
    DML_CK(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(PrepJob) * nprob, cudaMemcpyHostToDevice,
                           s));
    for (int j0 = 0; j0 < nprob; j0 += 65535) {  // grid.y holds at most 65535 problems
      const int nj = std::min(65535, nprob - j0);
      k_validate_all<<<dim3(prep_x, (unsigned)nj), 256, 0, s>>>(d_jobs + j0, d_err, d_max + j0);
      DML_CK(cudaGetLastError());
      ++st.launches;
    }
    int h_err[4] = {0, 0, 0, 0};
    std::vector<unsigned> h_max(nprob);
    DML_CK(cudaMemcpyAsync(h_err, d_err, sizeof(h_err), cudaMemcpyDeviceToHost, s));
    DML_CK(cudaMemcpyAsync(h_max.data(), d_max, sizeof(unsigned) * nprob,
                           cudaMemcpyDeviceToHost, s));
    DML_CK(cudaStreamSynchronize(s));
    if (h_err[0] & 1) {
      set_error("samples hold NaN or infinite values (the missing-value marker is -FLT_MAX)");
      throw InvalidArg{};
    }
    if (h_err[0] & 2) {
      set_error("classification targets must be integers in [0, n_classes)");
      throw InvalidArg{};
    }
    if (h_err[0] & 4) {
      set_error("regression targets hold NaN or infinite values");
      throw InvalidArg{};
    }
    for (int i = 0; i < nprob; ++i) {
      float mx;
      std::memcpy(&mx, &h_max[i], 4);
      hp[i].S = hp[i].task == 1 ? quant_scale_from_max(mx, hp[i].N) : 0;
      jobs[i].S = hp[i].S;
    }
    DML_CK(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(PrepJob) * nprob, cudaMemcpyHostToDevice,
                           s));
    for (int j0 = 0; j0 < nprob; j0 += 65535) {
      k_prep_all<<<dim3(prep_x, (unsigned)std::min(65535, nprob - j0)), 256, 0, s>>>(d_jobs + j0);
      DML_CK(cudaGetLastError());
      ++st.launches;
    }
    for (int i = 0; i < nprob; ++i) {
      ProbDesc& P = hp[i];
      const int grid = (int)std::min<long long>(4096, (P.N + 255) / 256);
      if (descs[i].balanced) {  // per-class row lists for the balanced bootstrap
        long long* off = (long long*)alloc(sizeof(long long) * (P.C + 1));
        int* rows = (int*)alloc(sizeof(int) * P.N);
        DML_CK(cudaMemsetAsync(off, 0, sizeof(long long) * (P.C + 1), s));
        k_class_count<<<grid, 256, 0, s>>>(ph[i].y, P.N, off);
        k_class_offsets<<<1, 32, 0, s>>>(off, P.C);
        k_class_rows<<<P.C, 1024, 0, s>>>(ph[i].y, P.N, off, rows);
        DML_CK(cudaGetLastError());
        st.launches += 3;
        P.balanced = 1;
        P.bal_m = P.N / P.C;
        P.class_rows = rows;
        P.class_off = off;
      }
      // RF nodes larger than a warp sort value ranks (ranks.cu); the plain
      // path sorts raw keys, as the reference does
      if (P.algo == DML_ALGO_RF && P.N > 256 && !plain) {
        uint32_t* rank = (uint32_t*)alloc(sizeof(uint32_t) * P.N * P.F);
        float* vals = (float*)alloc(sizeof(float) * P.N * P.F);
        if (compute_ranks(P.X, P.N, P.F, rank, vals, s)) {
          P.rank = rank;
          P.vals = vals;
          st.launches += 3;
        } else {
          clear_error();
        }
      }
    }
    const long long* H = H_n > 0 ? nlogn_table(H_n, s) : nullptr;

    // --------------------------------------------------------- entries
    int* rowsA = (int*)alloc(sizeof(int) * total_slots);
    int* rowsB = (int*)alloc(sizeof(int) * total_slots);
    int* wA = any_weights ? (int*)alloc(sizeof(int) * total_slots) : nullptr;
    int* wB = any_weights ? (int*)alloc(sizeof(int) * total_slots) : nullptr;
    // bootstrap multiplicities per entry slot, read by k_roots
    int* boot = any_weights ? (int*)alloc(sizeof(int) * total_slots) : nullptr;
    // big-node scratch: 4 words per entry of the largest RF tree, per CTA
    int max_mand = 1, max_opt = 0;
    long long slot_stride = 0;
    for (auto& P : hp) {
      max_mand = std::max(max_mand, P.n_mand);
      max_opt = std::max(max_opt, P.n_opt);
      if (P.algo == DML_ALGO_RF && P.N > tune.smem_cap) slot_stride = std::max(slot_stride, P.N);
    }
    int sms = 148, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int big_grid = tune.big_ctas * sms;  // persistent CTAs
    if (slot_stride > 0) {
      // per-CTA scratch is 16 bytes per entry of the largest tree: at most 48 GB
      // and a third of the free device memory
      size_t free_b = 0, total_b = 0;
      cudaMemGetInfo(&free_b, &total_b);
      const long long budget = std::min<long long>(48ll << 30, (long long)free_b / 3);
      big_grid = (int)std::max(1ll, std::min<long long>(big_grid, budget / (16 * slot_stride)));
    }
    uint32_t* big_slot =
        slot_stride > 0 ? (uint32_t*)alloc(sizeof(uint32_t) * 4 * slot_stride * big_grid) : nullptr;
    bool any_cls = false, any_reg = false;
    for (auto& P : hp) {
      any_cls = any_cls || P.task == 0;
      any_reg = any_reg || P.task != 0;
    }
    uint32_t* big_pv =
        slot_stride > 0 && any_cls ? (uint32_t*)alloc(sizeof(uint32_t) * total_slots) : nullptr;
    long long* big_pq =
        slot_stride > 0 && any_reg ? (long long*)alloc(sizeof(long long) * total_slots) : nullptr;
    // [0] retry count of the big-node search, [1..2] its item counters per phase
    int* d_nretry = (int*)alloc(sizeof(int) * 3);
    // the largest entry weight (0 without bootstrap weights: read as 1)
    int* d_maxw = (int*)alloc(sizeof(int));
    ProbDesc* d_probs = (ProbDesc*)alloc(sizeof(ProbDesc) * nprob);
    DML_CK(cudaMemcpyAsync(d_probs, hp.data(), sizeof(ProbDesc) * nprob, cudaMemcpyHostToDevice, s));
    std::vector<int> tree_prob(total_trees);
    for (int i = 0; i < nprob; ++i)
      for (int t = 0; t < hp[i].n_trees; ++t) tree_prob[hp[i].tree0 + t] = i;
    int* d_tree_prob = (int*)alloc(sizeof(int) * total_trees);
    DML_CK(cudaMemcpyAsync(d_tree_prob, tree_prob.data(), sizeof(int) * total_trees,
                           cudaMemcpyHostToDevice, s));
    long long* fbase[2];
    long long* lbase[2];
    for (int b = 0; b < 2; ++b) {
      fbase[b] = (long long*)alloc(sizeof(long long) * nprob);
      lbase[b] = (long long*)alloc(sizeof(long long) * nprob);
      DML_CK(cudaMemsetAsync(fbase[b], 0, sizeof(long long) * nprob, s));
      DML_CK(cudaMemsetAsync(lbase[b], 0, sizeof(long long) * nprob, s));
    }
    int* d_qcount = (int*)alloc(sizeof(int) * kNumQ);
    int* d_summary = (int*)alloc(sizeof(int) * 2);
    // [0..3] fit totals, then 4 per node class: [2] tries x entries, [3] entries
    constexpr int kStatWords = 4 + 4 * kNumQ;
    long long* d_stats = (long long*)alloc(sizeof(long long) * kStatWords);
    DML_CK(cudaMemsetAsync(d_stats, 0, sizeof(long long) * kStatWords, s));
    Summary* h_sum = nullptr;
    DML_CK(cudaMallocHost(&h_sum, sizeof(Summary)));

    cudaEvent_t ev0, ev1;
    DML_CK(cudaEventCreate(&ev0));
    DML_CK(cudaEventCreate(&ev1));
    DML_CK(cudaEventRecord(ev0, s));

    // ------------------------------------------------------------ roots
    int n = total_trees;
    cur.reserve(n, s, false);
    cnt_cur.reserve((size_t)n * Cmax, s, false);
    res_cur.reserve(n, s, false);
    for (auto& q : qlist) q.reserve(n, s, false);
    DML_CK(cudaMemsetAsync(d_qcount, 0, sizeof(int) * kNumQ, s));
    auto queues = [&]() {
      Queues Q;
      for (int i = 0; i < kNumQ; ++i) Q.list[i] = qlist[i].p;
      Q.count = d_qcount;
      Q.rf_small_cap = tune.smem_cap;
      Q.rf_warp_max = tune.warp_max;
      return Q;
    };
    if (any_weights) {
      DML_CK(cudaMemsetAsync(boot, 0, sizeof(int) * total_slots, s));
      long long maxN = 0;
      for (auto& P : hp) maxN = std::max(maxN, P.N);
      const int chunk = 1 << 16;
      dim3 g((unsigned)((maxN + chunk - 1) / chunk), (unsigned)total_trees);
      k_boot_count<<<g, 256, 0, s>>>(d_probs, d_tree_prob, boot, chunk);
      DML_CK(cudaGetLastError());
      ++st.launches;
    }
    {
      DML_CK(cudaMemsetAsync(d_maxw, 0, sizeof(int), s));  // read as at least 1
      if (any_weights) {
        int sms = 148, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        k_max_weight<<<sms * 4, 256, 0, s>>>(boot, total_slots, d_maxw);
        DML_CK(cudaGetLastError());
        ++st.launches;
      }
    }
    k_roots<1024><<<total_trees, 1024, 0, s>>>(d_probs, d_tree_prob, boot, rowsA,
                                               wA, cur.p, cnt_cur.p, Cmax, res_cur.p, queues(),
                                               d_stats);
    DML_CK(cudaGetLastError());
    ++st.launches;
    DML_CK(cudaMemcpyAsync(h_sum->qcount, d_qcount, sizeof(int) * kNumQ, cudaMemcpyDeviceToHost, s));
    DML_CK(cudaStreamSynchronize(s));

    long long log_base = 0, plog_base = 0;
    int depth = 0;
    float search_ms_total = 0.0f;
    cudaEvent_t es0, es1, qev[kNumQ][2];
    DML_CK(cudaEventCreate(&es0));
    DML_CK(cudaEventCreate(&es1));
    for (auto& e : qev) {
      DML_CK(cudaEventCreate(&e[0]));
      DML_CK(cudaEventCreate(&e[1]));
    }
    // On small fits the node classes of a level run on streams of their own:
    // each node is in one class and writes only its own results and entry
    // range, so the classes are independent, and their launches overlap where
    // a level is too small to fill the GPU (the 4601 x 57, 64-tree ERT fit:
    // 2.4 -> 1.8 ms).  On large fits the classes' kernels compete for SMs and
    // caches instead (the 1M x 128 fit: 728 -> 826 ms), so they run one after
    // another on the fit stream, as they do on the plain path and with
    // DML_SERIAL_CLASSES=1.
    const char* senv = getenv("DML_SERIAL_CLASSES");
    const bool concurrent =
        !plain && !(senv && senv[0] == '1') && total_slots <= kConcurrentClassEntries;
    cudaStream_t qstream[kNumQ];
    cudaEvent_t ev_fork, ev_join[kNumQ];
    DML_CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    for (int q = 0; q < kNumQ; ++q) {
      qstream[q] = s;
      DML_CK(cudaEventCreateWithFlags(&ev_join[q], cudaEventDisableTiming));
      if (concurrent) DML_CK(cudaStreamCreateWithFlags(&qstream[q], cudaStreamNonBlocking));
    }
    // launch order: the longest classes first, so that the short ones fill
    // their tails
    static constexpr int kClassOrder[kNumQ] = {kQRfBig, kQRfSmall, kQRfW16, kQRfW8, kQRfW4,
                                               kQRfW2,  kQErt,     kQErtW,  kQWarp, kQG16,
                                               kQG8};
    double queue_ms[kNumQ] = {};
    int queue_launches[kNumQ] = {};
    const char* tenv = getenv("DML_TRACE");
    const bool trace = tenv && tenv[0] == '1';
    while (n > 0) {
      NvtxRange level_range("dml level %d: %d nodes", depth, n);
      // ------------------------------------------- search + partition
      LevelArgs a;
      a.probs = d_probs;
      a.nodes = cur.p;
      a.cnt = cnt_cur.p;
      a.Cmax = Cmax;
      a.res = res_cur.p;
      res_cnt.reserve((size_t)n * Cmax, s, false);
      a.res_cnt = res_cnt.p;
      a.rowsA = rowsA;
      a.wA = wA;
      a.rowsB = rowsB;
      a.wB = wB;
      a.H = H;
      a.stats = d_stats;
      a.smem_cap = tune.smem_cap;
      int qc[kNumQ];
      std::memcpy(qc, h_sum->qcount, sizeof(qc));
      // the big class's buffers, allocated in stream order on s before the fork
      if (qc[kQRfBig] > 0) {
        const int nb = qc[kQRfBig];
        big_cand.reserve((size_t)nb * kMaxTries, s, false);
        big_candL.reserve((size_t)nb * kMaxTries * Cmax, s, false);
        big_partial.reserve((size_t)nb, s, false);
        big_partialL.reserve((size_t)nb * Cmax, s, false);
        big_retry.reserve((size_t)nb, s, false);
        big_index.reserve((size_t)n, s, false);
      }
      DML_CK(cudaEventRecord(es0, s));
      if (concurrent) DML_CK(cudaEventRecord(ev_fork, s));
      float qms[kNumQ] = {};
      for (int q : kClassOrder) {
        if (qc[q] <= 0) continue;
        NvtxRange class_range("dml search %s: %d nodes", kQueueNames[q], qc[q]);
        cudaStream_t sq = qstream[q];
        if (concurrent) DML_CK(cudaStreamWaitEvent(sq, ev_fork, 0));
        if (q == kQRfBig) {
          // per-(node, try) items on a persistent grid with per-CTA scratch
          const int nb = qc[q];
          BigArgs b;
          b.L = a;
          b.big = qlist[q].p;
          b.nbig = nb;
          b.retry = big_retry.p;
          b.nretry = d_nretry;
          b.cand = big_cand.p;
          b.candL = big_candL.p;
          b.slot = big_slot;
          b.slot_stride = slot_stride;
          b.partial = big_partial.p;
          b.partialL = big_partialL.p;
          b.retry_out = big_retry.p;
          b.nretry_out = d_nretry;
          b.big_index = big_index.p;
          b.pv = big_pv;
          b.pq = big_pq;
          b.item_ctr = d_nretry + 1;
          b.maxw = d_maxw;
          b.L.stats = d_stats + 4 + 4 * q;
          DML_CK(cudaEventRecord(qev[q][0], sq));
          const int chunk = plain ? kPlainChunk : nb;
          for (int off = 0; off < nb; off += chunk) {
            b.big = qlist[q].p + off;
            b.nbig = std::min(chunk, nb - off);
            DML_CK(cudaMemsetAsync(d_nretry, 0, sizeof(int) * 3, sq));
            launch_big(CW, b, 1, big_grid, std::min(b.nbig, 65535), max_mand, sq);
            launch_big(CW, b, 2, big_grid, std::min(b.nbig, 65535), std::max(1, max_opt), sq);
            st.launches += 5;
            queue_launches[q] += 5;
            if (plain) DML_CK(cudaStreamSynchronize(sq));
          }
          DML_CK(cudaEventRecord(qev[q][1], sq));
        } else {
          LevelArgs aq = a;
          aq.stats = d_stats + 4 + 4 * q;
          DML_CK(cudaEventRecord(qev[q][0], sq));
          if (!plain) {
            aq.work = qlist[q].p;
            launch_search(CW, q, aq, qc[q], sq);
            ++st.launches;
            ++queue_launches[q];
          } else {
            for (int off = 0; off < qc[q]; off += kPlainChunk) {
              aq.work = qlist[q].p + off;
              launch_search(CW, q, aq, std::min(kPlainChunk, qc[q] - off), sq);
              ++st.launches;
              ++queue_launches[q];
              DML_CK(cudaStreamSynchronize(sq));
            }
          }
          DML_CK(cudaEventRecord(qev[q][1], sq));
        }
        if (concurrent) {
          DML_CK(cudaEventRecord(ev_join[q], sq));
          DML_CK(cudaStreamWaitEvent(s, ev_join[q], 0));
        }
      }
      DML_CK(cudaEventRecord(es1, s));
      // -------------------------------------------------- scans
      int nparts = (n + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems);
      parts.reserve(nparts, s, false);
      childpos.reserve((size_t)n + 1, s, false);
      leafpos.reserve((size_t)n + 1, s, false);
      k_scan_part<<<nparts, kScanBlock, 0, s>>>(res_cur.p, n, parts.p);
      k_scan_top<<<1, kScanBlock, 0, s>>>(parts.p, nparts, childpos.p, leafpos.p, n, d_summary);
      k_scan_apply<<<nparts, kScanBlock, 0, s>>>(res_cur.p, n, parts.p, childpos.p, leafpos.p);
      DML_CK(cudaGetLastError());
      st.launches += 3;
      // ------------------------------------------------ emission
      nxt.reserve((size_t)2 * n, s, false);
      cnt_nxt.reserve((size_t)2 * n * Cmax, s, false);
      res_nxt.reserve((size_t)2 * n, s, false);
      for (auto& q : qlist) q.reserve((size_t)2 * n, s, false);
      node_log.reserve((size_t)(log_base + n), s, true);
      gain_log.reserve((size_t)(log_base + n), s, true);
      prob_log.reserve((size_t)(plog_base + n) * Cmax, s, true);
      segs.reserve((size_t)(depth + 1) * nprob, s, true);
      DML_CK(cudaMemsetAsync(segs.p + (size_t)depth * nprob, 0, sizeof(Seg) * nprob, s));
      DML_CK(cudaMemsetAsync(d_qcount, 0, sizeof(int) * kNumQ, s));
      // forests without nodes at this level keep their bases
      DML_CK(cudaMemcpyAsync(fbase[(depth + 1) & 1], fbase[depth & 1], sizeof(long long) * nprob,
                             cudaMemcpyDeviceToDevice, s));
      DML_CK(cudaMemcpyAsync(lbase[(depth + 1) & 1], lbase[depth & 1], sizeof(long long) * nprob,
                             cudaMemcpyDeviceToDevice, s));
      EmitArgs e;
      e.probs = d_probs;
      e.cur = cur.p;
      e.cnt = cnt_cur.p;
      e.res = res_cur.p;
      e.res_cnt = res_cnt.p;
      e.childpos = childpos.p;
      e.leafpos = leafpos.p;
      e.n = n;
      e.Cmax = Cmax;
      e.log_base = log_base;
      e.plog_base = plog_base;
      e.node_log = node_log.p;
      e.gain_log = gain_log.p;
      e.prob_log = prob_log.p;
      e.fbase_cur = fbase[depth & 1];
      e.lbase_cur = lbase[depth & 1];
      e.fbase_next = fbase[(depth + 1) & 1];
      e.lbase_next = lbase[(depth + 1) & 1];
      e.seg = segs.p + (size_t)depth * nprob;
      e.next = nxt.p;
      e.next_cnt = cnt_nxt.p;
      e.next_res = res_nxt.p;
      e.Q = queues();
      e.stats = d_stats;
      k_emit<<<(n + 255) / 256, 256, 0, s>>>(e);
      DML_CK(cudaGetLastError());
      ++st.launches;
      DML_CK(cudaMemcpyAsync(h_sum, d_summary, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
      DML_CK(cudaMemcpyAsync(h_sum->qcount, d_qcount, sizeof(int) * kNumQ,
                             cudaMemcpyDeviceToHost, s));
      DML_CK(cudaStreamSynchronize(s));
      float sm = 0.0f;
      cudaEventElapsedTime(&sm, es0, es1);
      for (int q = 0; q < kNumQ; ++q)
        if (qc[q] > 0) {
          cudaEventElapsedTime(&qms[q], qev[q][0], qev[q][1]);
          queue_ms[q] += qms[q];
        }
      search_ms_total += sm;
      if (trace)
        fprintf(stderr,
                "[dml] level %2d nodes %9d | g8 %8d %7.2f | g16 %8d %7.2f | w32 %8d %7.2f | "
                "ertw %7d %7.2f | ert %6d %7.2f | w64 %7d %7.2f | w128 %7d %7.2f | w256 %7d %7.2f | "
                "w512 %7d %7.2f | cta %7d %7.2f | big %5d %7.2f | search %8.2f ms\n",
                depth, n, qc[kQG8], qms[kQG8], qc[kQG16], qms[kQG16], qc[kQWarp], qms[kQWarp],
                qc[kQErtW], qms[kQErtW], qc[kQErt], qms[kQErt], qc[kQRfW2], qms[kQRfW2], qc[kQRfW4],
                qms[kQRfW4], qc[kQRfW8], qms[kQRfW8], qc[kQRfW16], qms[kQRfW16], qc[kQRfSmall],
                qms[kQRfSmall], qc[kQRfBig], qms[kQRfBig], sm);
      if (trace) {  // per class: entries and tries x entries searched at this level
        static long long prev[kStatWords];
        long long cur_st[kStatWords];
        if (depth == 0) std::memset(prev, 0, sizeof(prev));
        DML_CK(cudaMemcpy(cur_st, d_stats, sizeof(cur_st), cudaMemcpyDeviceToHost));
        fprintf(stderr, "[dml] level %2d work", depth);
        for (int q = 0; q < kNumQ; ++q)
          if (qc[q] > 0)
            fprintf(stderr, " | q%d entries %lld tries %lld", q,
                    cur_st[4 + 4 * q + 3] - prev[4 + 4 * q + 3],
                    cur_st[4 + 4 * q + 2] - prev[4 + 4 * q + 2]);
        fprintf(stderr, "\n");
        std::memcpy(prev, cur_st, sizeof(prev));
      }
      log_base += n;
      plog_base += h_sum->leaves;
      n = h_sum->children;
      std::swap(cur, nxt);
      std::swap(cnt_cur, cnt_nxt);
      std::swap(res_cur, res_nxt);
      std::swap(rowsA, rowsB);
      std::swap(wA, wB);
      ++depth;
    }
    DML_CK(cudaEventRecord(ev1, s));
    DML_CK(cudaEventSynchronize(ev1));
    float loop_ms = 0.0f;
    cudaEventElapsedTime(&loop_ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaEventDestroy(es0);
    cudaEventDestroy(es1);
    for (auto& e : qev) {
      cudaEventDestroy(e[0]);
      cudaEventDestroy(e[1]);
    }
    cudaEventDestroy(ev_fork);
    for (int q = 0; q < kNumQ; ++q) {
      cudaEventDestroy(ev_join[q]);
      if (concurrent) cudaStreamDestroy(qstream[q]);
    }
    long long h_stats[kStatWords];
    DML_CK(cudaMemcpy(h_stats, d_stats, sizeof(h_stats), cudaMemcpyDeviceToHost));
    cudaFreeHost(h_sum);
    st.nodes = log_base;
    st.entries = h_stats[0];
    st.weighted_rows = h_stats[1];
    st.entry_tries = 0;
    for (int q = 0; q < kNumQ; ++q) {
      st.queue_ms[q] = queue_ms[q];
      st.queue_launches[q] = queue_launches[q];
      st.queue_entry_tries[q] = h_stats[4 + 4 * q + 2];
      st.queue_entries[q] = h_stats[4 + 4 * q + 3];
      st.entry_tries += st.queue_entry_tries[q];
    }
    st.levels = depth;
    st.level_loop_ms = loop_ms;
    st.search_ms = search_ms_total;

    // --------------------------------------------------- per-forest models
    std::vector<long long> fnodes(nprob), fleaves(nprob);
    DML_CK(cudaMemcpyAsync(fnodes.data(), fbase[depth & 1], sizeof(long long) * nprob,
                           cudaMemcpyDeviceToHost, s));
    DML_CK(cudaMemcpyAsync(fleaves.data(), lbase[depth & 1], sizeof(long long) * nprob,
                           cudaMemcpyDeviceToHost, s));
    std::vector<Seg> hseg((size_t)depth * nprob);
    if (nprob > 1 && depth > 0)
      DML_CK(cudaMemcpyAsync(hseg.data(), segs.p, sizeof(Seg) * hseg.size(),
                             cudaMemcpyDeviceToHost, s));
    DML_CK(cudaStreamSynchronize(s));
    // one block for every forest's node, gain, probability and predict arrays
    auto al = [](long long b) { return (b + 255) & ~255ll; };
    long long block_bytes = 0;
    for (int i = 0; i < nprob; ++i)
      block_bytes += al(sizeof(ClassifyNode) * std::max<long long>(1, fnodes[i])) +
                     al(sizeof(float) * std::max<long long>(1, fnodes[i])) +
                     al(sizeof(float) * std::max<long long>(1, fleaves[i] * hp[i].C)) +
                     al(sizeof(PNode) * std::max<long long>(1, fnodes[i]));
    ForestBlock* block = new ForestBlock();
    if (alloc_fault_fire() || cudaMalloc(&block->base, block_bytes) != cudaSuccess) {
      delete block;
      cudaGetLastError();
      set_error("device allocation of %lld bytes for the forests failed%s", block_bytes,
                alloc_fault_note());
      throw CudaError{cudaErrorMemoryAllocation};
    }
    char* bp = (char*)block->base;
    std::vector<GatherSeg> gsegs;
    for (int i = 0; i < nprob; ++i) {
      dml_forest* f = new dml_forest();
      forests.push_back(f);
      f->task = hp[i].task;
      f->n_trees = hp[i].n_trees;
      f->n_classes = hp[i].C;
      f->n_features = hp[i].F;
      f->n_nodes = fnodes[i];
      f->n_probs = fleaves[i] * hp[i].C;
      f->fit_ms = loop_ms;
      cudaGetDevice(&f->device);
      f->block = block;
      block->refs.fetch_add(1);
      f->nodes = (ClassifyNode*)bp;
      bp += al(sizeof(ClassifyNode) * std::max<long long>(1, f->n_nodes));
      f->gains = (float*)bp;
      bp += al(sizeof(float) * std::max<long long>(1, f->n_nodes));
      f->probs = (float*)bp;
      bp += al(sizeof(float) * std::max<long long>(1, f->n_probs));
      f->pnodes = (PNode*)bp;
      bp += al(sizeof(PNode) * std::max<long long>(1, f->n_nodes));
      if (nprob == 1) {
        DML_CK(cudaMemcpyAsync(f->nodes, node_log.p, sizeof(ClassifyNode) * f->n_nodes,
                               cudaMemcpyDeviceToDevice, s));
        DML_CK(cudaMemcpyAsync(f->gains, gain_log.p, sizeof(float) * f->n_nodes,
                               cudaMemcpyDeviceToDevice, s));
        DML_CK(cudaMemcpyAsync(f->probs, prob_log.p, sizeof(float) * f->n_probs,
                               cudaMemcpyDeviceToDevice, s));
        f->max_depth = depth - 1;
      } else {
        long long no = 0, po = 0;
        for (int d = 0; d < depth; ++d) {
          const Seg& sg = hseg[(size_t)d * nprob + i];
          if (sg.node_cnt <= 0) continue;
          f->max_depth = d;
          GatherSeg g;
          g.node_pos = sg.node_pos;
          g.node_cnt = sg.node_cnt;
          g.node_dst = f->nodes + no;
          g.gain_dst = f->gains + no;
          g.leaf_rank = sg.leaf_rank;
          g.leaf_cnt = sg.leaf_cnt;
          g.C = hp[i].C;
          g.prob_dst = f->probs + po;
          gsegs.push_back(g);
          no += sg.node_cnt;
          po += sg.leaf_cnt * hp[i].C;
        }
      }
    }
    if (!gsegs.empty()) {
      GatherSeg* d_gsegs = (GatherSeg*)alloc(sizeof(GatherSeg) * gsegs.size());
      DML_CK(cudaMemcpyAsync(d_gsegs, gsegs.data(), sizeof(GatherSeg) * gsegs.size(),
                             cudaMemcpyHostToDevice, s));
      k_gather_segments<<<(unsigned)gsegs.size(), 256, 0, s>>>(d_gsegs, node_log.p, gain_log.p,
                                                               prob_log.p, Cmax);
      DML_CK(cudaGetLastError());
      ++st.launches;
    }
    for (dml_forest* f : forests) {
      dml_status ps = forest_build_pnodes(f, s);
      if (ps != DML_OK) throw CudaError{cudaErrorUnknown};
      ++st.launches;
    }
    DML_CK(cudaStreamSynchronize(s));
    release_all();
    DML_CK(cudaStreamSynchronize(s));
    finish_stats(st);
  } catch (...) {
    // a failure in the middle of a level can leave kernels queued on the
    // node classes' own streams, which are joined to s only after all of a
    // level's launches: wait for the whole device before the buffers go
    cudaDeviceSynchronize();
    for (dml_forest* f : forests) dml_forest_free(f);
    release_all();
    cudaStreamSynchronize(s);
    throw;
  }
  return forests;
}

dml_status forest_build_pnodes(dml_forest* f, cudaStream_t s) {
  if (!f->block) {  // forests of a fit have theirs in the fit's block
    cudaFree(f->pnodes);
    f->pnodes = nullptr;
    if (cudaMalloc(&f->pnodes, sizeof(PNode) * std::max<long long>(1, f->n_nodes)) !=
        cudaSuccess) {
      set_error("device allocation failed for the predict layout");
      return DML_ERR_OOM;
    }
  }
  int g = (int)std::min<long long>(8192, (f->n_nodes + 255) / 256 + 1);
  k_to_pnodes<<<g, 256, 0, s>>>(f->nodes, f->n_nodes, f->probs, f->n_classes, f->task, f->pnodes);
  if (cudaGetLastError() != cudaSuccess) {
    set_error("launch failure building the predict layout");
    return DML_ERR_CUDA;
  }
  return DML_OK;
}

// The compact layout, built once per forest by its first bulk prediction,
// when the features and every child offset fit 32 bits; a word past the
// nodes flags an offset that does not (the layout is then dropped, and bulk
// prediction walks the 16-byte one).  Synchronises s.
void forest_build_pnodes8(const dml_forest* f, cudaStream_t s) {
  std::lock_guard<std::mutex> lock(f->p8_mu);
  if (f->p8_ready.load(std::memory_order_acquire)) return;
  const int g = (int)std::min<long long>(8192, (f->n_nodes + 255) / 256 + 1);
  int fb = 1;
  while ((1 << fb) - 1 < f->n_features) ++fb;
  if (fb <= 16 && f->n_nodes > 0 && f->n_classes < (1 << (32 - fb)) &&
      cudaMalloc(&f->pnodes8, sizeof(PNode8) * (f->n_nodes + 1)) == cudaSuccess) {
    int* flag = reinterpret_cast<int*>(f->pnodes8 + f->n_nodes);
    int h_flag = 1;
    if (cudaMemsetAsync(flag, 0, sizeof(int), s) == cudaSuccess) {
      k_to_pnodes8<<<g, 256, 0, s>>>(f->pnodes, f->n_nodes, fb, f->pnodes8, flag);
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess)
        h_flag = 1;
    }
    if (h_flag) {
      cudaGetLastError();
      cudaFree(f->pnodes8);
      f->pnodes8 = nullptr;
    } else {
      f->p8_bits = fb;
    }
  } else {
    cudaGetLastError();
    f->pnodes8 = nullptr;
  }
  f->p8_ready.store(true, std::memory_order_release);
}

static dml_status fit_entry(const dml_fit_desc* descs, int n, dml_forest** out, void* stream,
                            bool plain) {
  clear_error();
  if (!descs || !out || n <= 0) {
    set_error("null argument");
    return DML_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  alloc_fault_arm();
  try {
    std::vector<dml_forest*> fs = run_fit(descs, n, plain, s);
    for (int i = 0; i < n; ++i) out[i] = fs[i];
    return DML_OK;
  } catch (InvalidArg&) {
    return DML_ERR_INVALID_ARG;
  } catch (CudaError& e) {
    return e.e == cudaErrorMemoryAllocation ? DML_ERR_OOM : DML_ERR_CUDA;
  } catch (std::bad_alloc&) {
    set_error("host allocation failed");
    return DML_ERR_OOM;
  } catch (...) {
    set_error("internal error");
    return DML_ERR_INTERNAL;
  }
}

}  // namespace dml

// ---------------------------------------------------------------------------
// Allocation-free fit.
//
// For callers that cannot allocate device memory while they fit: a process
// whose device memory is owned by its own allocator (a framework's caching
// allocator, an arena sized at start-up) or partitioned by a budget, so that a
// library allocating on its own would take memory nobody accounted for, and a
// latency-critical service that keeps cudaMalloc / cudaFree (which can
// synchronise the device and can fail under fragmentation) out of its steady
// state.  Every working buffer of the fit comes from one file-scope device array
// of kNaArenaBytes (about 20 MiB) that every GPU which loads this library holds
// until the process exits; the model is written to device buffers the caller
// owns.  The problem must fit the array: at most kNaMaxRows rows,
// n_trees * n_rows <= kNaMaxSlots, at most kNaMaxClasses classes.  All calls
// share the array and keep the last call's contents there (each call clears
// what must start at zero), so calls whose work overlaps on the GPU (other
// streams, other host threads) race: serialise them.  The call synchronises its
// stream to read the validation result and then once per tree level (the next
// level's size).  The first call on a device sets the array up with that device
// current: it looks up the array's device address and uploads the n*ln(n) table
// once.
namespace dml {
namespace noalloc {
constexpr long long kNaMaxRows = 4096;
constexpr long long kNaMaxSlots = 65536;
constexpr int kNaMaxClasses = 8;
constexpr long long kNaMaxLevels = kNaMaxRows + 1;

constexpr long long align256(long long x) { return (x + 255) / 256 * 256; }

// byte offsets of the buffers inside the array
constexpr long long oErr = 0;
constexpr long long oMax = oErr + 256;
constexpr long long oLab = oMax + 256;
constexpr long long oQ = oLab + align256(4 * kNaMaxRows);
constexpr long long oH = oQ + align256(8 * kNaMaxRows);
constexpr long long oProb = oH + align256(8 * (kNaMaxRows + 1));
constexpr long long oTreeProb = oProb + align256(sizeof(ProbDesc));
constexpr long long oRowsA = oTreeProb + align256(4 * kNaMaxSlots);
constexpr long long oRowsB = oRowsA + align256(4 * kNaMaxSlots);
constexpr long long oWA = oRowsB + align256(4 * kNaMaxSlots);
constexpr long long oWB = oWA + align256(4 * kNaMaxSlots);
constexpr long long oBoot = oWB + align256(4 * kNaMaxSlots);
constexpr long long oNodes0 = oBoot + align256(4 * kNaMaxSlots);
constexpr long long oNodes1 = oNodes0 + align256(sizeof(LNode) * kNaMaxSlots);
constexpr long long oCnt0 = oNodes1 + align256(sizeof(LNode) * kNaMaxSlots);
constexpr long long oCnt1 = oCnt0 + align256(4 * kNaMaxClasses * kNaMaxSlots);
constexpr long long oRes0 = oCnt1 + align256(4 * kNaMaxClasses * kNaMaxSlots);
constexpr long long oRes1 = oRes0 + align256(sizeof(NodeRes) * kNaMaxSlots);
constexpr long long oResCnt = oRes1 + align256(sizeof(NodeRes) * kNaMaxSlots);
constexpr long long oChild = oResCnt + align256(4 * kNaMaxClasses * kNaMaxSlots);
constexpr long long oLeaf = oChild + align256(4 * (kNaMaxSlots + 1));
constexpr long long oParts = oLeaf + align256(4 * (kNaMaxSlots + 1));
constexpr long long oQueues = oParts + align256(8 * (kNaMaxSlots / (kScanBlock * kScanItems) + 2));
constexpr long long oQCount = oQueues + align256(4LL * kNumQ * kNaMaxSlots);
constexpr long long oSummary = oQCount + 256;
constexpr long long oStats = oSummary + 256;
constexpr long long oBases = oStats + 256;
constexpr long long oSeg = oBases + 256;
constexpr long long kNaArenaBytes = oSeg + 256;
}  // namespace noalloc
}  // namespace dml

static __device__ __align__(256) unsigned char g_noalloc_arena[dml::noalloc::kNaArenaBytes];

namespace dml {
namespace noalloc {
constexpr int kMaxDevices = 64;
static unsigned char* g_arena_dev[kMaxDevices];
static std::mutex g_arena_mu;

// The array's device address on the current device, set up once per device:
// cudaGetSymbolAddress with the device current (the array's name is only a
// host-side stand-in), then the n*ln(n) table for every row count the array
// admits (H[n] does not depend on the problem) uploaded to its slot.
static unsigned char* arena_on_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    set_error("no current CUDA device for the allocation-free fit");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_arena_mu);
  if (!g_arena_dev[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_arena);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaGetSymbolAddress of the allocation-free scratch failed: %s",
                cudaGetErrorString(e));
      return nullptr;
    }
    std::vector<long long> table((size_t)kNaMaxRows + 1);
    build_nlogn_table(kNaMaxRows, table.data());
    e = cudaMemcpy((unsigned char*)p + oH, table.data(), sizeof(long long) * table.size(),
                   cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("upload of the allocation-free n*ln(n) table failed: %s", cudaGetErrorString(e));
      return nullptr;
    }
    g_arena_dev[dev] = (unsigned char*)p;
  }
  return g_arena_dev[dev];
}
}  // namespace noalloc

static dml_status run_fit_noalloc(const dml_fit_desc& d, ClassifyNode* nodes_out,
                                  long long node_cap, float* probs_out, long long prob_cap,
                                  long long* n_nodes, long long* n_probs, cudaStream_t s) {
  using namespace noalloc;
  if (d.memory != DML_DEVICE) {
    set_error("the allocation-free fit takes device pointers only");
    return DML_ERR_INVALID_ARG;
  }
  if ((d.algo != DML_ALGO_RF && d.algo != DML_ALGO_ERT) ||
      (d.task != DML_CLASSIFICATION && d.task != DML_REGRESSION) || d.n_trees <= 0 ||
      d.n_rows <= 0 || d.n_features <= 0 || !d.samples || !d.targets || d.max_depth < 0 ||
      d.min_node_size < 0 || d.n_features_try < 0 || d.tree_offset < 0 ||
      (d.task == DML_CLASSIFICATION && d.n_classes < 1)) {
    set_error("invalid fit parameters");
    return DML_ERR_INVALID_ARG;
  }
  if (d.balanced != 0) {
    set_error("the allocation-free fit has no balanced sampling");
    return DML_ERR_INVALID_ARG;
  }
  if (d.n_rows > kNaMaxRows || (long long)d.n_trees * d.n_rows > kNaMaxSlots ||
      (d.task == DML_CLASSIFICATION && d.n_classes > kNaMaxClasses)) {
    set_error("the allocation-free fit holds at most %lld rows, n_trees * n_rows <= %lld and "
              "%d classes (got %lld rows, %d trees, %d classes)",
              kNaMaxRows, kNaMaxSlots, kNaMaxClasses, (long long)d.n_rows, d.n_trees,
              d.n_classes);
    return DML_ERR_INVALID_ARG;
  }
  const int C = d.task == DML_CLASSIFICATION ? d.n_classes : 1;
  const long long need_nodes = (long long)d.n_trees * (2 * d.n_rows - 1);
  const long long need_probs = (long long)d.n_trees * d.n_rows * C;
  if (!nodes_out || !probs_out || node_cap < need_nodes || prob_cap < need_probs) {
    set_error("output buffers too small: need %lld nodes and %lld probabilities", need_nodes,
              need_probs);
    return DML_ERR_INVALID_ARG;
  }
  unsigned char* A = arena_on_current_device();
  if (!A) {
    if (last_error_str()[0] == 0) set_error("no scratch for this device");
    return DML_ERR_CUDA;
  }
  try {
    ProbDesc P;
    std::memset(&P, 0, sizeof(P));
    P.N = d.n_rows;
    P.F = d.n_features;
    P.C = C;
    P.K = d.n_features_try > 0 ? d.n_features_try
                               : (int)std::round(std::log((double)d.n_features)) + 1;
    P.n_mand = std::min(P.K, P.F);
    P.n_opt = P.K < P.F ? std::min(P.F - P.K, 10) : 0;
    if (P.n_mand + P.n_opt > kMaxTries) {
      set_error("at most %d tries per node", kMaxTries);
      return DML_ERR_INVALID_ARG;
    }
    P.max_depth = d.max_depth;
    P.min_node_size = d.min_node_size;
    P.min_leaf = std::max(1, d.min_leaf);
    P.algo = d.algo;
    P.task = d.task;
    P.seed = d.seed;
    P.n_trees = d.n_trees;
    P.tree_key0 = d.tree_offset;
    P.tree0 = 0;
    P.ent0 = 0;
    P.X = d.samples;
    P.lab = (int*)(A + oLab);
    P.q = (long long*)(A + oQ);
    const long long total_slots = (long long)d.n_trees * d.n_rows;
    const int Cmax = C;
    const int CW = Cmax <= 2 ? 1 : Cmax <= 4 ? 2 : 4;
    int* d_err = (int*)(A + oErr);
    unsigned* d_max = (unsigned*)(A + oMax);
    DML_CK(cudaMemsetAsync(d_err, 0, 16, s));
    DML_CK(cudaMemsetAsync(d_max, 0, 4, s));
    const long long nx = P.N * P.F;
    k_validate<<<(int)std::min<long long>(4096, (nx + 255) / 256), 256, 0, s>>>(
        d.samples, nx, d.targets, P.N, P.task, P.C, d_err, d_max);
    DML_CK(cudaGetLastError());
    int h_err = 0;
    unsigned h_max = 0;
    DML_CK(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    DML_CK(cudaMemcpyAsync(&h_max, d_max, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    DML_CK(cudaStreamSynchronize(s));
    if (h_err & 1) {
      set_error("samples hold NaN or infinite values (the missing-value marker is -FLT_MAX)");
      return DML_ERR_INVALID_ARG;
    }
    if (h_err & 2) {
      set_error("classification targets must be integers in [0, n_classes)");
      return DML_ERR_INVALID_ARG;
    }
    if (h_err & 4) {
      set_error("regression targets hold NaN or infinite values");
      return DML_ERR_INVALID_ARG;
    }
    float mx;
    std::memcpy(&mx, &h_max, 4);
    P.S = P.task == 1 ? quant_scale_from_max(mx, P.N) : 0;
    k_prep_targets<<<(int)std::min<long long>(4096, (P.N + 255) / 256), 256, 0, s>>>(
        d.targets, P.N, P.task, P.S, P.lab == nullptr ? nullptr : (int*)(A + oLab),
        (long long*)(A + oQ));
    DML_CK(cudaGetLastError());
    // the table was uploaded when the array was set up on this device
    const long long* H = P.task == 0 ? (const long long*)(A + oH) : nullptr;
    ProbDesc* d_probs = (ProbDesc*)(A + oProb);
    DML_CK(cudaMemcpyAsync(d_probs, &P, sizeof(ProbDesc), cudaMemcpyHostToDevice, s));
    // every tree belongs to problem 0
    int* d_tree_prob = (int*)(A + oTreeProb);
    DML_CK(cudaMemsetAsync(d_tree_prob, 0, sizeof(int) * d.n_trees, s));
    int* rowsA = (int*)(A + oRowsA);
    int* rowsB = (int*)(A + oRowsB);
    int* wA = d.algo == DML_ALGO_RF ? (int*)(A + oWA) : nullptr;
    int* wB = d.algo == DML_ALGO_RF ? (int*)(A + oWB) : nullptr;
    int* wcnt = (int*)(A + oBoot);
    LNode* cur = (LNode*)(A + oNodes0);
    LNode* nxt = (LNode*)(A + oNodes1);
    int* cnt_cur = (int*)(A + oCnt0);
    int* cnt_nxt = (int*)(A + oCnt1);
    NodeRes* res_cur = (NodeRes*)(A + oRes0);
    NodeRes* res_nxt = (NodeRes*)(A + oRes1);
    int* res_cnt = (int*)(A + oResCnt);
    int* childpos = (int*)(A + oChild);
    int* leafpos = (int*)(A + oLeaf);
    int2* parts = (int2*)(A + oParts);
    int* d_qcount = (int*)(A + oQCount);
    int* d_summary = (int*)(A + oSummary);
    long long* d_stats = (long long*)(A + oStats);
    long long* fbase[2] = {(long long*)(A + oBases), (long long*)(A + oBases) + 1};
    long long* lbase[2] = {(long long*)(A + oBases) + 2, (long long*)(A + oBases) + 3};
    Seg* seg = (Seg*)(A + oSeg);
    DML_CK(cudaMemsetAsync(A + oBases, 0, 4 * sizeof(long long), s));
    DML_CK(cudaMemsetAsync(d_stats, 0, 4 * sizeof(long long), s));
    DML_CK(cudaMemsetAsync(d_qcount, 0, sizeof(int) * kNumQ, s));
    Queues Q;
    for (int i = 0; i < kNumQ; ++i) Q.list[i] = (int*)(A + oQueues) + (long long)i * kNaMaxSlots;
    Q.count = d_qcount;
    Q.rf_small_cap = kSmemCap;
    Q.rf_warp_max = 256;
    if (d.algo == DML_ALGO_RF) {
      DML_CK(cudaMemsetAsync(wcnt, 0, sizeof(int) * total_slots, s));
      const int chunk = 1 << 16;
      dim3 g((unsigned)((P.N + chunk - 1) / chunk), (unsigned)d.n_trees);
      k_boot_count<<<g, 256, 0, s>>>(d_probs, d_tree_prob, wcnt, chunk);
      DML_CK(cudaGetLastError());
    }
    k_roots<1024><<<d.n_trees, 1024, 0, s>>>(d_probs, d_tree_prob, wcnt, rowsA, wA, cur,
                                             cnt_cur, Cmax, res_cur, Q, d_stats);
    DML_CK(cudaGetLastError());
    int qc[kNumQ];
    DML_CK(cudaMemcpyAsync(qc, d_qcount, sizeof(int) * kNumQ, cudaMemcpyDeviceToHost, s));
    DML_CK(cudaStreamSynchronize(s));
    int n = d.n_trees;
    long long log_base = 0, plog_base = 0;
    int depth = 0;
    while (n > 0) {
      if (depth >= kNaMaxLevels) {
        set_error("tree deeper than the allocation-free fit supports");
        return DML_ERR_INTERNAL;
      }
      LevelArgs a;
      std::memset(&a, 0, sizeof(a));
      a.probs = d_probs;
      a.nodes = cur;
      a.cnt = cnt_cur;
      a.Cmax = Cmax;
      a.res = res_cur;
      a.res_cnt = res_cnt;
      a.rowsA = rowsA;
      a.wA = wA;
      a.rowsB = rowsB;
      a.wB = wB;
      a.H = H;
      a.stats = d_stats;
      a.smem_cap = kSmemCap;
      for (int q = 0; q < kNumQ; ++q) {
        if (qc[q] <= 0) continue;
        if (q == kQRfBig) {
          set_error("internal: node too large for the allocation-free fit");
          return DML_ERR_INTERNAL;
        }
        a.work = Q.list[q];
        launch_search(CW, q, a, qc[q], s);
      }
      const int nparts = (n + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems);
      k_scan_part<<<nparts, kScanBlock, 0, s>>>(res_cur, n, parts);
      k_scan_top<<<1, kScanBlock, 0, s>>>(parts, nparts, childpos, leafpos, n, d_summary);
      k_scan_apply<<<nparts, kScanBlock, 0, s>>>(res_cur, n, parts, childpos, leafpos);
      DML_CK(cudaGetLastError());
      DML_CK(cudaMemsetAsync(d_qcount, 0, sizeof(int) * kNumQ, s));
      DML_CK(cudaMemcpyAsync(fbase[(depth + 1) & 1], fbase[depth & 1], sizeof(long long),
                             cudaMemcpyDeviceToDevice, s));
      DML_CK(cudaMemcpyAsync(lbase[(depth + 1) & 1], lbase[depth & 1], sizeof(long long),
                             cudaMemcpyDeviceToDevice, s));
      EmitArgs e;
      e.probs = d_probs;
      e.cur = cur;
      e.cnt = cnt_cur;
      e.res = res_cur;
      e.res_cnt = res_cnt;
      e.childpos = childpos;
      e.leafpos = leafpos;
      e.n = n;
      e.Cmax = Cmax;
      e.log_base = log_base;
      e.plog_base = plog_base;
      e.node_log = nodes_out;   // one forest: log order is the model order
      e.gain_log = nullptr;
      e.prob_log = probs_out;   // Cmax == C: leaf payloads packed
      e.fbase_cur = fbase[depth & 1];
      e.lbase_cur = lbase[depth & 1];
      e.fbase_next = fbase[(depth + 1) & 1];
      e.lbase_next = lbase[(depth + 1) & 1];
      e.seg = seg;
      e.next = nxt;
      e.next_cnt = cnt_nxt;
      e.next_res = res_nxt;
      e.Q = Q;
      e.stats = d_stats;
      k_emit<<<(n + 255) / 256, 256, 0, s>>>(e);
      DML_CK(cudaGetLastError());
      int summary[2];
      DML_CK(cudaMemcpyAsync(summary, d_summary, sizeof(summary), cudaMemcpyDeviceToHost, s));
      DML_CK(cudaMemcpyAsync(qc, d_qcount, sizeof(int) * kNumQ, cudaMemcpyDeviceToHost, s));
      DML_CK(cudaStreamSynchronize(s));
      log_base += n;
      plog_base += summary[1];
      n = summary[0];
      std::swap(cur, nxt);
      std::swap(cnt_cur, cnt_nxt);
      std::swap(res_cur, res_nxt);
      std::swap(rowsA, rowsB);
      std::swap(wA, wB);
      ++depth;
    }
    *n_nodes = log_base;
    *n_probs = plog_base * C;
    return DML_OK;
  } catch (CudaError& e) {
    return DML_ERR_CUDA;
  }
}

}  // namespace dml

extern "C" {

dml_status dml_fit(const dml_fit_desc* desc, dml_forest** out, void* stream) {
  return dml::fit_entry(desc, 1, out, stream, false);
}

dml_status dml_fit_batched(int32_t n, const dml_fit_desc* descs, dml_forest** out, void* stream) {
  return dml::fit_entry(descs, n, out, stream, false);
}

dml_status dml_fit_plain(const dml_fit_desc* desc, dml_forest** out, void* stream) {
  return dml::fit_entry(desc, 1, out, stream, true);
}

dml_status dml_fit_noalloc(const dml_fit_desc* desc, void* node_array, int64_t node_capacity,
                           float* probs, int64_t prob_capacity, int64_t* n_nodes,
                           int64_t* n_probs, void* stream) {
  dml::clear_error();
  if (!desc || !n_nodes || !n_probs) {
    dml::set_error("null argument");
    return DML_ERR_INVALID_ARG;
  }
  long long nn = 0, np = 0;
  dml_status st = dml::run_fit_noalloc(*desc, (dml::ClassifyNode*)node_array, node_capacity,
                                       probs, prob_capacity, &nn, &np, (cudaStream_t)stream);
  *n_nodes = nn;
  *n_probs = np;
  return st;
}

dml_status dml_last_fit_stats(dml_fit_stats* stats) {
  if (!stats) return DML_ERR_INVALID_ARG;
  *stats = dml::g_last_stats;
  return DML_OK;
}

const char* dml_last_error(void) { return dml::last_error_str(); }

}  // extern "C"
