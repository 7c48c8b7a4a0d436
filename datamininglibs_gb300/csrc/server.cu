// Prediction server: resident forests, continuous batching, HBM-budget
// admission.  No reference counterpart (the reference predicts one data frame
// per call, gpudte_algorithm.cc:270-331).
//
// Two lanes, each with n_streams batch slots and its own worker thread:
//  * small lane (requests of at most small_rows rows): high-priority streams;
//    a batch packs whole requests of any forests into 16-row tiles whose rows
//    are walked by 8 threads each (one eighth of the trees per thread), which
//    cuts a row's chain of dependent node loads by 8;
//  * large lane: low-priority streams; requests are cut into slices of at most
//    max_batch_rows rows and a batch packs slices into the same 16-row tiles
//    (128-row tiles, one thread per row walking every tree, for forests whose
//    rows or per-tree values do not fit a tile's shared memory).
// Blocks of a low-priority launch are short (one tile), so a small batch waits
// for at most one block per SM.  Requests that arrive while batches run join
// the next batch of their lane as soon as a slot and budget free up.  A small
// request whose input and output are both pinned is read and written by the
// kernel in place through mapped pointers (no copies); other pinned buffers
// are copied by DMA, pageable ones are staged through pinned slot buffers.  A
// request completes when all of its rows are back.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "dml_device.cuh"
#include "engine.h"

namespace dml {

const char* last_error_str();
void clear_error();
void init_pool_once();

namespace {

constexpr int kTileRows = 128;      // large lane: rows per tile (one thread per row)
constexpr int kSplit = 8;           // small lane: threads per row
constexpr int kSplitRows = kTileRows / kSplit;
// a feature's 16 rows padded to 17 words in shared memory: lanes reading
// different features of one row meet different banks
constexpr int kSplitStride = kSplitRows + 1;
constexpr int kSplitMaxTrees = 512;  // small-lane regression keeps [rows][trees] leaf values
constexpr int kSplitMaxFeatures = 1024;  // small-lane tiles stage [features][16 rows] in shared memory
constexpr int kSplitSmem = 112 * 1024;  // >= 4 * (17 * 1024 features + 16 * 512 trees)

struct PredTile {
  const PNode* nodes;
  const float* X;   // feature-major rows of the slice: X[f * n + i]
  float* out;       // [n * width]
  long long n;      // row pitch of X (rows of the slice or request)
  int row0, rows;   // this tile
  int n_trees, C, task, F;
};

// Large lane: a thread walks every tree for its row (tree order, so regression
// sums match dml_predict bit for bit).
__global__ void __launch_bounds__(kTileRows) k_predict_tiles(const PredTile* __restrict__ tiles) {
  extern __shared__ int votes[];  // [kTileRows][C]
  const PredTile t = tiles[blockIdx.x];
  const int r = threadIdx.x;
  const bool act = r < t.rows;
  const long long row = (long long)t.row0 + r;
  int* my = votes + r * t.C;
  if (t.task == 0)
    for (int c = 0; c < t.C; ++c) my[c] = 0;
  float acc = 0.0f;
  if (act) {
    auto xr = [&](int f) { return __ldg(t.X + (long long)f * t.n + row); };
    int k = 0;
    for (; k + 4 <= t.n_trees; k += 4) {  // four trees in lockstep, consumed in order
      int4 lf[4];
      walk_trees<4>(t.nodes, k, xr, lf);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (t.task == 0)
          my[lf[j].y] += 1;
        else
          acc = __fadd_rn(acc, __int_as_float(lf[j].z));
      }
    }
    for (; k < t.n_trees; ++k) {
      int4 lf[1];
      walk_trees<1>(t.nodes, k, xr, lf);
      if (t.task == 0)
        my[lf[0].y] += 1;
      else
        acc = __fadd_rn(acc, __int_as_float(lf[0].z));
    }
    if (t.task == 0)
      for (int c = 0; c < t.C; ++c) t.out[row * t.C + c] = (float)my[c];
    else
      t.out[row] = acc;
  }
}

// Small lane: the tile's 16 rows are staged in shared memory (from device
// staging or straight from the caller's pinned buffer), then 8 threads per row
// walk trees g, g+8, ..., four of them in lockstep (four node loads in
// flight: a request's latency is the chain of dependent node loads); votes
// meet in shared memory (integer counts, order-free); regression leaf values
// are kept per tree and summed in tree order by one thread.
__global__ void __launch_bounds__(kTileRows) k_predict_tiles_split(
    const PredTile* __restrict__ tiles) {
  extern __shared__ int sm[];  // xs [F][kSplitStride], then votes [kSplitRows][C] or values
  const PredTile t = tiles[blockIdx.x];
  const int g = threadIdx.x % kSplit;
  const int r = threadIdx.x / kSplit;
  const bool act = r < t.rows;
  const long long row = (long long)t.row0 + r;
  float* xs = reinterpret_cast<float*>(sm);
  int* acc = sm + t.F * kSplitStride;
  for (int e = threadIdx.x; e < t.F * kSplitRows; e += kTileRows) {
    const int f = e / kSplitRows, rr = e % kSplitRows;
    xs[f * kSplitStride + rr] = rr < t.rows ? t.X[(long long)f * t.n + t.row0 + rr] : 0.0f;
  }
  if (t.task == 0)
    for (int i = threadIdx.x; i < kSplitRows * t.C; i += kTileRows) acc[i] = 0;
  __syncthreads();
  float* vals = reinterpret_cast<float*>(acc) + r * t.n_trees;
  if (act) {
    const int4* nd = reinterpret_cast<const int4*>(t.nodes);
    for (int k0 = g; k0 < t.n_trees; k0 += 4 * kSplit) {
      int4 p[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = k0 + j * kSplit;
        p[j] = k < t.n_trees ? __ldg(nd + k) : make_int4(-1, 0, 0, 0);
      }
      bool more = true;
      while (more) {
        more = false;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (p[j].x >= 0) {
            const float x = xs[p[j].y * kSplitStride + r];
            p[j] = __ldg(nd + (goes_left(x, __int_as_float(p[j].z)) ? p[j].x : p[j].x + 1));
            more = more || p[j].x >= 0;
          }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = k0 + j * kSplit;
        if (k < t.n_trees) {
          if (t.task == 0)
            atomicAdd(&acc[r * t.C + p[j].y], 1);
          else
            vals[k] = __int_as_float(p[j].z);
        }
      }
    }
  }
  __syncthreads();
  if (act) {
    if (t.task == 0) {
      for (int c = g; c < t.C; c += kSplit) t.out[row * t.C + c] = (float)acc[r * t.C + c];
    } else if (g == 0) {
      float sum = 0.0f;
      for (int k = 0; k < t.n_trees; ++k) sum = __fadd_rn(sum, vals[k]);
      t.out[row] = sum;
    }
  }
}

using Clock = std::chrono::steady_clock;

struct Request {
  long long id;
  int forest;
  const float* samples;
  long long n;
  float* out;
  Clock::time_point t_submit;
  int width, n_features;
  bool pinned_in, pinned_out;
  bool mapped = false;                 // the small-lane kernel reads and writes the caller's
  const float* d_samples = nullptr;    // pinned buffers through these device pointers
  float* d_out = nullptr;
  long long next_row = 0;   // first row not yet handed to a batch
  long long rows_left = 0;  // rows not yet completed
};

struct Piece {  // rows [row0, row0 + rows) of a request in a batch
  std::shared_ptr<Request> req;
  long long row0, rows;
  size_t in_off, out_off;
};

struct Batch {
  std::vector<Piece> pieces;
  cudaEvent_t done = nullptr;
  bool busy = false;
};

struct Slot {
  cudaStream_t stream = nullptr;
  char* h_in = nullptr;   // pinned staging
  char* h_out = nullptr;
  char* d_in = nullptr;
  char* d_out = nullptr;
  PredTile* d_tiles = nullptr;
  PredTile* h_tiles = nullptr;
  size_t cap = 0;         // bytes of each direction
  int tile_cap = 0;
  bool small = false;
  Batch batch;
};

}  // namespace
}  // namespace dml

struct dml_server {
  dml_server_config cfg;
  int device = 0;
  long long small_rows = 4096;
  std::vector<const dml_forest*> forests;
  std::mutex mu;
  std::condition_variable cv_work[2], cv_done;  // cv_work[1]: small lane, [0]: large lane
  std::deque<std::shared_ptr<dml::Request>> q_small, q_large;
  std::unordered_map<long long, double> done;  // id -> latency ms
  std::vector<double> latencies;
  long long next_id = 1, completed = 0, rows = 0, launches = 0, rejected = 0;
  dml::Clock::time_point first_submit, last_done;
  bool have_first = false, stop = false;
  std::vector<dml::Slot> slots;  // n_streams small-lane slots, then n_streams large-lane
  std::thread worker[2];  // [1] drives the small lane's slots, [0] the large lane's
  size_t small_cap = 0, large_cap = 0;
};

namespace dml {
namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

bool split_ok(const dml_forest* f) {
  return f->n_features <= kSplitMaxFeatures &&
         (f->task == DML_CLASSIFICATION || f->n_trees <= kSplitMaxTrees);
}

// Completes the lane's finished batches; returns true if any slot finished.
bool reap(dml_server* s, bool small) {
  bool any = false;
  for (Slot& sl : s->slots) {
    if (sl.small != small || !sl.batch.busy) continue;
    if (cudaEventQuery(sl.batch.done) != cudaSuccess) continue;
    for (const Piece& p : sl.batch.pieces) {
      const Request& r = *p.req;
      if (!r.pinned_out && !(sl.small && r.mapped))
        std::memcpy(r.out + p.row0 * r.width, sl.h_out + p.out_off,
                    sizeof(float) * p.rows * r.width);
    }
    auto now = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (const Piece& p : sl.batch.pieces) {
        Request& r = *p.req;
        r.rows_left -= p.rows;
        if (r.rows_left == 0) {
          double ms = std::chrono::duration<double, std::milli>(now - r.t_submit).count();
          s->done[r.id] = ms;
          s->latencies.push_back(ms);
          s->completed++;
          s->rows += r.n;
        }
      }
      s->last_done = now;
    }
    s->cv_done.notify_all();
    sl.batch.pieces.clear();
    sl.batch.busy = false;
    any = true;
  }
  return any;
}

// Packs queued work of the slot's lane into the slot and launches it.
bool launch_batch(dml_server* s, Slot& sl) {
  Batch& b = sl.batch;
  b.pieces.clear();
  // rows per tile of a request's forest: 16-row staged tiles, 8 threads a row,
  // wherever the forest allows them; 128-row tiles (a thread a row) otherwise
  auto tile_rows_of = [&](const dml_forest* f) {
    return sl.small || split_ok(f) ? kSplitRows : kTileRows;
  };
  const long long max_rows = sl.small ? std::max<long long>(s->small_rows * 16, 65536)
                                      : s->cfg.max_batch_rows;
  size_t in_used = 0, out_used = 0;
  long long rows = 0;
  int tiles = 0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto& q = sl.small ? s->q_small : s->q_large;
    while (!q.empty() && rows < max_rows) {
      std::shared_ptr<Request> r = q.front();
      const int tile_rows = tile_rows_of(s->forests[r->forest]);
      const long long row_in = (long long)sizeof(float) * r->n_features;
      const long long row_out = (long long)sizeof(float) * r->width;
      // rows of this request that fit the batch's remaining room (64 rows of
      // slack cover the 256-byte alignment of each piece)
      long long room = max_rows - rows;
      room = std::min(room, (long long)(sl.cap - in_used) / row_in - 64);
      room = std::min(room, (long long)(sl.cap - out_used) / row_out - 64);
      room = std::min(room, (long long)(sl.tile_cap - tiles) * tile_rows);
      const long long want = r->n - r->next_row;
      const bool direct = sl.small && r->mapped;  // no staging room needed
      if (direct)
        room = std::min(max_rows - rows, (long long)(sl.tile_cap - tiles) * tile_rows);
      if (room <= 0 || (sl.small && room < want)) break;  // small requests are not split
      const long long take = std::min(want, room);
      Piece p{r, r->next_row, take, in_used, out_used};
      if (!direct) {
        in_used += align256(row_in * take);
        out_used += align256(row_out * take);
      }
      rows += take;
      tiles += (int)((take + tile_rows - 1) / tile_rows);
      r->next_row += take;
      if (r->next_row == r->n) q.pop_front();
      b.pieces.push_back(std::move(p));
    }
  }
  if (b.pieces.empty()) return false;
  cudaStream_t st = sl.stream;
  // inputs to the device
  for (const Piece& p : b.pieces) {
    const Request& r = *p.req;
    const bool direct = sl.small && r.mapped;
    char* d_stage = sl.d_in + p.in_off;
    const size_t rb = sizeof(float) * p.rows;
    if (direct) {
      // the kernel reads the caller's buffer
    } else if (r.pinned_in) {
      if (p.rows == r.n)
        cudaMemcpyAsync(d_stage, r.samples, rb * r.n_features, cudaMemcpyHostToDevice, st);
      else
        cudaMemcpy2DAsync(d_stage, rb, r.samples + p.row0, sizeof(float) * r.n, rb, r.n_features,
                          cudaMemcpyHostToDevice, st);
    } else {
      char* h = sl.h_in + p.in_off;
      if (p.rows == r.n)
        std::memcpy(h, r.samples, rb * r.n_features);
      else
        for (int j = 0; j < r.n_features; ++j)
          std::memcpy(h + rb * j, r.samples + (long long)j * r.n + p.row0, rb);
      cudaMemcpyAsync(d_stage, h, rb * r.n_features, cudaMemcpyHostToDevice, st);
    }
  }
  // tiles: the staged (16-row) ones first, then the 128-row ones
  int nt = 0, n_split = 0;
  int shm_split = sizeof(int), shm_rows = sizeof(int);
  for (int pass = 0; pass < 2; ++pass) {
    for (const Piece& p : b.pieces) {
      const Request& r = *p.req;
      const dml_forest* f = s->forests[r.forest];
      const int tile_rows = tile_rows_of(f);
      if ((tile_rows == kSplitRows) != (pass == 0)) continue;
      const bool direct = sl.small && r.mapped;
      for (long long r0 = 0; r0 < p.rows; r0 += tile_rows) {
        PredTile& t = sl.h_tiles[nt++];
        t.nodes = f->pnodes;
        t.X = direct ? r.d_samples : (const float*)(sl.d_in + p.in_off);
        t.out = direct ? r.d_out : (float*)(sl.d_out + p.out_off);
        t.n = direct ? r.n : p.rows;
        t.row0 = (int)r0;
        t.rows = (int)std::min<long long>(tile_rows, p.rows - r0);
        t.n_trees = f->n_trees;
        t.C = r.width;
        t.task = f->task;
        t.F = f->n_features;
      }
      if (pass == 0)
        shm_split = std::max(
            shm_split, (int)sizeof(int) * (kSplitStride * f->n_features +
                                           (f->task == DML_CLASSIFICATION ? kSplitRows * r.width
                                                                          : kSplitRows * f->n_trees)));
      else
        shm_rows = std::max(
            shm_rows, (int)sizeof(int) * (f->task == DML_CLASSIFICATION ? kTileRows * r.width : 1));
    }
    if (pass == 0) n_split = nt;
  }
  cudaMemcpyAsync(sl.d_tiles, sl.h_tiles, sizeof(PredTile) * nt, cudaMemcpyHostToDevice, st);
  if (n_split > 0) k_predict_tiles_split<<<n_split, kTileRows, shm_split, st>>>(sl.d_tiles);
  if (nt > n_split)
    k_predict_tiles<<<nt - n_split, kTileRows, shm_rows, st>>>(sl.d_tiles + n_split);
  for (const Piece& p : b.pieces) {
    const Request& r = *p.req;
    const size_t ob = sizeof(float) * p.rows * r.width;
    if (sl.small && r.mapped) continue;  // written by the kernel
    if (r.pinned_out)
      cudaMemcpyAsync(r.out + p.row0 * r.width, sl.d_out + p.out_off, ob, cudaMemcpyDeviceToHost,
                      st);
    else
      cudaMemcpyAsync(sl.h_out + p.out_off, sl.d_out + p.out_off, ob, cudaMemcpyDeviceToHost, st);
  }
  cudaEventRecord(b.done, st);
  b.busy = true;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->launches++;
  }
  return true;
}

// One worker per lane, so that the small lane's launches and completions never
// wait behind the large lane's host work (staging, result copies).
void worker_main(dml_server* s, bool small) {
  cudaSetDevice(s->device);
  auto& q = small ? s->q_small : s->q_large;
  auto& cv = s->cv_work[small ? 1 : 0];
  const auto pace = std::chrono::microseconds(s->cfg.max_wait_us);
  Clock::time_point last_launch = Clock::now() - std::chrono::seconds(1);
  while (true) {
    bool progressed = reap(s, small);
    bool idle = true;
    for (Slot& sl : s->slots)
      if (sl.small == small) idle = idle && !sl.batch.busy;
    for (Slot& sl : s->slots) {
      if (sl.small != small || sl.batch.busy) continue;
      bool pending;
      long long waiting = 0;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        pending = !q.empty();
        if (small)
          for (auto& r : q) waiting += r->n - r->next_row;
      }
      if (!pending) continue;
      // with batches in flight, the small lane launches the next one after
      // max_wait_us (or a batch's worth of rows), so that requests arriving
      // meanwhile share it
      if (small && !idle && Clock::now() - last_launch < pace && waiting < s->small_rows) continue;
      if (small && idle && s->cfg.max_wait_us > 0) {
        // an idle lane lets a batch fill briefly while few rows wait
        std::unique_lock<std::mutex> lk(s->mu);
        long long waiting = 0;
        for (auto& r : q) waiting += r->n - r->next_row;
        if (waiting < s->small_rows)
          cv.wait_for(lk, std::chrono::microseconds(s->cfg.max_wait_us));
        idle = false;
      }
      if (launch_batch(s, sl)) {
        progressed = true;
        idle = false;
        if (small) last_launch = Clock::now();
      }
    }
    bool any_busy = false;
    for (Slot& sl : s->slots)
      if (sl.small == small) any_busy |= sl.batch.busy;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop && q.empty() && !any_busy) break;
    if (!progressed) {
      if (any_busy) {
        // the small lane polls its batches without sleeping (a sleep rounds up
        // to tens of microseconds); the large lane naps between polls
        lk.unlock();
        if (small)
          std::this_thread::yield();
        else
          std::this_thread::sleep_for(std::chrono::microseconds(10));
      } else {
        cv.wait_for(lk, std::chrono::milliseconds(5), [&] { return s->stop || !q.empty(); });
      }
    }
  }
}

}  // namespace
}  // namespace dml

using namespace dml;

extern "C" {

dml_status dml_server_create(const dml_server_config* cfg, dml_server** out) {
  clear_error();
  if (!cfg || !out || cfg->hbm_budget_bytes <= 0 || cfg->max_batch_rows <= 0 ||
      cfg->n_streams <= 0 || cfg->n_streams > 32 || cfg->max_wait_us < 0 || cfg->small_rows < 0) {
    set_error("invalid server configuration");
    return DML_ERR_INVALID_ARG;
  }
  init_pool_once();
  alloc_fault_arm();
  dml_server* s = new dml_server();
  s->cfg = *cfg;
  s->small_rows = cfg->small_rows > 0 ? cfg->small_rows : 4096;
  cudaGetDevice(&s->device);
  int prio_low = 0, prio_high = 0;
  cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
  cudaFuncSetAttribute(k_predict_tiles_split, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       kSplitSmem);
  // a quarter of the budget for the small lane, the rest for the large lane;
  // each slot's share is split between inputs and outputs
  const int ns = cfg->n_streams;
  s->small_cap = (size_t)(cfg->hbm_budget_bytes / 4 / ns / 2) & ~(size_t)255;
  s->large_cap = (size_t)(cfg->hbm_budget_bytes * 3 / 4 / ns / 2) & ~(size_t)255;
  s->slots.resize(2 * ns);
  bool ok = s->small_cap >= (1 << 16) && s->large_cap >= (1 << 16);
  for (int i = 0; i < 2 * ns && ok; ++i) {
    Slot& sl = s->slots[i];
    sl.small = i < ns;
    sl.cap = sl.small ? s->small_cap : s->large_cap;
    const long long lane_rows = sl.small ? std::max<long long>(s->small_rows * 16, 65536)
                                         : cfg->max_batch_rows;
    sl.tile_cap = (int)std::min<long long>(1 << 22, lane_rows / kSplitRows + 1024);
    auto dmalloc = [](void* p, size_t bytes) {  // device buffers; injectable failure
      return !alloc_fault_fire() && cudaMalloc((void**)p, bytes) == cudaSuccess;
    };
    ok = cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking,
                                      sl.small ? prio_high : prio_low) == cudaSuccess &&
         cudaMallocHost(&sl.h_in, sl.cap) == cudaSuccess &&
         cudaMallocHost(&sl.h_out, sl.cap) == cudaSuccess &&
         cudaMallocHost(&sl.h_tiles, sizeof(PredTile) * sl.tile_cap) == cudaSuccess &&
         dmalloc(&sl.d_in, sl.cap) && dmalloc(&sl.d_out, sl.cap) &&
         dmalloc(&sl.d_tiles, sizeof(PredTile) * sl.tile_cap) &&
         cudaEventCreateWithFlags(&sl.batch.done, cudaEventDisableTiming) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    set_error("could not allocate the server's streams and staging buffers%s",
              alloc_fault_note());
    s->stop = true;
    dml_server_destroy(s);
    return DML_ERR_OOM;
  }
  s->worker[0] = std::thread(worker_main, s, false);
  s->worker[1] = std::thread(worker_main, s, true);
  *out = s;
  return DML_OK;
}

dml_status dml_server_add_forest(dml_server* s, const dml_forest* forest, int32_t* forest_id) {
  clear_error();
  if (!s || !forest || !forest_id || !forest->pnodes) {
    set_error("invalid arguments");
    return DML_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  s->forests.push_back(forest);
  *forest_id = (int32_t)s->forests.size() - 1;
  return DML_OK;
}

dml_status dml_server_submit(dml_server* s, int32_t forest_id, const float* samples,
                             int64_t n_rows, float* out, int64_t* request_id) {
  clear_error();
  if (!s || !samples || !out || !request_id || n_rows <= 0 || n_rows > (1LL << 31)) {
    set_error("invalid request");
    return DML_ERR_INVALID_ARG;
  }
  auto r = std::make_shared<Request>();
  const bool pin_in = is_pinned(samples), pin_out = is_pinned(out);
  if (pin_in && pin_out) {
    void* dx = nullptr;
    void* dy = nullptr;
    if (cudaHostGetDevicePointer(&dx, (void*)samples, 0) == cudaSuccess &&
        cudaHostGetDevicePointer(&dy, (void*)out, 0) == cudaSuccess) {
      r->mapped = true;
      r->d_samples = (const float*)dx;
      r->d_out = (float*)dy;
    } else {
      cudaGetLastError();
    }
  }
  bool to_small = false;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (forest_id < 0 || forest_id >= (int32_t)s->forests.size()) {
      set_error("unknown forest id %d", forest_id);
      return DML_ERR_INVALID_ARG;
    }
    const dml_forest* f = s->forests[forest_id];
    r->width = f->task == DML_CLASSIFICATION ? f->n_classes : 1;
    r->n_features = f->n_features;
    // admission: a small request must fit a small slot whole; a large one is
    // sliced, and a slice of 128 rows must fit a large slot
    const size_t row_in = sizeof(float) * f->n_features, row_out = sizeof(float) * r->width;
    const bool small_fit = n_rows <= s->small_rows && split_ok(f) &&
                           align256(row_in * n_rows) + 64 * row_in <= s->small_cap &&
                           align256(row_out * n_rows) + 64 * row_out <= s->small_cap;
    if (!small_fit && (192 * row_in > s->large_cap || 192 * row_out > s->large_cap)) {
      s->rejected++;
      set_error("a row of forest %d does not fit the server's device budget", forest_id);
      return DML_ERR_BUDGET;
    }
    r->id = s->next_id++;
    r->forest = forest_id;
    r->samples = samples;
    r->n = n_rows;
    r->out = out;
    r->pinned_in = pin_in;
    r->pinned_out = pin_out;
    r->rows_left = n_rows;
    r->t_submit = Clock::now();
    if (!s->have_first) {
      s->first_submit = r->t_submit;
      s->have_first = true;
    }
    (small_fit ? s->q_small : s->q_large).push_back(r);
    *request_id = r->id;
    to_small = small_fit;
  }
  s->cv_work[to_small ? 1 : 0].notify_one();
  return DML_OK;
}

dml_status dml_server_poll(dml_server* s, int64_t request_id, double* latency_ms) {
  if (!s) return DML_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->done.find(request_id);
  if (it == s->done.end()) return DML_ERR_NOT_READY;
  if (latency_ms) *latency_ms = it->second;
  s->done.erase(it);
  return DML_OK;
}

dml_status dml_server_wait(dml_server* s, int64_t request_id, double* latency_ms) {
  if (!s) return DML_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (request_id <= 0 || request_id >= s->next_id) {
    set_error("unknown request id");
    return DML_ERR_INVALID_ARG;
  }
  // bounded wait: a request never takes longer than this unless the GPU stalls
  const auto deadline = Clock::now() + std::chrono::seconds(120);
  while (s->done.find(request_id) == s->done.end()) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout &&
        s->done.find(request_id) == s->done.end()) {
      set_error("request %lld timed out", (long long)request_id);
      return DML_ERR_TIMEOUT;
    }
  }
  auto it = s->done.find(request_id);
  if (latency_ms) *latency_ms = it->second;
  s->done.erase(it);
  return DML_OK;
}

dml_status dml_server_stats_get(dml_server* s, dml_server_stats* st) {
  if (!s || !st) return DML_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(st, 0, sizeof(*st));
  st->completed = s->completed;
  st->rows = s->rows;
  st->launches = s->launches;
  st->rejected = s->rejected;
  if (!s->latencies.empty()) {
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto q = [&](double p) { return l[std::min(l.size() - 1, (size_t)(p * (l.size() - 1) + 0.5))]; };
    st->p50_ms = q(0.50);
    st->p99_ms = q(0.99);
    double sum = 0;
    for (double x : l) sum += x;
    st->mean_ms = sum / l.size();
    double span = std::chrono::duration<double>(s->last_done - s->first_submit).count();
    st->rows_per_s = span > 0 ? s->rows / span : 0;
  }
  return DML_OK;
}

void dml_server_destroy(dml_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  for (auto& cv : s->cv_work) cv.notify_all();
  for (auto& w : s->worker)
    if (w.joinable()) w.join();
  for (Slot& sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.batch.done) cudaEventDestroy(sl.batch.done);
    cudaFreeHost(sl.h_in);
    cudaFreeHost(sl.h_out);
    cudaFreeHost(sl.h_tiles);
    cudaFree(sl.d_in);
    cudaFree(sl.d_out);
    cudaFree(sl.d_tiles);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  delete s;
}

}  // extern "C"
