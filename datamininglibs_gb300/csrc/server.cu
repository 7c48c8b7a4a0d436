// Prediction server: resident forests, continuous batching, HBM-budget
// admission.  No reference counterpart (the reference predicts one data frame
// per call, gpudte_algorithm.cc:270-331).
//
// A worker thread keeps up to n_streams batches in flight.  A batch packs the
// queued requests (any mix of forests) that fit the batch-row limit and the
// free part of the device budget into one launch over a list of 128-row
// tiles; each tile walks its request's forest for its rows.  Requests that
// arrive while batches run join the next batch as soon as a stream slot and
// budget free up.  Request rows are staged through pinned host memory; results
// are copied back to the caller's buffer when the batch's event completes.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
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

constexpr int kTileRows = 128;

struct PredTile {
  const PNode* nodes;
  const float* X;   // feature-major rows of the request: X[f * n + i]
  float* out;       // [n * width]
  long long n;      // rows of the request
  int row0, rows;   // this tile
  int n_trees, C, task, pad;
};

template <int UNUSED>
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
    for (int k = 0; k < t.n_trees; ++k) {
      int4 p = __ldg(reinterpret_cast<const int4*>(t.nodes) + k);
      while (p.x >= 0) {
        const float x = __ldg(t.X + (long long)p.y * t.n + row);
        const int nx = goes_left(x, __int_as_float(p.z)) ? p.x : p.x + 1;
        p = __ldg(reinterpret_cast<const int4*>(t.nodes) + nx);
      }
      if (t.task == 0)
        my[p.y] += 1;
      else
        acc = __fadd_rn(acc, __int_as_float(p.z));
    }
    if (t.task == 0)
      for (int c = 0; c < t.C; ++c) t.out[row * t.C + c] = (float)my[c];
    else
      t.out[row] = acc;
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
  size_t in_bytes, out_bytes;
};

struct Batch {
  std::vector<Request> reqs;
  std::vector<size_t> in_off, out_off;  // offsets in the slot's staging buffers
  size_t bytes = 0;
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
  size_t cap = 0;         // bytes of each staging direction
  int tile_cap = 0;
  Batch batch;
};

}  // namespace
}  // namespace dml

struct dml_server {
  dml_server_config cfg;
  int device = 0;
  std::vector<const dml_forest*> forests;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<dml::Request> queue;
  std::unordered_map<long long, double> done;  // id -> latency ms
  std::vector<double> latencies;
  long long next_id = 1, completed = 0, rows = 0, launches = 0, rejected = 0;
  dml::Clock::time_point first_submit, last_done;
  bool have_first = false, stop = false;
  std::vector<dml::Slot> slots;
  std::thread worker;
  size_t budget_per_slot = 0;
};

namespace dml {
namespace {

size_t req_in_bytes(const dml_forest* f, long long n) { return sizeof(float) * (size_t)n * f->n_features; }
size_t req_out_bytes(const dml_forest* f, long long n) {
  return sizeof(float) * (size_t)n * (f->task == DML_CLASSIFICATION ? f->n_classes : 1);
}
size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Completes finished batches; returns true if any slot finished.
bool reap(dml_server* s) {
  bool any = false;
  for (Slot& sl : s->slots) {
    if (!sl.batch.busy) continue;
    if (cudaEventQuery(sl.batch.done) != cudaSuccess) continue;
    for (size_t i = 0; i < sl.batch.reqs.size(); ++i) {
      const Request& r = sl.batch.reqs[i];
      std::memcpy(r.out, sl.h_out + sl.batch.out_off[i], r.out_bytes);
    }
    auto now = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (const Request& r : sl.batch.reqs) {
        double ms = std::chrono::duration<double, std::milli>(now - r.t_submit).count();
        s->done[r.id] = ms;
        s->latencies.push_back(ms);
        s->completed++;
        s->rows += r.n;
      }
      s->last_done = now;
    }
    s->cv_done.notify_all();
    sl.batch.reqs.clear();
    sl.batch.busy = false;
    any = true;
  }
  return any;
}

// Packs queued requests into a free slot and launches the batch.
bool launch_batch(dml_server* s, Slot& sl) {
  Batch& b = sl.batch;
  b.reqs.clear();
  b.in_off.clear();
  b.out_off.clear();
  size_t in_used = 0, out_used = 0;
  long long rows = 0;
  int tiles = 0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    while (!s->queue.empty()) {
      const Request& r = s->queue.front();
      const int rt = (int)((r.n + kTileRows - 1) / kTileRows);
      if (!b.reqs.empty() && (rows + r.n > s->cfg.max_batch_rows ||
                              in_used + align256(r.in_bytes) > sl.cap ||
                              out_used + align256(r.out_bytes) > sl.cap || tiles + rt > sl.tile_cap))
        break;
      if (b.reqs.empty() && (align256(r.in_bytes) > sl.cap || align256(r.out_bytes) > sl.cap ||
                             rt > sl.tile_cap))
        break;  // cannot happen: rejected at submit
      b.in_off.push_back(in_used);
      b.out_off.push_back(out_used);
      in_used += align256(r.in_bytes);
      out_used += align256(r.out_bytes);
      rows += r.n;
      tiles += rt;
      b.reqs.push_back(r);
      s->queue.pop_front();
    }
  }
  if (b.reqs.empty()) return false;
  int nt = 0;
  for (size_t i = 0; i < b.reqs.size(); ++i) {
    const Request& r = b.reqs[i];
    const dml_forest* f = s->forests[r.forest];
    std::memcpy(sl.h_in + b.in_off[i], r.samples, r.in_bytes);
    for (long long r0 = 0; r0 < r.n; r0 += kTileRows) {
      PredTile& t = sl.h_tiles[nt++];
      t.nodes = f->pnodes;
      t.X = (const float*)(sl.d_in + b.in_off[i]);
      t.out = (float*)(sl.d_out + b.out_off[i]);
      t.n = r.n;
      t.row0 = (int)r0;
      t.rows = (int)std::min<long long>(kTileRows, r.n - r0);
      t.n_trees = f->n_trees;
      t.C = f->task == DML_CLASSIFICATION ? f->n_classes : 1;
      t.task = f->task;
      t.pad = 0;
    }
  }
  cudaMemcpyAsync(sl.d_in, sl.h_in, in_used, cudaMemcpyHostToDevice, sl.stream);
  cudaMemcpyAsync(sl.d_tiles, sl.h_tiles, sizeof(PredTile) * nt, cudaMemcpyHostToDevice, sl.stream);
  int Cmax = 1;
  for (const Request& r : b.reqs) {
    const dml_forest* f = s->forests[r.forest];
    if (f->task == DML_CLASSIFICATION) Cmax = std::max(Cmax, f->n_classes);
  }
  k_predict_tiles<0><<<nt, kTileRows, sizeof(int) * kTileRows * Cmax, sl.stream>>>(sl.d_tiles);
  cudaMemcpyAsync(sl.h_out, sl.d_out, out_used, cudaMemcpyDeviceToHost, sl.stream);
  cudaEventRecord(b.done, sl.stream);
  b.busy = true;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->launches++;
  }
  return true;
}

void worker_main(dml_server* s) {
  cudaSetDevice(s->device);
  while (true) {
    bool progressed = reap(s);
    bool have_free = false;
    for (Slot& sl : s->slots)
      if (!sl.batch.busy) {
        have_free = true;
        bool pending;
        {
          std::lock_guard<std::mutex> lk(s->mu);
          pending = !s->queue.empty();
        }
        if (!pending) break;
        if (s->cfg.max_wait_us > 0) {
          // let a batch fill briefly when the GPU is idle and few rows wait
          std::unique_lock<std::mutex> lk(s->mu);
          long long waiting = 0;
          for (const Request& r : s->queue) waiting += r.n;
          bool idle = true;
          for (Slot& o : s->slots) idle = idle && !o.batch.busy;
          if (idle && waiting < s->cfg.max_batch_rows / 8)
            s->cv_work.wait_for(lk, std::chrono::microseconds(s->cfg.max_wait_us));
        }
        progressed |= launch_batch(s, sl);
      }
    bool any_busy = false;
    for (Slot& sl : s->slots) any_busy |= sl.batch.busy;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop && s->queue.empty() && !any_busy) break;
    if (!progressed) {
      if (any_busy || (!s->queue.empty() && !have_free)) {
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(20));
      } else {
        s->cv_work.wait_for(lk, std::chrono::milliseconds(5),
                            [&] { return s->stop || !s->queue.empty(); });
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
      cfg->n_streams <= 0 || cfg->n_streams > 64 || cfg->max_wait_us < 0) {
    set_error("invalid server configuration");
    return DML_ERR_INVALID_ARG;
  }
  init_pool_once();
  dml_server* s = new dml_server();
  s->cfg = *cfg;
  cudaGetDevice(&s->device);
  s->slots.resize(cfg->n_streams);
  // half of a slot's share of the budget for inputs, half for outputs
  s->budget_per_slot = (size_t)(cfg->hbm_budget_bytes / cfg->n_streams / 2) & ~(size_t)255;
  bool ok = s->budget_per_slot >= 4096;
  for (Slot& sl : s->slots) {
    if (!ok) break;
    sl.cap = s->budget_per_slot;
    sl.tile_cap = (int)std::min<long long>(
        1 << 22, cfg->max_batch_rows / kTileRows + 4 * 1024);
    ok = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess &&
         cudaMallocHost(&sl.h_in, sl.cap) == cudaSuccess &&
         cudaMallocHost(&sl.h_out, sl.cap) == cudaSuccess &&
         cudaMallocHost(&sl.h_tiles, sizeof(PredTile) * sl.tile_cap) == cudaSuccess &&
         cudaMalloc(&sl.d_in, sl.cap) == cudaSuccess && cudaMalloc(&sl.d_out, sl.cap) == cudaSuccess &&
         cudaMalloc(&sl.d_tiles, sizeof(PredTile) * sl.tile_cap) == cudaSuccess &&
         cudaEventCreateWithFlags(&sl.batch.done, cudaEventDisableTiming) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    set_error("could not allocate the server's streams and staging buffers");
    s->stop = true;
    dml_server_destroy(s);
    return DML_ERR_OOM;
  }
  s->worker = std::thread(worker_main, s);
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
  if (!s || !samples || !out || !request_id || n_rows <= 0 || n_rows > (1 << 20)) {
    set_error("invalid request (rows must be in 1 .. 1048576)");
    return DML_ERR_INVALID_ARG;
  }
  Request r;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (forest_id < 0 || forest_id >= (int32_t)s->forests.size()) {
      set_error("unknown forest id %d", forest_id);
      return DML_ERR_INVALID_ARG;
    }
    const dml_forest* f = s->forests[forest_id];
    r.in_bytes = req_in_bytes(f, n_rows);
    r.out_bytes = req_out_bytes(f, n_rows);
    if (align256(r.in_bytes) > s->budget_per_slot || align256(r.out_bytes) > s->budget_per_slot ||
        n_rows > s->cfg.max_batch_rows) {
      s->rejected++;
      set_error("request of %lld rows exceeds the server's per-batch budget", (long long)n_rows);
      return DML_ERR_BUDGET;
    }
    r.id = s->next_id++;
    r.forest = forest_id;
    r.samples = samples;
    r.n = n_rows;
    r.out = out;
    r.t_submit = Clock::now();
    if (!s->have_first) {
      s->first_submit = r.t_submit;
      s->have_first = true;
    }
    s->queue.push_back(r);
    *request_id = r.id;
  }
  s->cv_work.notify_one();
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
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
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
