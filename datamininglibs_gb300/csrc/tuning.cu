// Fit tuning: which search kernel takes RF nodes of which size, and how many
// persistent CTAs per SM the big-node items run with.  Every choice computes
// the same splits (the kernels differ only in how they sort and scan), so the
// tuning changes speed, never results.
//
// dml_autotune times each candidate on a sample of the problem (its first
// sample_trees trees) and keeps the fastest for the problem's shape bucket:
// algorithm, task, class-count width, log2 rows, log2 features and features
// tried per node.  Tunings live in memory and, when DML_TUNE_CACHE names a
// file, in that file (one JSON object per line), read once per process.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"

namespace dml {

void clear_error();

namespace {

std::mutex g_mu;
std::map<std::string, Tuning> g_table;
bool g_loaded = false;
thread_local const Tuning* g_force = nullptr;  // set while dml_autotune times a candidate

int log2_round(double x) { return (int)std::lround(std::log2(std::max(1.0, x))); }

std::string key_of(const dml_fit_desc& d) {
  const int C = d.task == DML_CLASSIFICATION ? d.n_classes : 1;
  const int K = d.n_features_try > 0 ? d.n_features_try
                                     : (int)std::round(std::log((double)d.n_features)) + 1;
  char buf[128];
  std::snprintf(buf, sizeof(buf), "a%d-t%d-c%d-n%d-f%d-k%d", d.algo, d.task, class_width(C),
                log2_round((double)d.n_rows), log2_round((double)d.n_features), K);
  return buf;
}

const char* cache_path() {
  const char* p = std::getenv("DML_TUNE_CACHE");
  return p && *p ? p : nullptr;
}

void load_locked() {
  if (g_loaded) return;
  g_loaded = true;
  const char* path = cache_path();
  if (!path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  char line[512];
  while (std::fgets(line, sizeof(line), f)) {
    char key[128];
    Tuning t;
    if (std::sscanf(line,
                    " {\"key\": \"%127[^\"]\", \"warp_max\": %d, \"smem_cap\": %d, \"big_ctas\": %d",
                    key, &t.warp_max, &t.smem_cap, &t.big_ctas) == 4 &&
        valid_tuning(t))
      g_table[key] = t;
  }
  std::fclose(f);
}

void save_locked(const std::string& key, const Tuning& t, double ms) {
  const char* path = cache_path();
  if (!path) return;
  FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "{\"key\": \"%s\", \"warp_max\": %d, \"smem_cap\": %d, \"big_ctas\": %d, "
                  "\"sample_ms\": %.3f}\n", key.c_str(), t.warp_max, t.smem_cap, t.big_ctas, ms);
  std::fclose(f);
}

}  // namespace

int class_width(int C) {
  return C <= 2 ? 1 : C <= 4 ? 2 : C <= 8 ? 4 : C <= 10 ? 5 : C <= 16 ? 8 : 16;
}

bool valid_tuning(const Tuning& t) {
  return (t.warp_max == 64 || t.warp_max == 128 || t.warp_max == 256 || t.warp_max == 512) &&
         t.smem_cap >= 257 &&
         t.smem_cap <= kSearchSmemCap && t.big_ctas >= 1 && t.big_ctas <= 4;
}

Tuning default_tuning(int CW) { return Tuning{512, kDefaultSmemCap, big_ctas_per_sm(CW)}; }

// The tuning of a fit: the forced candidate, the stored tuning of the largest
// problem's bucket, or the defaults.
Tuning tuning_for(const dml_fit_desc* descs, int nprob, int CW) {
  if (g_force) return *g_force;
  int big = 0;
  for (int i = 1; i < nprob; ++i)
    if ((double)descs[i].n_rows * descs[i].n_trees > (double)descs[big].n_rows * descs[big].n_trees)
      big = i;
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  auto it = g_table.find(key_of(descs[big]));
  Tuning t = it != g_table.end() ? it->second : default_tuning(CW);
  t.big_ctas = std::min(t.big_ctas, default_tuning(CW).big_ctas);  // what the kernel's registers allow
  return t;
}

}  // namespace dml

using namespace dml;

extern "C" {

dml_status dml_tuning_get(const dml_fit_desc* desc, dml_tuning* out) {
  clear_error();
  if (!desc || !out) {
    set_error("null argument");
    return DML_ERR_INVALID_ARG;
  }
  const int C = desc->task == DML_CLASSIFICATION ? desc->n_classes : 1;
  const Tuning t = tuning_for(desc, 1, class_width(C));
  out->warp_max = t.warp_max;
  out->smem_cap = t.smem_cap;
  out->big_ctas_per_sm = t.big_ctas;
  out->reserved = 0;
  return DML_OK;
}

dml_status dml_autotune(const dml_fit_desc* desc, int32_t sample_trees, dml_tuning* best,
                        void* stream) {
  clear_error();
  if (!desc || !best || sample_trees <= 0) {
    set_error("null argument or sample_trees <= 0");
    return DML_ERR_INVALID_ARG;
  }
  dml_fit_desc d = *desc;
  d.n_trees = std::min(d.n_trees, sample_trees);
  const int C = d.task == DML_CLASSIFICATION ? d.n_classes : 1;
  const int max_ctas = default_tuning(class_width(C)).big_ctas;
  std::vector<Tuning> cands;
  if (d.algo == DML_ALGO_RF) {
    for (int wm : {256, 512})
      for (int cap : {1024, 2048, kSearchSmemCap})
        for (int bc = std::max(1, max_ctas - 1); bc <= max_ctas; ++bc)
          cands.push_back(Tuning{wm, cap, bc});
  } else {
    cands.push_back(default_tuning(class_width(C)));  // ERT has no RF thresholds
  }
  double best_ms = 1e300;
  Tuning best_t = cands[0];
  for (int pass = 0; pass < 2; ++pass)  // the first pass warms caches and the memory pool
    for (const Tuning& t : cands) {
      g_force = &t;
      dml_forest* f = nullptr;
      const dml_status st = dml_fit(&d, &f, stream);
      g_force = nullptr;
      if (st != DML_OK) return st;
      dml_fit_stats fs;
      dml_last_fit_stats(&fs);
      dml_forest_free(f);
      if (pass == 1 && fs.level_loop_ms < best_ms) {
        best_ms = fs.level_loop_ms;
        best_t = t;
      }
    }
  {
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    const std::string key = key_of(*desc);
    g_table[key] = best_t;
    save_locked(key, best_t, best_ms);
  }
  best->warp_max = best_t.warp_max;
  best->smem_cap = best_t.smem_cap;
  best->big_ctas_per_sm = best_t.big_ctas;
  best->reserved = 0;
  return DML_OK;
}

}  // extern "C"
