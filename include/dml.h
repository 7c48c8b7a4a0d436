/* dml.h — C ABI of the GB300 random-forest / extremely-randomized-trees engine.
 *
 * Drop-in boundary for the fit/predict path of novelari/DataminingLibs
 * (lib_ensembles).  Plain C types only: pointers, sizes, status codes; CUDA
 * streams are passed as `void*` (a cudaStream_t, or NULL for the default
 * stream).  No entry point throws; every one returns a dml_status and leaves a
 * message for dml_last_error() (per calling thread).
 *
 * Data layout (lib_data): samples are feature-major, samples[f * n_rows + i]
 * (lib_parsing/source/csv_parser.cc:92-96, lib_ensembles/source/gpudte.cu:65-68);
 * targets hold one float per row: the class index as a float for
 * classification (MlDataFrame<float>::GetTargets), the value for regression.
 *
 * Model layout (lib_models): dml_forest_export writes the reference's
 * kNodeArray of gpuDTE_NodeHeader_Classify<float> = {int child_start,
 * child_count, probability_start, attribute; float split_point}
 * (lib_ensembles/source/gpudte_algorithm_shared.h:82-90) with the roots of the
 * trees at 0..n_trees-1, and kProbArray with n_classes floats per leaf (class
 * counts) or one float per leaf (regression mean).
 */
#ifndef DML_H_
#define DML_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define DML_API __attribute__((visibility("default")))
#else
#define DML_API
#endif

typedef enum {
  DML_OK = 0,
  DML_ERR_INVALID_ARG = 1,
  DML_ERR_OOM = 2,
  DML_ERR_CUDA = 3,
  DML_ERR_TIMEOUT = 4,
  DML_ERR_BUDGET = 5,
  DML_ERR_NOT_READY = 6,
  DML_ERR_INTERNAL = 7
} dml_status;

/* EnsemblesInterface::CreateGpuRfAlgorithm / CreateGpuErtAlgorithm
 * (lib_ensembles/source/ensembles_interface.cc:14-26). */
typedef enum { DML_ALGO_RF = 0, DML_ALGO_ERT = 1 } dml_algo;
/* AlgorithmsInterface::AlgorithmType (lib_algorithms/include/algorithms_interface.h:9). */
typedef enum { DML_CLASSIFICATION = 0, DML_REGRESSION = 1 } dml_task;
/* Where the pointers of a call live. */
typedef enum { DML_HOST = 0, DML_DEVICE = 1 } dml_memory;

/* Fit parameters and data: the EnsemblesLib DteParams (ensembles_interface.h:28-38)
 * plus the data frame.  n_features_try = kNrFeatures (0 -> round(ln F) + 1),
 * max_depth = kMaxDepth, min_node_size = kMinNodeSize, n_trees = kNrTrees,
 * task = kAlgoType.  min_leaf (>= 1) and seed are additions. */
typedef struct {
  int32_t algo;
  int32_t task;
  int32_t n_trees;
  int32_t n_features_try;
  int32_t max_depth;
  int32_t min_node_size;
  int32_t min_leaf;
  int32_t n_classes; /* classification: labels are 0..n_classes-1; <= 32 */
  uint64_t seed;
  int64_t n_rows;
  int32_t n_features;
  int32_t memory; /* dml_memory of samples/targets */
  const float* samples;
  const float* targets;
  /* RNG key of the first tree: a forest fitted as parts with tree_offset =
   * the trees before each part equals the forest fitted at once. */
  int32_t tree_offset;
  /* kEasyEnsemble (gpudte_algorithm.cc:582-583, gpurf.cu:73-100): RF
   * classification only; each tree draws n_rows / n_classes rows of every
   * non-empty class, uniformly with replacement, instead of n_rows rows. */
  int32_t balanced;
} dml_fit_desc;

typedef struct dml_forest dml_forest;

typedef struct {
  int32_t task;
  int32_t n_trees;
  int32_t n_classes; /* 1 for regression */
  int32_t n_features;
  int64_t n_nodes;
  int64_t n_probs;
  int32_t max_depth; /* deepest level reached */
  int32_t reserved;
  double fit_ms;     /* device time of the level loop of the fit that built it */
} dml_forest_info;

/* Node classes of the split search (the index of the per-class statistics)
 * and the kernels that search them. */
enum {
  DML_Q_WARP32 = 0,   /* <= 32 entries, one warp per node (k_group_nodes<32>) */
  DML_Q_ERT = 1,      /* ERT, > 256 entries, one CTA per node (k_ert_cta) */
  DML_Q_RF_SMEM = 2,  /* RF, above the warp classes up to the tuned cap (at most 4096
                       * entries), CTA, shared-memory sort (k_rf_smem) */
  DML_Q_RF_BIG = 3,   /* RF, > 4096 entries, per-try items (k_rf_big_items + _decide) */
  DML_Q_RF_W64 = 4,   /* RF, 33..64 entries, warp register sort (k_warp_rf<2>) */
  DML_Q_RF_W128 = 5,  /* RF, 65..128 entries (k_warp_rf<4>) */
  DML_Q_RF_W256 = 6,  /* RF, 129..256 entries (k_warp_rf<8>) */
  DML_Q_GROUP16 = 7,  /* <= 16 entries, 16 lanes per node (k_group_nodes<16>) */
  DML_Q_GROUP8 = 8,   /* <= 8 entries, 8 lanes per node (k_group_nodes<8>) */
  DML_Q_RF_W512 = 9,  /* RF, 257..512 entries (k_warp_rf<16>) */
  DML_Q_ERT_W256 = 10, /* ERT, 33..256 entries, one warp per node (k_ert_warp<8>) */
  DML_NUM_QUEUES = 11
};

/* Fit statistics of the last dml_fit/dml_fit_batched on this thread. */
typedef struct {
  int64_t nodes;         /* internal + leaf nodes created, all forests */
  int64_t entries;       /* sum over levels of the searched nodes' distinct row entries */
  int64_t weighted_rows; /* the same with bootstrap multiplicities */
  int64_t entry_tries;   /* sum over searched nodes of tries evaluated x entries */
  int32_t levels;
  int32_t launches;      /* kernel launches of the fit */
  double level_loop_ms;  /* device time of the level loop (CUDA events) */
  double search_ms;      /* device time in the split-search kernels */
  /* per node class (DML_Q_*): device time (CUDA events around the class's
   * launches on the fit stream), searched entries, tries x entries */
  double queue_ms[DML_NUM_QUEUES];
  int64_t queue_entries[DML_NUM_QUEUES];
  int64_t queue_entry_tries[DML_NUM_QUEUES];
  int32_t queue_launches[DML_NUM_QUEUES]; /* kernel launches per class */
  int32_t reserved;
} dml_fit_stats;

/* GpuDteAlgorithm<T>::Fit (lib_ensembles/source/gpudte_algorithm.cc:15-267),
 * reached through MlAlgorithm<T>::Fit (lib_algorithms/include/ml_algorithm.h:29-30).
 * Builds the forest on the current device; *out is a device-resident handle. */
DML_API dml_status dml_fit(const dml_fit_desc* desc, dml_forest** out, void* stream);

/* No reference counterpart as one call: n independent forests (uneven row,
 * feature and class counts) built together, one launch set per tree level for
 * all of them.  out[i] receives forest i. */
DML_API dml_status dml_fit_batched(int32_t n, const dml_fit_desc* descs, dml_forest** out,
                                   void* stream);

/* The per-level chunked launch structure of the reference
 * (gpudte_algorithm.cc:145-253: <= 512 nodes per launch, host syncs per chunk),
 * on this engine's kernels: same results as dml_fit.  The baseline that the
 * batched level path is measured against. */
DML_API dml_status dml_fit_plain(const dml_fit_desc* desc, dml_forest** out, void* stream);

/* No counterpart in the reference.  dml_fit for callers that cannot allocate
 * device memory while they fit: a process whose device memory is owned by its
 * own allocator (a framework's caching allocator, an arena sized at start-up)
 * or partitioned by a budget, where memory a library allocates on its own is
 * memory nobody accounted for; a latency-critical service that keeps
 * cudaMalloc / cudaFree (which can synchronise the device and can fail under
 * fragmentation) out of its steady state.  Same trees as dml_fit.  It
 * allocates nothing: its working buffers live in one static device array of
 * about 20 MiB that every GPU loading this library holds until the process
 * exits, so the problem must fit it: at most 4096 rows, n_trees * n_rows <=
 * 65536, at most 8 classes; larger problems are rejected with
 * DML_ERR_INVALID_ARG.  samples and targets must be device pointers
 * (desc->memory == DML_DEVICE).  The model is written to caller-owned device
 * buffers: node_array (Classify layout, 20 bytes per node, room for
 * n_trees * (2 * n_rows - 1) nodes) and probs (room for n_trees * n_rows *
 * n_classes floats); *n_nodes / *n_probs receive the sizes used.  The call
 * synchronises its stream once to read the data check and once per tree level.
 * Calls share the static array, which keeps the last call's contents: calls
 * whose work overlaps on the GPU race, so serialise them.  The first call on a
 * device sets the array up with that device current (looks up its address and
 * uploads a constant table). */
DML_API dml_status dml_fit_noalloc(const dml_fit_desc* desc, void* node_array,
                                   int64_t node_capacity, float* probs, int64_t prob_capacity,
                                   int64_t* n_nodes, int64_t* n_probs, void* stream);

DML_API dml_status dml_last_fit_stats(dml_fit_stats* stats);

/* Scheduling of RF fits (no counterpart in the reference): nodes of up to
 * warp_max entries (64, 128, 256 or 512) are searched by one warp, up to
 * smem_cap entries (257 .. 4096) by one CTA in shared memory, larger ones as
 * per-try items on big_ctas_per_sm (1 .. 4, at most what the item kernel's
 * registers allow) persistent CTAs per SM.  Results do not depend on
 * it.  dml_autotune fits the first sample_trees trees of desc once per
 * candidate, keeps the fastest for desc's shape (algorithm, task, classes,
 * log2 rows, log2 features, features tried) for later fits of that shape in
 * this process, and appends it to the file named by the environment variable
 * DML_TUNE_CACHE when set (read back by later processes).  dml_tuning_get
 * gives the tuning a fit of desc would use. */
typedef struct {
  int32_t warp_max;
  int32_t smem_cap;
  int32_t big_ctas_per_sm;
  int32_t reserved;
} dml_tuning;

DML_API dml_status dml_autotune(const dml_fit_desc* desc, int32_t sample_trees, dml_tuning* best,
                                void* stream);
DML_API dml_status dml_tuning_get(const dml_fit_desc* desc, dml_tuning* out);

/* Out-of-bag estimate of an RF forest (gpurf.cu:290-359, kOobEstimate) and the
 * permutation run of one feature (gpurf.cu:361-438, kFeatureImp).  desc is the
 * descriptor the forest was fitted with (data, seed, tree_offset, balanced):
 * the trees' bags are drawn again from it.  Every (tree, row) pair whose row is
 * out of the tree's bag walks the tree; with permuted_feature >= 0 the value of
 * that feature is taken from row (Philox(seed; row, tree, kTagPermute) % n_rows)
 * at every node that splits on it (the reference draws a random row per node
 * visit).  Sums are reduced in a fixed order.  Permutation importance of a
 * feature = (pairs_correct - permuted pairs_correct) / pairs for
 * classification, (permuted pairs_sq_err - pairs_sq_err) / pairs for
 * regression. */
typedef struct {
  int64_t pairs;         /* (tree, row) pairs with the row out of the tree's bag */
  int64_t pairs_correct; /* classification: pairs whose tree votes the row's class */
  double pairs_sq_err;   /* regression: sum over pairs of (target - tree output)^2 */
  int64_t rows;          /* rows out of the bag of at least one tree */
  int64_t rows_correct;  /* classification: rows whose out-of-bag vote is their class */
  double rows_sq_err;    /* regression: sum over rows of (target - mean OOB output)^2 */
} dml_oob_stats;

DML_API dml_status dml_oob_estimate(const dml_forest* forest, const dml_fit_desc* desc,
                                    int32_t permuted_feature, dml_oob_stats* out, void* stream);

/* GpuDteAlgorithm<T>::Predict (gpudte_algorithm.cc:270-331).  samples is
 * feature-major [n_features * n_rows]; out receives n_rows * n_classes vote
 * counts (classification) or n_rows sums of tree outputs (regression), as
 * MlResultData::AddPredictions holds them (ml_resultdata_impl.cc:17-21). */
DML_API dml_status dml_predict(const dml_forest* forest, const float* samples, int64_t n_rows,
                               float* out, int32_t memory, void* stream);

/* The same votes with the reference's predict launch structure
 * (gpudte_algorithm.cc:292-311, gpudte.cu:311-359): one thread per (tree, row),
 * at most 65,536 threads per launch, a host sync after every launch, and host
 * samples copied in and votes copied out on every call.  Launches cover one
 * tree at a time, so sums keep tree order and equal dml_predict's.  The
 * denominator of the serving speed-up; not a fast path. */
DML_API dml_status dml_predict_plain(const dml_forest* forest, const float* samples,
                                     int64_t n_rows, float* out, int32_t memory, void* stream);

DML_API dml_status dml_forest_info_get(const dml_forest* forest, dml_forest_info* info);

/* The model slots kNodeArray / kProbArray (lib_models/include/models_interface.h:9-19,
 * filled at gpudte_algorithm.cc:257-258).  node_array receives n_nodes * 20
 * bytes, probs n_probs floats (host memory). */
DML_API dml_status dml_forest_export(const dml_forest* forest, void* node_array, float* probs);

/* The FP32 information (or variance) gain of every node's chosen split, in
 * kNodeArray order: n_nodes floats, NaN for leaves.  The reference computes
 * these gains in its split search (entropy_over_columns -
 * entropy_conditioned_on_rows, lib_ensembles/source/gpudte.cu:76-117;
 * gpurf.cu:618-768, gpuert.cu:275-381) and keeps only the winning split, so it
 * has no counterpart call.  memory says where `gains` lives (DML_HOST: the call
 * returns when the copy is done; DML_DEVICE: ordered on `stream`).  Forests
 * built by dml_forest_import / dml_forest_load hold no gains
 * (DML_ERR_INVALID_ARG). */
DML_API dml_status dml_forest_gains(const dml_forest* forest, float* gains, int32_t memory,
                                    void* stream);

/* A device-resident forest from kNodeArray / kProbArray in the layout above
 * (host memory), e.g. a model built by the reference or merged on the host. */
DML_API dml_status dml_forest_import(int32_t task, int32_t n_trees, int32_t n_classes,
                                     int32_t n_features, const void* node_array, int64_t n_nodes,
                                     const float* probs, int64_t n_probs, dml_forest** out);

/* Forest files (no counterpart in the reference, whose models live only in
 * MlModel slots, ml_model_impl.cc:6-10): little-endian
 *   "DMLF", u32 version = 1, i32 task, n_trees, n_classes, n_features,
 *   i64 n_nodes, n_probs, the kNodeArray records (20 bytes each),
 *   the kProbArray floats, u64 FNV-1a hash of everything before it.
 * Load checks the header, sizes and hash, then imports as dml_forest_import. */
DML_API dml_status dml_forest_save(const dml_forest* forest, const char* path);
DML_API dml_status dml_forest_load(const char* path, dml_forest** out);

DML_API void dml_forest_free(dml_forest* forest);

DML_API const char* dml_last_error(void);

/* GpuDevice::GetDeviceCount (lib_gpu/include/gpu_device.h:22) and the device
 * choice of GpuInterface::CreateGpuDevice(dev_id) (lib_gpu/source/
 * gpu_interface.cc:13-40) for the calling thread: the engine runs on the
 * calling thread's current CUDA device. */
DML_API dml_status dml_device_count(int32_t* count);
DML_API dml_status dml_set_device(int32_t device);

/* ------------------------------------------------------------------ serving
 * No reference counterpart (the reference has no serving path): a resident-
 * forest prediction server with continuous batching.  Requests are admitted
 * while earlier ones run, as HBM budget and batch slots free up; their work
 * shares kernel launches across streams.  Two lanes: requests of at most
 * small_rows rows run on high-priority streams with the trees of a row split
 * over 8 threads (latency); larger requests run on low-priority streams in
 * slices of at most max_batch_rows rows (throughput), so a large request never
 * holds the device for long.  Host buffers that are pinned (cudaHostAlloc /
 * cudaHostRegister) are copied by DMA directly; others are staged. */
typedef struct dml_server dml_server;

typedef struct {
  int64_t hbm_budget_bytes;   /* device bytes for request inputs/outputs */
  int32_t max_batch_rows;     /* rows packed into one large-lane launch (slice size) */
  int32_t n_streams;          /* launches in flight per lane */
  int32_t max_wait_us;        /* how long an idle small-lane batch waits to fill */
  int32_t small_rows;         /* requests up to this many rows take the small lane; 0 = 4096 */
} dml_server_config;

typedef struct {
  int64_t completed;
  int64_t rows;
  double p50_ms;
  double p99_ms;
  double mean_ms;
  double rows_per_s;
  int64_t launches;
  int64_t rejected;
} dml_server_stats;

DML_API dml_status dml_server_create(const dml_server_config* cfg, dml_server** out);
/* The forest stays owned by the caller and must outlive the server. */
DML_API dml_status dml_server_add_forest(dml_server* s, const dml_forest* forest, int32_t* forest_id);
/* samples: host feature-major [n_features * n_rows]; out: host buffer of
 * n_rows * width floats, written when the request completes.  Both must stay
 * valid until dml_server_poll reports the request done. */
DML_API dml_status dml_server_submit(dml_server* s, int32_t forest_id, const float* samples,
                                     int64_t n_rows, float* out, int64_t* request_id);
/* DML_OK when done, DML_ERR_NOT_READY while pending; latency_ms is the time
 * from submit to completion. */
DML_API dml_status dml_server_poll(dml_server* s, int64_t request_id, double* latency_ms);
DML_API dml_status dml_server_wait(dml_server* s, int64_t request_id, double* latency_ms);
DML_API dml_status dml_server_stats_get(dml_server* s, dml_server_stats* stats);
DML_API void dml_server_destroy(dml_server* s);

#ifdef __cplusplus
}
#endif
#endif /* DML_H_ */
