// Pinning harness (test infrastructure): the reference's own device functions
// from lib_ensembles/source/gpudte.cu, compiled unchanged as host C++ with
// ref_shim/host_emulation.h and run with one thread per block, plus the
// reference's host-side data frame, result data and CSV parser.  Built by
// oracle/ref.mk into oracle/_ref/libref.so; used only to generate and check
// golden vectors for the oracle (tests/golden/make_golden.py).
//
// Functions exercised (file:line in the reference project):
//   GpuDte<T>::entropy_over_columns / entropy_conditioned_on_rows / lnFunc
//       lib_ensembles/source/gpudte.cu:70-117
//   GpuDte<T>::gpudte_perform_split  lib_ensembles/source/gpudte.cu:156-309
//   GpuDte<T>::gpudte_predict        lib_ensembles/source/gpudte.cu:311-359
//   MlResultDataImpl<T>::GetAccuracy lib_data/source/ml_resultdata_impl.cc:23-38
//   CsvParser<T>::Parse              lib_parsing/source/csv_parser.cc:36-104
#include "host_emulation.h"

#include "lib_ensembles/source/gpudte.cu"

#include "lib_data/include/lib_data.h"
#include "lib_parsing/include/parsing_interface.h"

#include <cstdint>
#include <vector>

EmuDim3 threadIdx = {0, 0, 0};
EmuDim3 blockIdx = {0, 0, 0};
EmuDim3 blockDim = {1, 1, 1};
EmuDim3 gridDim = {1, 1, 1};

namespace le = lib_ensembles;
using Shared = le::GpuDteAlgorithmShared;

template <class T>
struct Emu : le::GpuDte<T> {
  void CallCudaKernel(int, int, Shared::GpuParams<T>&,
                      Shared::GpuDteKernelId) override {}
};

extern "C" {

// prior - posterior exactly as GpuErt::eval_numeric_attribute forms it
// (gpuert.cu:316-321): m is the 2 x C count matrix, row-major by side.
float ref_entropy_gain_f(const float* m, int C) {
  Emu<float> e;
  std::vector<float> mm(m, m + 2 * C);
  float prior = e.entropy_over_columns(mm.data(), 2, C);
  float post = e.entropy_conditioned_on_rows(mm.data(), 2, C);
  return prior - post;
}

double ref_entropy_gain_d(const double* m, int C) {
  Emu<double> e;
  std::vector<double> mm(m, m + 2 * C);
  double prior = e.entropy_over_columns(mm.data(), 2, C);
  double post = e.entropy_conditioned_on_rows(mm.data(), 2, C);
  return prior - post;
}

// One call of gpudte_perform_split for one classification node with one
// thread.  indices[0..count) are the node's (expanded) row ids, prob_tmp is
// the 2 x C histogram of the chosen split.  Outputs: the back buffer's node
// range (partitioned row ids), whether the node became a leaf, the two child
// counts and the node's probability row.
int ref_perform_split_f(int nr_targets, int nr_instances, const float* dataset,
                        int attribute, float split_point, int count, int depth,
                        int max_depth, int min_node_size, const int* indices,
                        const float* prob_tmp, int* indices_out, int* child_counts,
                        float* node_probs) {
  Emu<float> e;
  Shared::gpuDTE_StaticInfo si;
  std::memset(&si, 0, sizeof(si));
  si.max_node_size = min_node_size;
  si.max_node_depth = max_depth;
  si.node_buffer_size = 1024;
  Shared::gpuDTE_DatasetInfo di;
  std::memset(&di, 0, sizeof(di));
  di.data_type = 0;
  di.nr_instances = nr_instances;
  di.nr_attributes = 1 << 20;
  di.nr_target_values = nr_targets;
  Shared::gpuDTE_IterationInfo it;
  std::memset(&it, 0, sizeof(it));
  it.read_buffer_id = 0;
  it.write_buffer_id = 1;
  it.prob_buffer_id = 0;
  it.depth = depth;
  it.node_offset = 0;
  it.tick_tock = true;
  std::vector<float> probs(nr_targets, 0.0f), tmp(prob_tmp, prob_tmp + 2 * nr_targets);
  float* pb[2] = {probs.data(), probs.data()};
  std::vector<int> attr_types(attribute + 1, 0x02020202);
  int node_counts[40] = {0};
  std::vector<int> ib0(indices, indices + count), ib1(count, -1);
  int* ib[2] = {ib0.data(), ib1.data()};
  int cursors[3] = {0, 0, 1};
  std::vector<Shared::gpuDTE_NodeHeader_Train<float>> nb0(1), nb1(2), nb2(2);
  nb0[0].tracking_id = 0;
  nb0[0].parent_id = -2;
  nb0[0].node_index_start = 0;
  nb0[0].node_index_count = count;
  nb0[0].attribute = attribute;
  nb0[0].split_point = split_point;
  Shared::gpuDTE_NodeHeader_Train<float>* nb[3] = {nb0.data(), nb1.data(), nb2.data()};
  e.gpudte_perform_split(si, di, it, pb, tmp.data(), const_cast<float*>(dataset),
                         attr_types.data(), node_counts, ib, cursors, nb);
  std::memcpy(indices_out, ib1.data(), sizeof(int) * count);
  for (int i = 0; i < nr_targets; ++i) node_probs[i] = probs[i];
  int leaf = nb0[0].attribute == -1;
  child_counts[0] = leaf ? 0 : nb1[0].node_index_count;
  child_counts[1] = leaf ? 0 : nb1[1].node_index_count;
  return leaf;
}

// gpudte_predict for every (tree, row) thread id, in tid order.  nodes is the
// Classify<float> array (20 bytes per node), roots at 0..n_trees-1.
void ref_predict_f(const void* nodes, const float* probs, int n_trees, int C,
                   int data_type, const float* X, int N, float* out) {
  Emu<float> e;
  int width = data_type == 0 ? C : 1;
  std::memset(out, 0, sizeof(float) * (size_t)N * width);
  std::vector<int> attr_types(1, 0x02020202);
  for (long long tid = 0; tid < (long long)n_trees * N; ++tid)
    e.gpudte_predict((int)tid, N, data_type, width,
                     (Shared::gpuDTE_NodeHeader_Classify<float>*)nodes,
                     const_cast<float*>(X), const_cast<float*>(probs), out,
                     attr_types.data());
}

// CsvParser through ParsingInterface::ParseData<float>.  Returns 0 on success.
int ref_parse_csv_f(const char* text, int* n_rows, int* n_features,
                    int* n_targets, float* samples, float* targets, int cap) {
  std::vector<char> raw(text, text + std::strlen(text) + 1);
  try {
    auto df = lib_parsing::ParsingInterface::GetInstance().ParseData<float>(
        lib_parsing::ParsingInterface::kCsv, raw);
    *n_rows = df->GetNrSamples();
    *n_features = df->GetNrFeatures();
    *n_targets = df->GetNrTargets();
    const auto& s = df->GetSamples();
    const auto& t = df->GetTargets();
    if ((int)s.size() > cap || (int)t.size() > cap) return 2;
    std::memcpy(samples, s.data(), s.size() * sizeof(float));
    std::memcpy(targets, t.data(), t.size() * sizeof(float));
    return 0;
  } catch (...) {
    return 1;
  }
}

float ref_accuracy_f(const float* preds, int N, int C, const float* targets) {
  auto rd = lib_data::DataInterface::GetInstance().CreateResultData<float>();
  std::vector<std::vector<float>> p(N);
  for (int i = 0; i < N; ++i) p[i].assign(preds + (size_t)i * C, preds + (size_t)(i + 1) * C);
  rd->AddPredictions(p);
  std::vector<float> t(targets, targets + N);
  return rd->GetAccuracy(t);
}

}  // extern "C"
