// Implementation of the C++ drop-in (shim/include/datamininglibs.h) over the
// C ABI (include/dml.h).
//
// Restated from the reference (file:line in novelari/DataminingLibs):
//   CoreInterface::ThrowException          lib_core/source/core_interface.cc:28-33
//   MlDataFrameImpl                        lib_data/source/ml_dataframe_impl.cc:12-55
//   MlResultDataImpl (accuracy, +=)        lib_data/source/ml_resultdata_impl.cc:17-71
//   MlModelImpl                            lib_models/source/ml_model_impl.cc:6-10
//   MlAlgorithmParamsImpl                  lib_algorithms/source/ml_algorithm_params_impl.cc:6-16
//   EnsemblesInterface param packs         lib_ensembles/source/ensembles_interface.cc:28-58
//   GpuAlgorithm (device fan-out)          lib_algorithms/source/gpu_algorithm.cc:17-50
//   GpuDteAlgorithm Fit/Predict/Aggregate/Split
//                                          lib_ensembles/source/gpudte_algorithm.cc:15-484
//   CsvParser                              lib_parsing/source/csv_parser.cc:36-104
// Differences from the reference, on purpose: all parameters are honoured when
// a pack is split across devices (the reference rebuilds default packs and
// keeps only the tree count, gpudte_algorithm.cc:474-484); trees left over by
// an uneven split go to the first parts instead of being dropped
// (gpudte_algorithm.cc:412-413); parts carry the RNG key of their first tree,
// so a forest built in parts equals the forest built at once.
#include "datamininglibs.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <iterator>
#include <locale>
#include <sstream>
#include <thread>

#include "../../../include/dml.h"

// ------------------------------------------------------------------ core
namespace lib_core {
namespace {
std::mutex g_debug_mu;
col_array<string> g_debug;
}  // namespace
CoreInterface& CoreInterface::GetInstance() {
  static CoreInterface instance;
  return instance;
}
void CoreInterface::ThrowException(string msg) { throw template_exception(std::move(msg)); }
void CoreInterface::DebugMessage(string msg) {
  std::lock_guard<std::mutex> lk(g_debug_mu);
  g_debug.push_back(std::move(msg));
}
}  // namespace lib_core

namespace {
[[noreturn]] void throw_status(dml_status st, const char* what) {
  string msg = string(what) + ": ";
  const char* e = dml_last_error();
  msg += (e && e[0]) ? e : "error";
  (void)st;
  CoreLib::GetInstance().ThrowException(msg);
}
}  // namespace

// ------------------------------------------------------------------ data
namespace lib_data {
namespace {
template <typename T>
class MlDataFrameImpl : public MlDataFrame<T> {
 public:
  void AddTargetData(col_array<T> targets) override { targets_ = std::move(targets); }
  void AddSampleData(col_array<T> samples) override { samples_ = std::move(samples); }
  void AddFeatureMap(col_array<col_map<string, T>> m) override { feature_maps_ = std::move(m); }
  void AddTargetMap(col_map<string, T> m) override { target_map_ = std::move(m); }
  int GetNrSamples() override { return (int)targets_.size(); }
  int GetNrFeatures() override { return (int)feature_maps_.size(); }
  int GetNrTargets() override { return (int)target_map_.size(); }
  const col_array<T>& GetTargets() override { return targets_; }
  const col_array<T>& GetSamples() override { return samples_; }

 private:
  col_array<T> targets_, samples_;
  col_array<col_map<string, T>> feature_maps_;
  col_map<string, T> target_map_;
};

template <typename T>
class MlResultDataImpl : public MlResultData<T> {
 public:
  void AddSingleValue(string name, T value) override { single_[name] = value; }
  void AddMultipleValue(string name, col_array<T> vals) override {
    multiple_[name] = std::move(vals);
  }
  void AddPredictions(col_array<col_array<T>> p) override {
    if (predictions_.empty()) predictions_ = std::move(p);
  }
  // argmax with a strict '>' from 0 (ties and all-zero rows go to the lowest
  // class), a hit when |class - target| < 0.001
  T GetAccuracy(const col_array<T>& targets) override {
    T acc = 0;
    for (size_t i = 0; i < targets.size(); ++i) {
      T high = 0, target = 0;
      for (size_t c = 0; c < predictions_[i].size(); ++c)
        if (predictions_[i][c] > high) {
          high = predictions_[i][c];
          target = T(c);
        }
      if (std::abs(target - targets[i]) < 0.001) acc += 1;
    }
    return acc / targets.size();
  }
  T GetSingleValue(string name) override { return single_[name]; }
  col_array<T>& GetMultipleValue(string name) override { return multiple_[name]; }
  string ToString() override {
    string r;
    for (auto& p : single_) r += p.first + std::to_string(p.second) + "\r\n";
    for (auto& p : multiple_) {
      r += p.first + "[";
      for (auto& v : p.second) r += std::to_string(v) + ",";
      r += "]\r\n";
    }
    return r;
  }
  MlResultData<T>& operator+=(const MlResultData<T>& rhs) override {
    const auto& o = rhs.GetPredictions();
    for (size_t i = 0; i < predictions_.size() && i < o.size(); ++i)
      for (size_t c = 0; c < predictions_[i].size() && c < o[i].size(); ++c)
        predictions_[i][c] += o[i][c];
    return *this;
  }
  const col_array<col_array<T>>& GetPredictions() const override { return predictions_; }

 private:
  col_array<col_array<T>> predictions_;
  col_map<string, T> single_;
  col_map<string, col_array<T>> multiple_;
};
}  // namespace

DataInterface& DataInterface::GetInstance() {
  static DataInterface instance;
  return instance;
}
template <typename T>
sp<MlDataFrame<T>> DataInterface::CreateDataFrame() {
  return std::make_shared<MlDataFrameImpl<T>>();
}
template <typename T>
sp<MlResultData<T>> DataInterface::CreateResultData() {
  return std::make_shared<MlResultDataImpl<T>>();
}
template sp<MlDataFrame<float>> DataInterface::CreateDataFrame<float>();
template sp<MlDataFrame<double>> DataInterface::CreateDataFrame<double>();
template sp<MlResultData<float>> DataInterface::CreateResultData<float>();
template sp<MlResultData<double>> DataInterface::CreateResultData<double>();
}  // namespace lib_data

// ----------------------------------------------------------------- models
namespace lib_models {
namespace {
class MlModelImpl : public MlModel {
 public:
  bool Has(const int id) override { return id >= 0 && id < (int)data_.size() && !data_[id].empty(); }

 private:
  void AddData(const int id, sutil::any_type d) override {
    while (id >= (int)data_.size()) data_.emplace_back();
    data_[id] = std::move(d);
  }
  sutil::any_type& GetData(const int id) override {
    if (!Has(id)) CoreLib::GetInstance().ThrowException("model slot " + std::to_string(id) + " is empty");
    return data_[id];
  }
  col_array<sutil::any_type> data_;
};
}  // namespace
ModelsInterface& ModelsInterface::GetInstance() {
  static ModelsInterface instance;
  return instance;
}
sp<MlModel> ModelsInterface::CreateModel() { return std::make_shared<MlModelImpl>(); }
}  // namespace lib_models

// ------------------------------------------------------------- algorithms
namespace lib_algorithms {
namespace {
class MlAlgorithmParamsImpl : public MlAlgorithmParams {
 public:
  explicit MlAlgorithmParamsImpl(int n) : params_(n) {}
  bool Has(const int p) override { return p >= 0 && p < (int)params_.size() && !params_[p].empty(); }
  sp<MlAlgorithmParams> Clone() override {
    auto c = std::make_shared<MlAlgorithmParamsImpl>((int)params_.size());
    c->params_ = params_;
    return c;
  }

 private:
  void SetParam(const int p, const sutil::any_type v) override {
    if (p >= (int)params_.size()) params_.resize(p + 1);
    params_[p] = v;
  }
  sutil::any_type& GetParam(const int p) override {
    if (!Has(p)) CoreLib::GetInstance().ThrowException("parameter " + std::to_string(p) + " is not set");
    return params_[p];
  }
  col_array<sutil::any_type> params_;
};
}  // namespace
AlgorithmsInterface& AlgorithmsInterface::GetInstance() {
  static AlgorithmsInterface instance;
  return instance;
}
sp<MlAlgorithmParams> AlgorithmsInterface::CreateAlgorithmParams(int size) {
  return std::make_shared<MlAlgorithmParamsImpl>(size);
}
}  // namespace lib_algorithms

namespace lib_algorithms {
namespace {
// GpuAlgorithm<T>: the trees of a fit, or of a predict, spread over the
// visible GPUs with one host thread each (gpu_algorithm.cc:17-50).
template <typename T>
class GpuAlgorithm : public MlAlgorithm<T> {
  using MlModel = lib_models::MlModel;
  template <typename U>
  using MlDataFrame = lib_data::MlDataFrame<U>;
  template <typename U>
  using MlResultData = lib_data::MlResultData<U>;

 public:
  explicit GpuAlgorithm(sp<MlAlgorithm<T>> dev) : dev_(std::move(dev)) {}

  sp<MlModel> Fit(sp<MlDataFrame<T>> data, sp<MlAlgorithmParams> params) override {
    int count = devices(params);
    if (count <= 1) return dev_->Fit(data, params);
    auto packs = SplitParameterPack(params, count);
    col_array<sp<MlModel>> models(count);
    run(count, [&](int i) {
      packs[i]->Set(EnsemblesLib::kDevId, i);
      models[i] = dev_->Fit(data, packs[i]);
    });
    return AggregateModels(models);
  }

  sp<MlResultData<T>> Predict(sp<MlDataFrame<T>> data, sp<MlModel> model,
                              sp<MlAlgorithmParams> params) override {
    int count = devices(params);
    if (count <= 1) return dev_->Predict(data, model, params);
    auto parts = SplitModel(model, count);
    col_array<sp<MlResultData<T>>> results(count);
    run(count, [&](int i) { results[i] = dev_->Predict(data, parts[i], params); });
    return AggregateResults(results);
  }

  sp<MlModel> AggregateModels(col_array<sp<MlModel>> m) override { return dev_->AggregateModels(m); }
  col_array<sp<MlModel>> SplitModel(sp<MlModel> m, const int parts) override {
    return dev_->SplitModel(m, parts);
  }
  sp<MlResultData<T>> AggregateResults(col_array<sp<MlResultData<T>>> r) override {
    return dev_->AggregateResults(r);
  }
  col_array<sp<MlAlgorithmParams>> SplitParameterPack(sp<MlAlgorithmParams> p, const int parts) override {
    return dev_->SplitParameterPack(p, parts);
  }

 private:
  static int devices(const sp<MlAlgorithmParams>& params) {
    int n = 1;
    if (dml_device_count(&n) != DML_OK) n = 1;
    // an explicit kDevId keeps the work on that one device
    if (params->Has(EnsemblesLib::kDevId) && params->Get<int>(EnsemblesLib::kDevId) > 0) return 1;
    return std::max(1, n);
  }
  template <class Fn>
  static void run(int count, Fn fn) {
    std::vector<std::thread> th;
    std::vector<std::exception_ptr> err(count);
    for (int i = 0; i < count; ++i)
      th.emplace_back([&, i] {
        try {
          if (dml_set_device(i) != DML_OK) throw_status(DML_ERR_CUDA, "device selection");
          fn(i);
        } catch (...) {
          err[i] = std::current_exception();
        }
      });
    for (auto& t : th) t.join();
    for (auto& e : err)
      if (e) std::rethrow_exception(e);
  }
  sp<MlAlgorithm<T>> dev_;
};
}  // namespace

template <typename T>
sp<MlAlgorithm<T>> AlgorithmsInterface::CreateGpuAlgorithm(sp<MlAlgorithm<T>> algo) {
  if (!algo) CoreLib::GetInstance().ThrowException("CreateGpuAlgorithm: no algorithm");
  return std::make_shared<GpuAlgorithm<T>>(std::move(algo));
}
template sp<MlAlgorithm<float>> AlgorithmsInterface::CreateGpuAlgorithm<float>(
    sp<MlAlgorithm<float>>);
template sp<MlAlgorithm<double>> AlgorithmsInterface::CreateGpuAlgorithm<double>(
    sp<MlAlgorithm<double>>);
}  // namespace lib_algorithms

// -------------------------------------------------------------- ensembles
namespace lib_ensembles {
namespace {
using lib_algorithms::MlAlgorithm;
using lib_algorithms::MlAlgorithmParams;
using lib_data::MlDataFrame;
using lib_data::MlResultData;
using lib_models::MlModel;
template <typename T>
using Node = GpuDteAlgorithmShared::gpuDTE_NodeHeader_Classify<T>;

// model slot holding the device-resident forest of a fitted model
constexpr int kDeviceForestSlot = ModelsLib::kGpuDteModelEndMarker;

struct DeviceForest {
  dml_forest* f = nullptr;
  ~DeviceForest() { dml_forest_free(f); }
};

int get_int(const sp<MlAlgorithmParams>& p, int id, int dflt) {
  return p->Has(id) ? p->Get<int>(id) : dflt;
}

// A pack of this library holding every parameter of `src` that it has, each
// read with the type the reference stores it as (ensembles_interface.cc:28-58):
// the copy SplitParameterPack makes of a pack class that cannot clone itself.
sp<MlAlgorithmParams> copy_reference_params(const sp<MlAlgorithmParams>& src) {
  auto q = AlgorithmsLib::GetInstance().CreateAlgorithmParams(EnsemblesLib::kGb300EndMarker);
  const int ints[] = {EnsemblesLib::kDevId,   EnsemblesLib::kNrTrees,    EnsemblesLib::kNrFeatures,
                      EnsemblesLib::kMaxDepth, EnsemblesLib::kMinNodeSize, EnsemblesLib::kMinLeaf,
                      EnsemblesLib::kSeed,    EnsemblesLib::kTreeOffset};
  for (int id : ints)
    if (src->Has(id)) q->Set(id, src->Get<int>(id));
  if (src->Has(EnsemblesLib::kAlgoType))
    q->Set(EnsemblesLib::kAlgoType,
           src->Get<AlgorithmsLib::AlgorithmType>(EnsemblesLib::kAlgoType));
  for (int id : {(int)EnsemblesLib::kEasyEnsemble, (int)EnsemblesLib::kBagging})
    if (src->Has(id)) q->Set(id, src->Get<bool>(id));
  return q;
}

// The device forest of a model: the fitted one, or one imported from the
// kNodeArray / kProbArray slots (e.g. after AggregateModels).
template <typename T>
dml_forest* device_forest(const sp<MlModel>& model) {
  if (model->Has(kDeviceForestSlot))
    return model->Get<sp<DeviceForest>>(kDeviceForestSlot)->f;
  auto& nodes = model->Get<col_array<Node<T>>>(ModelsLib::kNodeArray);
  auto& probs = model->Get<col_array<T>>(ModelsLib::kProbArray);
  const int task = model->Get<AlgorithmsLib::AlgorithmType>(ModelsLib::kModelType);
  std::vector<int32_t> raw(nodes.size() * 5);
  for (size_t i = 0; i < nodes.size(); ++i) {
    raw[5 * i + 0] = nodes[i].child_start;
    raw[5 * i + 1] = nodes[i].child_count;
    raw[5 * i + 2] = nodes[i].probability_start;
    raw[5 * i + 3] = nodes[i].attribute;
    float sp32 = (float)nodes[i].split_point;
    std::memcpy(&raw[5 * i + 4], &sp32, 4);
  }
  std::vector<float> pr(probs.begin(), probs.end());
  auto h = std::make_shared<DeviceForest>();
  dml_status st = dml_forest_import(task, model->Get<int>(ModelsLib::kNrTrees),
                                    model->Get<int>(ModelsLib::kNrTargets),
                                    model->Get<int>(ModelsLib::kNrFeatures), raw.data(),
                                    (int64_t)nodes.size(), pr.data(), (int64_t)pr.size(), &h->f);
  if (st != DML_OK) throw_status(st, "model import");
  model->Add(kDeviceForestSlot, h);
  return h->f;
}

// Appends tree `root` of (nodes, probs) to (out_nodes, out_probs): the root
// at root_slot, descendants as child pairs in depth-first order with child and
// probability offsets rebased (gpudte_algorithm.cc:370-387).
template <typename T>
void append_tree(const col_array<Node<T>>& nodes, const col_array<T>& probs, int C, int root,
                 int root_slot, col_array<Node<T>>& out_nodes, col_array<T>& out_probs) {
  std::vector<std::pair<int, int>> stack;  // (source node, destination slot)
  out_nodes[root_slot] = nodes[root];
  stack.emplace_back(root, root_slot);
  while (!stack.empty()) {
    auto [src, dst] = stack.back();
    stack.pop_back();
    const Node<T>& n = nodes[src];
    if (n.child_count > 0) {
      const int cs = (int)out_nodes.size();
      for (int c = 0; c < n.child_count; ++c) out_nodes.push_back(nodes[n.child_start + c]);
      out_nodes[dst].child_start = cs;
      for (int c = n.child_count - 1; c >= 0; --c) stack.emplace_back(n.child_start + c, cs + c);
    } else {
      const int ps = (int)out_probs.size();
      for (int c = 0; c < C; ++c) out_probs.push_back(probs[n.probability_start + c]);
      out_nodes[dst].probability_start = ps;
    }
  }
}

// The engine fits and predicts in FP32 (its gains, thresholds and tie rules are
// pinned for FP32).  A double frame (the reference's MlAlgorithm<double>,
// gpudte.cu:391-420) is fitted only when every value is a float exactly:
// then the sort order, the candidate boundaries and the partitions are the ones
// the values define, and the fit equals the float frame's.  Any other value is
// refused with an exception naming it, never narrowed silently.  Thresholds
// are float midpoints, widened exactly into the model's double split points.
template <typename T>
std::vector<float> exact_floats(const col_array<T>& v, const char* what) {
  std::vector<float> out(v.size());
  for (size_t i = 0; i < v.size(); ++i) {
    out[i] = (float)v[i];
    if (!((T)out[i] == v[i]) && !(v[i] != v[i])) {
      char buf[160];
      std::snprintf(buf, sizeof(buf),
                    "Fit: %s %zu (%.17g) is not exactly a float; this engine fits in FP32 and "
                    "takes double frames whose values are floats", what, i, (double)v[i]);
      CoreLib::GetInstance().ThrowException(buf);
    }
  }
  return out;
}

// Predict values for the FP32 walk: each value rounded toward -infinity to a
// float (values below -FLT_MAX become -FLT_MAX, which goes left like any value
// below a threshold).  For a float threshold t, x < t exactly when the rounded
// value is below t, so a double frame gets the votes the reference's double
// comparison gives on this model's thresholds.
template <typename T>
std::vector<float> rounded_down(const col_array<T>& v) {
  std::vector<float> out(v.size());
  for (size_t i = 0; i < v.size(); ++i) {
    const T x = v[i];
    float f = (float)x;
    if (x != x) {
      out[i] = f;
      continue;
    }
    if ((T)f > x) f = std::nextafter(f, -INFINITY);
    if (f < -FLT_MAX) f = -FLT_MAX;
    out[i] = f;
  }
  return out;
}

// Fit / Predict of one device (GpuDteAlgorithm<T>).
template <typename T>
class DteAlgorithm : public MlAlgorithm<T> {
 public:
  explicit DteAlgorithm(int algo) : algo_(algo) {}

  sp<MlModel> Fit(sp<MlDataFrame<T>> data, sp<MlAlgorithmParams> params) override {
    const int N = data->GetNrSamples(), F = data->GetNrFeatures();
    const auto type = params->Has(EnsemblesLib::kAlgoType)
                          ? params->Get<AlgorithmsLib::AlgorithmType>(EnsemblesLib::kAlgoType)
                          : AlgorithmsLib::kClassification;
    const int C = type == AlgorithmsLib::kClassification ? data->GetNrTargets() : 1;
    if ((long long)N * F != (long long)data->GetSamples().size())
      CoreLib::GetInstance().ThrowException("data frame: samples do not hold features x rows values");
    std::vector<float> xs = exact_floats(data->GetSamples(), "sample");
    std::vector<float> ys = exact_floats(data->GetTargets(), "target");
    dml_fit_desc d;
    std::memset(&d, 0, sizeof(d));
    d.algo = algo_;
    d.task = type;
    d.n_trees = params->Get<int>(EnsemblesLib::kNrTrees);
    d.n_features_try = get_int(params, EnsemblesLib::kNrFeatures, 0);
    d.max_depth = get_int(params, EnsemblesLib::kMaxDepth, 1000);
    d.min_node_size = get_int(params, EnsemblesLib::kMinNodeSize, 5);
    d.min_leaf = get_int(params, EnsemblesLib::kMinLeaf, 1);
    d.n_classes = C;
    d.seed = (uint64_t)get_int(params, EnsemblesLib::kSeed, 0);
    d.n_rows = N;
    d.n_features = F;
    d.memory = DML_HOST;
    d.samples = xs.data();
    d.targets = ys.data();
    d.tree_offset = get_int(params, EnsemblesLib::kTreeOffset, 0);
    // kEasyEnsemble is read by the reference's RF bootstrap only (gpurf.cu:63-100,
    // gpudte_algorithm.cc:582-583); ERT uses every row
    d.balanced = algo_ == DML_ALGO_RF && type == AlgorithmsLib::kClassification &&
                 params->Has(EnsemblesLib::kEasyEnsemble) &&
                 params->Get<bool>(EnsemblesLib::kEasyEnsemble);
    auto h = std::make_shared<DeviceForest>();
    dml_status st = dml_fit(&d, &h->f, nullptr);
    if (st != DML_OK) throw_status(st, "Fit");
    dml_forest_info info;
    dml_forest_info_get(h->f, &info);
    std::vector<int32_t> raw((size_t)info.n_nodes * 5);
    std::vector<float> pr((size_t)info.n_probs);
    st = dml_forest_export(h->f, raw.data(), pr.data());
    if (st != DML_OK) throw_status(st, "Fit (model export)");
    col_array<Node<T>> nodes((size_t)info.n_nodes);
    for (size_t i = 0; i < nodes.size(); ++i) {
      nodes[i].child_start = raw[5 * i + 0];
      nodes[i].child_count = raw[5 * i + 1];
      nodes[i].probability_start = raw[5 * i + 2];
      nodes[i].attribute = raw[5 * i + 3];
      float sp32;
      std::memcpy(&sp32, &raw[5 * i + 4], 4);
      nodes[i].split_point = (T)sp32;
    }
    auto model = ModelsLib::GetInstance().CreateModel();
    model->Add(ModelsLib::kNrTrees, d.n_trees);
    model->Add(ModelsLib::kNrFeatures, F);
    model->Add(ModelsLib::kNrTargets, C);
    model->Add(ModelsLib::kModelType, type);
    model->Add(ModelsLib::kNodeArray, nodes);
    model->Add(ModelsLib::kProbArray, col_array<T>(pr.begin(), pr.end()));
    model->Add(kDeviceForestSlot, h);
    return model;
  }

  sp<MlResultData<T>> Predict(sp<MlDataFrame<T>> data, sp<MlModel> model,
                              sp<MlAlgorithmParams> params) override {
    (void)params;
    dml_forest* f = device_forest<T>(model);
    const int N = data->GetNrSamples();
    dml_forest_info info;
    dml_forest_info_get(f, &info);
    const int width = info.task == DML_CLASSIFICATION ? info.n_classes : 1;
    std::vector<float> xs = rounded_down(data->GetSamples());
    if ((long long)xs.size() != (long long)N * info.n_features)
      CoreLib::GetInstance().ThrowException("Predict: the frame's feature count differs from the model's");
    std::vector<float> out((size_t)N * width);
    dml_status st = dml_predict(f, xs.data(), N, out.data(), DML_HOST, nullptr);
    if (st != DML_OK) throw_status(st, "Predict");
    col_array<col_array<T>> preds(N);
    for (int i = 0; i < N; ++i)
      preds[i].assign(out.begin() + (size_t)i * width, out.begin() + (size_t)(i + 1) * width);
    auto r = DataLib::GetInstance().CreateResultData<T>();
    r->AddPredictions(std::move(preds));
    return r;
  }

  // Roots of every model first, then each tree's descendants
  // (gpudte_algorithm.cc:334-397).
  sp<MlModel> AggregateModels(col_array<sp<MlModel>> models) override {
    if (models.empty()) CoreLib::GetInstance().ThrowException("AggregateModels: no models");
    if (models.size() == 1) return models[0];
    int total = 0;
    for (auto& m : models) total += m->Get<int>(ModelsLib::kNrTrees);
    const int C = models[0]->Get<int>(ModelsLib::kNrTargets);
    col_array<Node<T>> nodes(total);
    col_array<T> probs;
    int t0 = 0;
    for (auto& m : models) {
      auto& mn = m->Get<col_array<Node<T>>>(ModelsLib::kNodeArray);
      auto& mp = m->Get<col_array<T>>(ModelsLib::kProbArray);
      const int trees = m->Get<int>(ModelsLib::kNrTrees);
      for (int t = 0; t < trees; ++t) append_tree<T>(mn, mp, C, t, t0 + t, nodes, probs);
      t0 += trees;
    }
    auto out = ModelsLib::GetInstance().CreateModel();
    out->Add(ModelsLib::kNrTrees, total);
    out->Add(ModelsLib::kNrFeatures, models[0]->Get<int>(ModelsLib::kNrFeatures));
    out->Add(ModelsLib::kNrTargets, C);
    out->Add(ModelsLib::kModelType, models[0]->Get<AlgorithmsLib::AlgorithmType>(ModelsLib::kModelType));
    out->Add(ModelsLib::kNodeArray, nodes);
    out->Add(ModelsLib::kProbArray, probs);
    return out;
  }

  // Trees split into `parts` consecutive groups (gpudte_algorithm.cc:400-463);
  // the remainder of an uneven split goes to the first groups.
  col_array<sp<MlModel>> SplitModel(sp<MlModel> model, const int parts) override {
    const int trees = model->Get<int>(ModelsLib::kNrTrees);
    const int C = model->Get<int>(ModelsLib::kNrTargets);
    auto& mn = model->Get<col_array<Node<T>>>(ModelsLib::kNodeArray);
    auto& mp = model->Get<col_array<T>>(ModelsLib::kProbArray);
    col_array<sp<MlModel>> out;
    int t0 = 0;
    for (int p = 0; p < parts; ++p) {
      const int k = trees / parts + (p < trees % parts ? 1 : 0);
      col_array<Node<T>> nodes(k);
      col_array<T> probs;
      for (int t = 0; t < k; ++t) append_tree<T>(mn, mp, C, t0 + t, t, nodes, probs);
      auto m = ModelsLib::GetInstance().CreateModel();
      m->Add(ModelsLib::kNrTrees, k);
      m->Add(ModelsLib::kNrFeatures, model->Get<int>(ModelsLib::kNrFeatures));
      m->Add(ModelsLib::kNrTargets, C);
      m->Add(ModelsLib::kModelType, model->Get<AlgorithmsLib::AlgorithmType>(ModelsLib::kModelType));
      m->Add(ModelsLib::kNodeArray, nodes);
      m->Add(ModelsLib::kProbArray, probs);
      out.push_back(m);
      t0 += k;
    }
    return out;
  }

  // Element-wise sum of the vote matrices (gpudte_algorithm.cc:466-470).
  sp<MlResultData<T>> AggregateResults(col_array<sp<MlResultData<T>>> results) override {
    for (size_t i = 1; i < results.size(); ++i) *results[0] += *results[i];
    return results[0];
  }

  // Every parameter is kept; the trees are split over the parts and each part
  // carries the RNG key of its first tree.
  col_array<sp<MlAlgorithmParams>> SplitParameterPack(sp<MlAlgorithmParams> params,
                                                      const int parts) override {
    const int trees = params->Get<int>(EnsemblesLib::kNrTrees);
    const int off0 = get_int(params, EnsemblesLib::kTreeOffset, 0);
    col_array<sp<MlAlgorithmParams>> out;
    int t0 = 0;
    for (int p = 0; p < parts; ++p) {
      const int k = trees / parts + (p < trees % parts ? 1 : 0);
      auto q = params->Clone();
      if (!q) q = copy_reference_params(params);
      q->Set(EnsemblesLib::kNrTrees, k);
      q->Set(EnsemblesLib::kTreeOffset, off0 + t0);
      out.push_back(q);
      t0 += k;
    }
    return out;
  }

 private:
  int algo_;
};

}  // namespace

EnsemblesInterface& EnsemblesInterface::GetInstance() {
  static EnsemblesInterface instance;
  return instance;
}

template <typename T>
sp<lib_algorithms::MlAlgorithm<T>> EnsemblesInterface::CreateGpuRfAlgorithm() {
  return AlgorithmsLib::GetInstance().CreateGpuAlgorithm<T>(
      std::make_shared<DteAlgorithm<T>>(DML_ALGO_RF));
}
template <typename T>
sp<lib_algorithms::MlAlgorithm<T>> EnsemblesInterface::CreateGpuErtAlgorithm() {
  return AlgorithmsLib::GetInstance().CreateGpuAlgorithm<T>(
      std::make_shared<DteAlgorithm<T>>(DML_ALGO_ERT));
}

static sp<lib_algorithms::MlAlgorithmParams> default_pack(bool bagging) {
  auto p = AlgorithmsLib::GetInstance().CreateAlgorithmParams(EnsemblesInterface::kGb300EndMarker);
  p->Set(EnsemblesInterface::kNrTrees, 100);
  p->Set(EnsemblesInterface::kNrFeatures, 0);
  p->Set(EnsemblesInterface::kMaxDepth, 1000);
  p->Set(EnsemblesInterface::kMinNodeSize, 5);
  p->Set(EnsemblesInterface::kAlgoType, AlgorithmsLib::kClassification);
  p->Set(EnsemblesInterface::kBagging, bagging);
  p->Set(EnsemblesInterface::kEasyEnsemble, false);
  p->Set(EnsemblesInterface::kMinLeaf, 1);
  p->Set(EnsemblesInterface::kSeed, 0);
  return p;
}
sp<lib_algorithms::MlAlgorithmParams> EnsemblesInterface::CreateGpuRfParamPack() {
  return default_pack(true);
}
sp<lib_algorithms::MlAlgorithmParams> EnsemblesInterface::CreateGpuErtParamPack() {
  return default_pack(false);
}

template sp<lib_algorithms::MlAlgorithm<float>> EnsemblesInterface::CreateGpuRfAlgorithm<float>();
template sp<lib_algorithms::MlAlgorithm<double>> EnsemblesInterface::CreateGpuRfAlgorithm<double>();
template sp<lib_algorithms::MlAlgorithm<float>> EnsemblesInterface::CreateGpuErtAlgorithm<float>();
template sp<lib_algorithms::MlAlgorithm<double>> EnsemblesInterface::CreateGpuErtAlgorithm<double>();
}  // namespace lib_ensembles

// ---------------------------------------------------------------- parsing
namespace lib_parsing {
namespace {
// Commas and tabs separate cells like white space (csv_parser.h: csv_ctype).
struct csv_ctype : std::ctype<char> {
  mask table_[table_size];
  csv_ctype() : std::ctype<char>(table_, false, 0) {
    std::copy_n(classic_table(), table_size, table_);
    table_[(unsigned char)','] = (mask)space;
    table_[(unsigned char)'\t'] = (mask)space;
  }
};

// One header line naming the columns, then one row per line; a cell that
// does not read as a number gets the next ordinal code of its column (first
// seen, first numbered); the last column is the target; samples are stored
// feature-major (csv_parser.cc:36-104).  Blank lines end the data.
template <typename T>
bool parse_csv(const sp<lib_data::MlDataFrame<T>>& data, std::istream& in) {
  std::locale loc(std::locale::classic(), new csv_ctype);
  string line;
  if (!std::getline(in, line)) return false;
  col_array<string> names;
  {
    std::istringstream ls(line);
    ls.imbue(loc);
    std::copy(std::istream_iterator<string>(ls), std::istream_iterator<string>(),
              std::back_inserter(names));
  }
  if (names.size() < 2) return false;
  const size_t ncol = names.size();
  col_array<col_map<string, T>> maps(ncol);
  col_array<T> next_id(ncol, 0);
  col_array<col_array<T>> cols(ncol - 1);
  col_array<T> targets;
  bool any = false;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    ls.imbue(loc);
    col_array<string> cells;
    std::copy(std::istream_iterator<string>(ls), std::istream_iterator<string>(),
              std::back_inserter(cells));
    if (cells.empty()) break;
    if (cells.size() != ncol) return false;
    for (size_t c = 0; c < ncol; ++c) {
      std::istringstream ps(cells[c]);
      T v;
      ps >> v;
      if (ps.fail()) {
        auto it = maps[c].find(cells[c]);
        if (it == maps[c].end()) it = maps[c].emplace(cells[c], next_id[c]++).first;
        v = it->second;
      } else {
        maps[c][cells[c]] = v;
      }
      if (c + 1 == ncol)
        targets.push_back(v);
      else
        cols[c].push_back(v);
    }
    any = true;
  }
  if (!any) return false;
  col_array<T> packed;
  packed.reserve(cols.size() * targets.size());
  for (auto& c : cols) packed.insert(packed.end(), c.begin(), c.end());
  data->AddTargetData(targets);
  data->AddSampleData(packed);
  data->AddTargetMap(maps.back());
  maps.pop_back();
  data->AddFeatureMap(maps);
  return true;
}
}  // namespace

ParsingInterface& ParsingInterface::GetInstance() {
  static ParsingInterface instance;
  return instance;
}

template <typename T>
sp<lib_data::MlDataFrame<T>> ParsingInterface::ParseData(ParserType type, col_array<char>& raw) {
  if (type != kCsv) CoreLib::GetInstance().ThrowException("only the CSV parser is available");
  auto data = DataLib::GetInstance().CreateDataFrame<T>();
  string text(raw.begin(), std::find(raw.begin(), raw.end(), '\0'));
  std::istringstream in(text);
  if (raw.empty() || !parse_csv<T>(data, in)) CoreLib::GetInstance().ThrowException("Parsing failed.");
  return data;
}

template <typename T>
sp<lib_data::MlDataFrame<T>> ParsingInterface::ParseFile(ParserType type, string path) {
  if (type != kCsv) CoreLib::GetInstance().ThrowException("only the CSV parser is available");
  auto data = DataLib::GetInstance().CreateDataFrame<T>();
  std::ifstream in(path);
  if (!in || !parse_csv<T>(data, in)) CoreLib::GetInstance().ThrowException("Parsing failed.");
  return data;
}

template sp<lib_data::MlDataFrame<float>> ParsingInterface::ParseData<float>(ParserType, col_array<char>&);
template sp<lib_data::MlDataFrame<double>> ParsingInterface::ParseData<double>(ParserType, col_array<char>&);
template sp<lib_data::MlDataFrame<float>> ParsingInterface::ParseFile<float>(ParserType, string);
template sp<lib_data::MlDataFrame<double>> ParsingInterface::ParseFile<double>(ParserType, string);
}  // namespace lib_parsing
