// A program written against the reference's own interfaces, the way the
// reference's code uses them, compiled unchanged against the drop-in
// (datamininglibs_gb300/shim):
//   * a parameter pack class with SetParam / GetParam only, as
//     lib_algorithms/source/ml_algorithm_params_impl.{h,cc} is written;
//   * a model class with AddData / GetData only, as
//     lib_models/source/ml_model_impl.{h,cc} is written;
//   * a single-device algorithm wrapped into the multi-device one through
//     AlgorithmsInterface::CreateGpuAlgorithm<T>, the pattern of
//     lib_ensembles/source/ensembles_interface.cc:14-26.
// Modes:
//   host                       the pack and model classes and SplitParameterPack
//                              through the wrapper (no GPU)
//   fit <data.bin>             fits through the wrapper with the reference-style
//                              pack, predicts through a reference-style model,
//                              and the double-frame rules (GPU)
#include <datamininglibs.h>

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>

#define CHECK(x)                                                     \
  do {                                                               \
    if (!(x)) {                                                      \
      std::cerr << "CHECK failed: " #x " line " << __LINE__ << "\n"; \
      return 1;                                                      \
    }                                                                \
  } while (0)

class RefStyleParams : public lib_algorithms::MlAlgorithmParams {
 public:
  explicit RefStyleParams(int nr_params) {
    params_ = col_array<sutil::any_type>(nr_params, sutil::any_type());
  }

 private:
  void SetParam(const int param, const sutil::any_type value) override {
    params_[param] = std::move(value);
  }
  sutil::any_type& GetParam(const int param) override { return params_[param]; }
  col_array<sutil::any_type> params_;
};

class RefStyleModel : public lib_models::MlModel {
 private:
  void AddData(const int id, const sutil::any_type data) override {
    while (id >= (int)data_.size()) data_.emplace_back(sutil::any_type());
    data_[id] = std::move(data);
  }
  sutil::any_type& GetData(const int id) override { return data_[id]; }
  col_array<sutil::any_type> data_;
};

// A user's single-device algorithm: counts its calls and delegates to the
// library's RF algorithm.
template <typename T>
class CountingRf : public lib_algorithms::MlAlgorithm<T> {
 public:
  CountingRf() : inner_(EnsemblesLib::GetInstance().CreateGpuRfAlgorithm<T>()) {}
  sp<lib_models::MlModel> Fit(sp<lib_data::MlDataFrame<T>> data,
                              sp<lib_algorithms::MlAlgorithmParams> params) override {
    ++fits;
    return inner_->Fit(data, params);
  }
  sp<lib_data::MlResultData<T>> Predict(sp<lib_data::MlDataFrame<T>> data,
                                        sp<lib_models::MlModel> model,
                                        sp<lib_algorithms::MlAlgorithmParams> params) override {
    ++predicts;
    return inner_->Predict(data, model, params);
  }
  sp<lib_models::MlModel> AggregateModels(col_array<sp<lib_models::MlModel>> models) override {
    return inner_->AggregateModels(models);
  }
  col_array<sp<lib_models::MlModel>> SplitModel(sp<lib_models::MlModel> model,
                                                const int parts) override {
    return inner_->SplitModel(model, parts);
  }
  sp<lib_data::MlResultData<T>> AggregateResults(
      col_array<sp<lib_data::MlResultData<T>>> results) override {
    return inner_->AggregateResults(results);
  }
  col_array<sp<lib_algorithms::MlAlgorithmParams>> SplitParameterPack(
      sp<lib_algorithms::MlAlgorithmParams> params, const int parts) override {
    return inner_->SplitParameterPack(params, parts);
  }
  int fits = 0, predicts = 0;

 private:
  sp<lib_algorithms::MlAlgorithm<T>> inner_;
};

// ensembles_interface.cc:14-26, with the user's algorithm in place of
// GpuDteAlgorithm<T>
template <typename T>
sp<lib_algorithms::MlAlgorithm<T>> CreateMyRf(sp<CountingRf<T>>& counter) {
  auto algo = std::make_shared<CountingRf<T>>();
  counter = algo;
  return AlgorithmsLib::GetInstance().CreateGpuAlgorithm<T>(algo);
}

// ensembles_interface.cc:28-42 on the reference-style pack class
static sp<lib_algorithms::MlAlgorithmParams> ref_style_rf_pack() {
  auto params = std::make_shared<RefStyleParams>(EnsemblesLib::kDteEndMarker);
  params->Set(EnsemblesLib::kNrTrees, 100);
  params->Set(EnsemblesLib::kNrFeatures, 0);
  params->Set(EnsemblesLib::kMaxDepth, 1000);
  params->Set(EnsemblesLib::kMinNodeSize, 5);
  params->Set(EnsemblesLib::kAlgoType, AlgorithmsLib::kClassification);
  params->Set(EnsemblesLib::kBagging, true);
  params->Set(EnsemblesLib::kEasyEnsemble, false);
  return params;
}

static int host_checks() {
  auto p = ref_style_rf_pack();
  CHECK(p->Has(EnsemblesLib::kNrTrees));
  CHECK(!p->Has(EnsemblesLib::kDevId));    // never set
  CHECK(!p->Has(EnsemblesLib::kMinLeaf));  // past the reference's ids
  CHECK(p->Clone() == nullptr);
  p->Set(EnsemblesLib::kNrTrees, 10);
  p->Set(EnsemblesLib::kMaxDepth, 7);
  sp<CountingRf<float>> counter;
  auto rf = CreateMyRf<float>(counter);
  auto packs = rf->SplitParameterPack(p, 3);
  CHECK(packs.size() == 3);
  const int want[3] = {4, 3, 3};
  int off = 0;
  for (int i = 0; i < 3; ++i) {
    CHECK(packs[i]->Get<int>(EnsemblesLib::kNrTrees) == want[i]);
    CHECK(packs[i]->Get<int>(EnsemblesLib::kTreeOffset) == off);
    CHECK(packs[i]->Get<int>(EnsemblesLib::kMaxDepth) == 7);
    CHECK(packs[i]->Get<int>(EnsemblesLib::kMinNodeSize) == 5);
    CHECK(packs[i]->Get<bool>(EnsemblesLib::kBagging));
    CHECK(packs[i]->Get<AlgorithmsLib::AlgorithmType>(EnsemblesLib::kAlgoType) ==
          AlgorithmsLib::kClassification);
    off += want[i];
  }
  CHECK(p->Get<int>(EnsemblesLib::kNrTrees) == 10);
  auto m = std::make_shared<RefStyleModel>();
  m->Add(ModelsLib::kNrTrees, 3);
  CHECK(m->Has(ModelsLib::kNrTrees));
  CHECK(!m->Has(ModelsLib::kGpuDteModelEndMarker));
  std::cout << "host ok\n";
  return 0;
}

using Node = lib_ensembles::GpuDteAlgorithmShared::gpuDTE_NodeHeader_Classify<double>;

// Votes of a double-precision walk of the model on the host: x < split_point
// goes left, -FLT_MAX is missing and goes left (gpudte.cu:311-359).
static std::vector<double> host_votes(const sp<lib_models::MlModel>& m,
                                      const std::vector<double>& X, int N, int F, int C) {
  auto& nodes = m->Get<std::vector<Node>>(ModelsLib::kNodeArray);
  auto& probs = m->Get<std::vector<double>>(ModelsLib::kProbArray);
  const int T = m->Get<int>(ModelsLib::kNrTrees);
  std::vector<double> v((size_t)N * C, 0.0);
  for (int i = 0; i < N; ++i)
    for (int t = 0; t < T; ++t) {
      int k = t;
      while (nodes[k].child_count > 0) {
        const double x = X[(size_t)nodes[k].attribute * N + i];
        const bool left = x == -FLT_MAX || x < nodes[k].split_point;
        k = nodes[k].child_start + (left ? 0 : 1);
      }
      int sel = 0;
      double hi = 0;
      for (int c = 0; c < C; ++c)
        if (probs[nodes[k].probability_start + c] > hi) {
          hi = probs[nodes[k].probability_start + c];
          sel = c;
        }
      v[(size_t)i * C + sel] += 1;
    }
  (void)F;
  return v;
}

template <typename T>
static std::vector<double> flat(const sp<lib_data::MlResultData<T>>& r) {
  std::vector<double> out;
  for (auto& row : r->GetPredictions())
    for (auto x : row) out.push_back((double)x);
  return out;
}

static int fit_checks(const char* path) {
  FILE* fp = std::fopen(path, "rb");
  CHECK(fp);
  int32_t N, F, C;
  CHECK(std::fread(&N, 4, 1, fp) == 1 && std::fread(&F, 4, 1, fp) == 1 &&
        std::fread(&C, 4, 1, fp) == 1);
  std::vector<float> X((size_t)N * F), y(N);
  CHECK(std::fread(X.data(), 4, X.size(), fp) == X.size());
  CHECK(std::fread(y.data(), 4, y.size(), fp) == y.size());
  std::fclose(fp);
  auto frame = [&](auto zero) {
    using T = decltype(zero);
    auto df = DataLib::GetInstance().CreateDataFrame<T>();
    df->AddSampleData(std::vector<T>(X.begin(), X.end()));
    df->AddTargetData(std::vector<T>(y.begin(), y.end()));
    df->AddFeatureMap(std::vector<std::map<std::string, T>>(F));
    std::map<std::string, T> tmap;
    for (int c = 0; c < C; ++c) tmap[std::to_string(c)] = (T)c;
    df->AddTargetMap(tmap);
    return df;
  };
  auto df = frame(0.0f);
  auto p = ref_style_rf_pack();
  p->Set(EnsemblesLib::kNrTrees, 8);
  p->Set(EnsemblesLib::kNrFeatures, 4);
  p->Set(EnsemblesLib::kMaxDepth, 12);
  // through the wrapper with the reference-style pack, and the library's own
  // factory and pack with the same values: one forest
  sp<CountingRf<float>> counter;
  auto mine = CreateMyRf<float>(counter);
  auto m1 = mine->Fit(df, p);
  CHECK(counter->fits >= 1);
  auto lp = EnsemblesLib::GetInstance().CreateGpuRfParamPack();
  lp->Set(EnsemblesLib::kNrTrees, 8);
  lp->Set(EnsemblesLib::kNrFeatures, 4);
  lp->Set(EnsemblesLib::kMaxDepth, 12);
  auto lib_rf = EnsemblesLib::GetInstance().CreateGpuRfAlgorithm<float>();
  auto m2 = lib_rf->Fit(df, lp);
  using NodeF = lib_ensembles::GpuDteAlgorithmShared::gpuDTE_NodeHeader_Classify<float>;
  auto& n1 = m1->Get<std::vector<NodeF>>(ModelsLib::kNodeArray);
  auto& n2 = m2->Get<std::vector<NodeF>>(ModelsLib::kNodeArray);
  CHECK(n1.size() == n2.size() && std::memcmp(n1.data(), n2.data(), sizeof(NodeF) * n1.size()) == 0);
  auto r1 = mine->Predict(df, m1, p);
  CHECK(counter->predicts >= 1);
  // the model's slots copied into a reference-style model class predict alike
  auto rm = std::make_shared<RefStyleModel>();
  rm->Add(ModelsLib::kNrTrees, m1->Get<int>(ModelsLib::kNrTrees));
  rm->Add(ModelsLib::kNrTargets, m1->Get<int>(ModelsLib::kNrTargets));
  rm->Add(ModelsLib::kNrFeatures, m1->Get<int>(ModelsLib::kNrFeatures));
  rm->Add(ModelsLib::kModelType, m1->Get<AlgorithmsLib::AlgorithmType>(ModelsLib::kModelType));
  rm->Add(ModelsLib::kNodeArray, n1);
  rm->Add(ModelsLib::kProbArray, m1->Get<std::vector<float>>(ModelsLib::kProbArray));
  CHECK(flat(mine->Predict(df, rm, p)) == flat(r1));
  // double frames whose values are floats: the float forest and votes
  auto dfd = frame(0.0);
  auto rfd = EnsemblesLib::GetInstance().CreateGpuRfAlgorithm<double>();
  auto md = rfd->Fit(dfd, p);
  auto& nd = md->Get<std::vector<Node>>(ModelsLib::kNodeArray);
  CHECK(nd.size() == n1.size());
  for (size_t i = 0; i < nd.size(); ++i)
    CHECK(nd[i].attribute == n1[i].attribute && nd[i].split_point == (double)n1[i].split_point);
  CHECK(flat(rfd->Predict(dfd, md, p)) == flat(r1));
  // a double value that no float equals: the fit refuses it by name
  auto bad = frame(0.0);
  {
    std::vector<double> xs = bad->GetSamples();
    xs[5] = xs[5] + 1e-12;
    if (xs[5] == (double)(float)xs[5]) xs[5] = 0.1;
    bad->AddSampleData(xs);
  }
  bool threw = false;
  try {
    rfd->Fit(bad, p);
  } catch (lib_core::template_exception& e) {
    threw = std::string(e.what()).find("not exactly a float") != std::string::npos;
  }
  CHECK(threw);
  // predicting double values that are not floats: the votes of a double walk
  // of the model on the host
  std::vector<double> Xd(X.begin(), X.end());
  for (size_t i = 0; i < Xd.size(); ++i)
    Xd[i] = (i % 3 == 0) ? Xd[i] * (1.0 + 1e-9) : (i % 3 == 1) ? Xd[i] - 1e-10 : Xd[i];
  auto dfp = frame(0.0);
  dfp->AddSampleData(Xd);
  CHECK(flat(rfd->Predict(dfp, md, p)) == host_votes(md, Xd, N, F, C));
  std::cout << "reference style ok\n";
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::string mode = argv[1];
  if (mode == "host") return host_checks();
  if (mode == "fit" && argc >= 3) return fit_checks(argv[2]);
  return 2;
}
