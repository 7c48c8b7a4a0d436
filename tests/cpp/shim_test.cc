// Test driver of the C++ drop-in (datamininglibs_gb300/shim): written against
// the reference's public API the way its tests are
// (lib_ensembles/test/test_gpurf.h, test_gpuert.h).  Modes:
//   parse <in.csv> <out.bin>   ParsingInterface::ParseFile<float>, dumped
//   fit <data.bin> <out_dir>   RF fit/predict, split + aggregate, double frames
//   host                       host-only parts: param packs, SplitParameterPack,
//                              SplitModel / AggregateModels (no GPU needed)
#include <datamininglibs.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>

#define CHECK(x)                                                   \
  do {                                                             \
    if (!(x)) {                                                    \
      std::cerr << "CHECK failed: " #x " line " << __LINE__ << "\n"; \
      return 1;                                                    \
    }                                                              \
  } while (0)

template <class T>
static void dump(std::ofstream& f, const std::vector<T>& v) {
  int64_t n = (int64_t)v.size();
  f.write((const char*)&n, 8);
  f.write((const char*)v.data(), sizeof(T) * v.size());
}

template <typename T>
static std::vector<float> votes(const sp<lib_data::MlResultData<T>>& r) {
  std::vector<float> out;
  for (auto& row : r->GetPredictions())
    for (auto v : row) out.push_back((float)v);
  return out;
}

static std::vector<int32_t> raw_nodes(const sp<lib_models::MlModel>& m) {
  using Node = lib_ensembles::GpuDteAlgorithmShared::gpuDTE_NodeHeader_Classify<float>;
  auto& nodes = m->Get<std::vector<Node>>(ModelsLib::kNodeArray);
  std::vector<int32_t> raw;
  for (auto& n : nodes) {
    int32_t sp;
    std::memcpy(&sp, &n.split_point, 4);
    raw.insert(raw.end(), {n.child_start, n.child_count, n.probability_start, n.attribute, sp});
  }
  return raw;
}

// The host-only parts of the algorithm API.  The model is three trees in the
// layout AggregateModels writes (roots first, then each tree's child pairs in
// depth-first order, leaves' probabilities in visiting order), so splitting
// it and aggregating the parts must give it back exactly.
static int host_checks() {
  using Node = lib_ensembles::GpuDteAlgorithmShared::gpuDTE_NodeHeader_Classify<float>;
  auto& ens = EnsemblesLib::GetInstance();
  for (int e = 0; e < 2; ++e) {  // ensembles_interface.cc:28-58
    auto p = e ? ens.CreateGpuErtParamPack() : ens.CreateGpuRfParamPack();
    CHECK(p->Get<int>(EnsemblesLib::kNrTrees) == 100);
    CHECK(p->Get<int>(EnsemblesLib::kNrFeatures) == 0);
    CHECK(p->Get<int>(EnsemblesLib::kMaxDepth) == 1000);
    CHECK(p->Get<int>(EnsemblesLib::kMinNodeSize) == 5);
    CHECK(p->Get<AlgorithmsLib::AlgorithmType>(EnsemblesLib::kAlgoType) ==
          AlgorithmsLib::kClassification);
    CHECK(p->Get<bool>(EnsemblesLib::kBagging) == (e == 0));
    CHECK(!p->Get<bool>(EnsemblesLib::kEasyEnsemble));
  }
  // every user value survives the split (the reference rebuilt default packs)
  auto rf = ens.CreateGpuRfAlgorithm<float>();
  auto p = ens.CreateGpuRfParamPack();
  p->Set(EnsemblesLib::kNrTrees, 10);
  p->Set(EnsemblesLib::kNrFeatures, 5);
  p->Set(EnsemblesLib::kMaxDepth, 7);
  p->Set(EnsemblesLib::kMinNodeSize, 9);
  p->Set(EnsemblesLib::kAlgoType, AlgorithmsLib::kRegression);
  p->Set(EnsemblesLib::kMinLeaf, 3);
  p->Set(EnsemblesLib::kSeed, 11);
  auto packs = rf->SplitParameterPack(p, 3);
  CHECK(packs.size() == 3);
  const int want[3] = {4, 3, 3};
  int off = 0;
  for (int i = 0; i < 3; ++i) {
    auto& q = packs[i];
    CHECK(q->Get<int>(EnsemblesLib::kNrTrees) == want[i]);
    CHECK(q->Get<int>(EnsemblesLib::kTreeOffset) == off);
    CHECK(q->Get<int>(EnsemblesLib::kNrFeatures) == 5);
    CHECK(q->Get<int>(EnsemblesLib::kMaxDepth) == 7);
    CHECK(q->Get<int>(EnsemblesLib::kMinNodeSize) == 9);
    CHECK(q->Get<AlgorithmsLib::AlgorithmType>(EnsemblesLib::kAlgoType) ==
          AlgorithmsLib::kRegression);
    CHECK(q->Get<int>(EnsemblesLib::kMinLeaf) == 3);
    CHECK(q->Get<int>(EnsemblesLib::kSeed) == 11);
    off += want[i];
  }
  CHECK(p->Get<int>(EnsemblesLib::kNrTrees) == 10);
  // tree 0: a split with two leaves; tree 1: one leaf; tree 2: two levels
  std::vector<Node> nodes = {
      {3, 2, -1, 1, 0.5f},  {-1, 0, 4, -1, -1.0f}, {5, 2, -1, 0, 0.25f},
      {-1, 0, 0, -1, -1.0f}, {-1, 0, 2, -1, -1.0f}, {7, 2, -1, 2, 0.75f},
      {-1, 0, 10, -1, -1.0f}, {-1, 0, 6, -1, -1.0f}, {-1, 0, 8, -1, -1.0f}};
  std::vector<float> probs = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12};
  auto m = ModelsLib::GetInstance().CreateModel();
  m->Add(ModelsLib::kNrTrees, 3);
  m->Add(ModelsLib::kNrTargets, 2);
  m->Add(ModelsLib::kNrFeatures, 4);
  m->Add(ModelsLib::kModelType, AlgorithmsLib::kClassification);
  m->Add(ModelsLib::kNodeArray, nodes);
  m->Add(ModelsLib::kProbArray, probs);
  for (int k = 1; k <= 3; ++k) {
    auto parts = rf->SplitModel(m, k);
    CHECK((int)parts.size() == k);
    int trees = 0;
    for (auto& q : parts) trees += q->Get<int>(ModelsLib::kNrTrees);
    CHECK(trees == 3);
    auto agg = rf->AggregateModels(parts);
    CHECK(agg->Get<int>(ModelsLib::kNrTrees) == 3);
    CHECK(agg->Get<int>(ModelsLib::kNrTargets) == 2);
    CHECK(agg->Get<int>(ModelsLib::kNrFeatures) == 4);
    CHECK(raw_nodes(agg) == raw_nodes(m));
    CHECK(agg->Get<std::vector<float>>(ModelsLib::kProbArray) == probs);
  }
  // one tree per part: each part's root is its tree's root, children re-based
  auto single = rf->SplitModel(m, 3);
  CHECK(single[1]->Get<std::vector<Node>>(ModelsLib::kNodeArray).size() == 1);
  CHECK(single[2]->Get<std::vector<Node>>(ModelsLib::kNodeArray)[0].child_start == 1);
  CHECK(single[2]->Get<std::vector<float>>(ModelsLib::kProbArray).size() == 6);
  // votes of split predictions add up (AggregateResults); the accuracy rule
  // takes the first class of the largest count, strictly greater than 0
  // (ml_resultdata_impl.cc:17-71), so ties and all-zero rows go to class 0
  auto r1 = DataLib::GetInstance().CreateResultData<float>();
  auto r2 = DataLib::GetInstance().CreateResultData<float>();
  r1->AddPredictions({{1, 1}, {0, 2}, {3, 1}, {0, 0}});
  r2->AddPredictions({{0, 0}, {0, 1}, {0, 0}, {0, 0}});
  auto sum = rf->AggregateResults({r1, r2});
  const std::vector<std::vector<float>> want_votes = {{1, 1}, {0, 3}, {3, 1}, {0, 0}};
  CHECK(sum->GetPredictions() == want_votes);
  const float acc = sum->GetAccuracy({0, 1, 1, 0});
  CHECK(std::abs(acc - 0.75f) < 1e-6f);
  std::cout << "host ok\n";
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::string mode = argv[1];
  if (mode == "host") return host_checks();
  if (argc < 4) return 2;
  auto& parser = ParsingLib::GetInstance();
  if (mode == "parse") {
    try {
      auto df = parser.ParseFile<float>(lib_parsing::ParsingInterface::kCsv, argv[2]);
      std::ofstream f(argv[3], std::ios::binary);
      int32_t hdr[3] = {df->GetNrSamples(), df->GetNrFeatures(), df->GetNrTargets()};
      f.write((const char*)hdr, sizeof(hdr));
      dump(f, df->GetSamples());
      dump(f, df->GetTargets());
    } catch (std::exception& e) {
      std::cerr << "parse failed: " << e.what() << "\n";
      return 3;
    }
    return 0;
  }
  if (mode != "fit") return 2;
  // data.bin: int32 N, F, C; float X[F*N] (feature-major); float y[N]
  std::ifstream in(argv[2], std::ios::binary);
  int32_t N, F, C;
  in.read((char*)&N, 4);
  in.read((char*)&F, 4);
  in.read((char*)&C, 4);
  std::vector<float> X((size_t)N * F), y(N);
  in.read((char*)X.data(), 4 * X.size());
  in.read((char*)y.data(), 4 * y.size());
  std::string dir = argv[3];

  auto& ens = EnsemblesLib::GetInstance();
  auto df = DataLib::GetInstance().CreateDataFrame<float>();
  df->AddSampleData(X);
  df->AddTargetData(y);
  df->AddFeatureMap(std::vector<std::map<std::string, float>>(F));
  std::map<std::string, float> tmap;
  for (int c = 0; c < C; ++c) tmap[std::to_string(c)] = (float)c;
  df->AddTargetMap(tmap);

  auto rf = ens.CreateGpuRfAlgorithm<float>();
  auto params = ens.CreateGpuRfParamPack();
  params->Set(EnsemblesLib::kNrTrees, 12);
  params->Set(EnsemblesLib::kAlgoType, AlgorithmsLib::kClassification);
  params->Set(EnsemblesLib::kNrFeatures, 5);
  params->Set(EnsemblesLib::kMaxDepth, 14);
  params->Set(EnsemblesLib::kMinNodeSize, 5);
  params->Set(EnsemblesLib::kMinLeaf, 2);
  params->Set(EnsemblesLib::kSeed, 3);
  auto model = rf->Fit(df, params);
  CHECK(model->Get<int>(ModelsLib::kNrTrees) == 12);
  auto res = rf->Predict(df, model, params);
  float acc = res->GetAccuracy(df->GetTargets());
  std::cout << "accuracy " << acc << "\n";
  {
    std::ofstream f(dir + "/model.bin", std::ios::binary);
    dump(f, raw_nodes(model));
    dump(f, model->Get<std::vector<float>>(ModelsLib::kProbArray));
    dump(f, votes(res));
  }
  // the same forest fitted as three parts (tree offsets carried), aggregated
  auto packs = rf->SplitParameterPack(params, 3);
  std::vector<sp<lib_models::MlModel>> parts;
  for (auto& p : packs) parts.push_back(rf->Fit(df, p));
  auto agg = rf->AggregateModels(parts);
  CHECK(agg->Get<int>(ModelsLib::kNrTrees) == 12);
  CHECK(votes(rf->Predict(df, agg, params)) == votes(res));
  // split a model, predict the parts, sum the votes
  auto split = rf->SplitModel(model, 5);
  std::vector<sp<lib_data::MlResultData<float>>> rs;
  for (auto& m : split) rs.push_back(rf->Predict(df, m, params));
  CHECK(votes(rf->AggregateResults(rs)) == votes(res));
  // double frames whose values are floats give the same forest
  auto dfd = DataLib::GetInstance().CreateDataFrame<double>();
  dfd->AddSampleData(std::vector<double>(X.begin(), X.end()));
  dfd->AddTargetData(std::vector<double>(y.begin(), y.end()));
  dfd->AddFeatureMap(std::vector<std::map<std::string, double>>(F));
  std::map<std::string, double> tmapd;
  for (int c = 0; c < C; ++c) tmapd[std::to_string(c)] = (double)c;
  dfd->AddTargetMap(tmapd);
  auto rfd = ens.CreateGpuRfAlgorithm<double>();
  auto md = rfd->Fit(dfd, params);
  CHECK(votes(rfd->Predict(dfd, md, params)) == votes(res));
  // ERT with the reference's default pack (K = round(ln F) + 1, 100 trees)
  auto ert = ens.CreateGpuErtAlgorithm<float>();
  auto ep = ens.CreateGpuErtParamPack();
  auto me = ert->Fit(df, ep);
  CHECK(me->Get<int>(ModelsLib::kNrTrees) == 100);
  auto re = ert->Predict(df, me, ep);
  {
    std::ofstream f(dir + "/ert.bin", std::ios::binary);
    dump(f, raw_nodes(me));
    dump(f, me->Get<std::vector<float>>(ModelsLib::kProbArray));
    dump(f, votes(re));
  }
  // errors surface as the reference's exception type
  bool threw = false;
  try {
    auto bad = ens.CreateGpuRfParamPack();
    bad->Set(EnsemblesLib::kNrTrees, 0);
    rf->Fit(df, bad);
  } catch (lib_core::template_exception& e) {
    threw = std::string(e.what()).find("Fit") != std::string::npos;
  }
  CHECK(threw);
  std::cout << "shim ok\n";
  return 0;
}
