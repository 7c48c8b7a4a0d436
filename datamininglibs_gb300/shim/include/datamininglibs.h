// C++ drop-in for the fit/predict path of novelari/DataminingLibs.
//
// Source-compatible with the reference's public surface for that path
// (source_shared/include/datamininglibs.h): the same namespaces, class names,
// factories, parameter ids and model slots, implemented over the C ABI of
// include/dml.h (the CUDA engine).  A program written against the reference's
//   lib_ensembles/include/ensembles_interface.h   EnsemblesInterface
//   lib_algorithms/include/ml_algorithm.h          MlAlgorithm<T>
//   lib_algorithms/include/ml_algorithm_params.h   MlAlgorithmParams
//   lib_algorithms/include/algorithms_interface.h  AlgorithmsInterface
//   lib_data/include/{data_interface,ml_dataframe,ml_resultdata}.h
//   lib_models/include/{models_interface,ml_model}.h
//   lib_parsing/include/parsing_interface.h        ParsingInterface (CSV)
//   lib_core/include/core_interface.h              CoreInterface::ThrowException
//   lib_ensembles/source/gpudte_algorithm_shared.h gpuDTE_NodeHeader_Classify<T>
// compiles against this header and links libdml_gb300_shim.so.
#pragma once
#include <cstdint>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

template <typename T>
using sp = std::shared_ptr<T>;
template <typename T>
using col_array = std::vector<T>;
template <typename T1, typename T2>
using col_map = std::map<T1, T2>;
using string = std::string;

namespace sutil {
// Type-erased value of a parameter or model slot; get_value<T> must name the
// stored type (as any_type.hpp:10-13 requires).
struct any_type {
  template <typename T>
  explicit any_type(T t) : ptr(std::make_shared<impl<T>>(t)) {}
  any_type() = default;
  template <typename T>
  T& get_value() {
    return static_cast<impl<T>*>(ptr.get())->val;
  }
  bool empty() const { return !ptr; }

 private:
  struct placeholder {
    virtual ~placeholder() = default;
  };
  template <typename T>
  struct impl : placeholder {
    explicit impl(T t) : val(std::move(t)) {}
    T val;
  };
  std::shared_ptr<placeholder> ptr;
};
}  // namespace sutil

namespace lib_core {
// The reference's exception type and thrower (core_interface.cc:7-33).
class template_exception : public std::exception {
 public:
  explicit template_exception(string desc) : description_(std::move(desc)) {}
  const char* what() const noexcept override { return description_.c_str(); }

 private:
  string description_;
};

class CoreInterface {
 public:
  static CoreInterface& GetInstance();
  [[noreturn]] void ThrowException(string msg);
  void DebugMessage(string msg);
};
}  // namespace lib_core
using CoreLib = lib_core::CoreInterface;

namespace lib_data {
template <typename T>
class MlDataFrame {
 public:
  virtual ~MlDataFrame() = default;
  virtual void AddTargetData(col_array<T> targets) = 0;
  virtual void AddSampleData(col_array<T> samples) = 0;
  virtual void AddFeatureMap(col_array<col_map<string, T>> col_map) = 0;
  virtual void AddTargetMap(col_map<string, T> col_map) = 0;
  virtual int GetNrSamples() = 0;
  virtual int GetNrFeatures() = 0;
  virtual int GetNrTargets() = 0;
  virtual const col_array<T>& GetTargets() = 0;
  virtual const col_array<T>& GetSamples() = 0;
};

template <typename T>
class MlResultData {
 public:
  virtual ~MlResultData() = default;
  virtual void AddSingleValue(string name, T value) = 0;
  virtual void AddMultipleValue(string name, col_array<T> vals) = 0;
  virtual void AddPredictions(col_array<col_array<T>> predictions) = 0;
  virtual T GetAccuracy(const col_array<T>& targets) = 0;
  virtual T GetSingleValue(string name) = 0;
  virtual col_array<T>& GetMultipleValue(string name) = 0;
  virtual string ToString() = 0;
  virtual MlResultData<T>& operator+=(const MlResultData<T>& rhs) = 0;
  virtual const col_array<col_array<T>>& GetPredictions() const = 0;
};

class DataInterface {
 public:
  static DataInterface& GetInstance();
  template <typename T>
  sp<MlDataFrame<T>> CreateDataFrame();
  template <typename T>
  sp<MlResultData<T>> CreateResultData();
};
}  // namespace lib_data
using DataLib = lib_data::DataInterface;

namespace lib_models {
class MlModel {
 public:
  virtual ~MlModel() = default;
  template <typename T>
  void Add(const int id, const T& data) {
    AddData(id, sutil::any_type(data));
  }
  template <typename T>
  T& Get(const int id) {
    return GetData(id).get_value<T>();
  }
  // Addition (not in the reference): whether slot `id` holds a value.  Models
  // of this library override it.  A model class written against the
  // reference's interface (AddData / GetData only) keeps this default, which
  // reads the reference's own slots (below kReferenceSlotEnd) through GetData
  // and reports the slots past them as empty.
  virtual bool Has(const int id) {
    return id >= 0 && id < kReferenceSlotEnd && !GetData(id).empty();
  }
  static constexpr int kReferenceSlotEnd = 6;  // ModelsInterface::kGpuDteModelEndMarker

 private:
  virtual void AddData(const int id, sutil::any_type data) = 0;
  virtual sutil::any_type& GetData(const int id) = 0;
};

class ModelsInterface {
 public:
  static ModelsInterface& GetInstance();
  sp<MlModel> CreateModel();
  enum GpuDteModel {
    kNrTrees,
    kNrTargets,
    kNrFeatures,
    kModelType,
    kNodeArray,
    kProbArray,
    kGpuDteModelEndMarker
  };
};
}  // namespace lib_models
using ModelsLib = lib_models::ModelsInterface;

namespace lib_algorithms {
class MlAlgorithmParams {
 public:
  virtual ~MlAlgorithmParams() = default;
  template <typename T>
  void Set(int param, T value) {
    SetParam(param, sutil::any_type(value));
  }
  template <typename T>
  const T& Get(const int param) {
    return GetParam(param).get_value<T>();
  }
  // Additions (not in the reference): whether `param` holds a value, and a
  // copy of the pack.  Packs of this library override both.  A pack class
  // written against the reference's interface (SetParam / GetParam only) keeps
  // these defaults: Has reads the reference's own ids (below kReferenceParamEnd)
  // through GetParam and reports the ids past them as unset, and Clone returns
  // null, for which SplitParameterPack copies the reference's ids into packs of
  // its own.
  virtual bool Has(const int param) {
    return param >= 0 && param < kReferenceParamEnd && !GetParam(param).empty();
  }
  virtual sp<MlAlgorithmParams> Clone() { return nullptr; }
  static constexpr int kReferenceParamEnd = 8;  // EnsemblesInterface::kDteEndMarker

 private:
  virtual void SetParam(const int param, const sutil::any_type value) = 0;
  virtual sutil::any_type& GetParam(const int param) = 0;
};

template <typename T>
class MlAlgorithm {
 public:
  virtual ~MlAlgorithm() = default;
  virtual sp<lib_models::MlModel> Fit(sp<lib_data::MlDataFrame<T>> data,
                                      sp<MlAlgorithmParams> params) = 0;
  virtual sp<lib_data::MlResultData<T>> Predict(sp<lib_data::MlDataFrame<T>> data,
                                                sp<lib_models::MlModel> model,
                                                sp<MlAlgorithmParams> params) = 0;
  virtual sp<lib_models::MlModel> AggregateModels(col_array<sp<lib_models::MlModel>> models) = 0;
  virtual col_array<sp<lib_models::MlModel>> SplitModel(sp<lib_models::MlModel> model,
                                                        const int parts) = 0;
  virtual sp<lib_data::MlResultData<T>> AggregateResults(
      col_array<sp<lib_data::MlResultData<T>>> results) = 0;
  virtual col_array<sp<MlAlgorithmParams>> SplitParameterPack(sp<MlAlgorithmParams> params,
                                                              const int parts) = 0;
};

class AlgorithmsInterface {
 public:
  static AlgorithmsInterface& GetInstance();
  enum AlgorithmType { kClassification = 0, kRegression };
  sp<MlAlgorithmParams> CreateAlgorithmParams(int size);
  // algorithms_interface.h:16 / algorithms_interface.cc:18-26: wraps a
  // single-device algorithm into the multi-device one (trees split over the
  // visible GPUs, one host thread each; models and votes aggregated).  T is
  // float or double.
  template <typename T>
  sp<MlAlgorithm<T>> CreateGpuAlgorithm(sp<MlAlgorithm<T>> algo);
};
}  // namespace lib_algorithms
using AlgorithmsLib = lib_algorithms::AlgorithmsInterface;

namespace lib_ensembles {
// gpudte_algorithm_shared.h:82-90: the node layout of the kNodeArray slot.
struct GpuDteAlgorithmShared {
  template <typename T>
  struct gpuDTE_NodeHeader_Classify {
    int child_start;
    int child_count;
    int probability_start;
    int attribute;
    T split_point;
  };
};

class EnsemblesInterface {
 public:
  static EnsemblesInterface& GetInstance();
  template <typename T>
  sp<lib_algorithms::MlAlgorithm<T>> CreateGpuRfAlgorithm();
  template <typename T>
  sp<lib_algorithms::MlAlgorithm<T>> CreateGpuErtAlgorithm();
  sp<lib_algorithms::MlAlgorithmParams> CreateGpuRfParamPack();
  sp<lib_algorithms::MlAlgorithmParams> CreateGpuErtParamPack();
  enum CommonParams { kDevId = 0, kCommonEndMarker };
  enum DteParams {
    kNrTrees = kCommonEndMarker,
    kAlgoType,
    kNrFeatures,
    kMaxDepth,
    kMinNodeSize,
    kEasyEnsemble,
    kBagging,
    kDteEndMarker,
    // additions past the reference's ids
    kMinLeaf = kDteEndMarker,  // int, >= 1
    kSeed,                     // int
    kTreeOffset,               // int: RNG key of the first tree of a part
    kGb300EndMarker
  };
};
}  // namespace lib_ensembles
using EnsemblesLib = lib_ensembles::EnsemblesInterface;
static_assert(lib_algorithms::MlAlgorithmParams::kReferenceParamEnd ==
                  (int)lib_ensembles::EnsemblesInterface::kDteEndMarker,
              "reference parameter ids end at kDteEndMarker");
static_assert(lib_models::MlModel::kReferenceSlotEnd ==
                  (int)lib_models::ModelsInterface::kGpuDteModelEndMarker,
              "reference model slots end at kGpuDteModelEndMarker");

namespace lib_parsing {
template <typename T>
class MlParser {
 public:
  virtual ~MlParser() = default;
  virtual bool Parse(sp<lib_data::MlDataFrame<T>> data, string filepath) = 0;
  virtual bool Parse(sp<lib_data::MlDataFrame<T>> data, col_array<char>& raw_data) = 0;
};

class ParsingInterface {
 public:
  static ParsingInterface& GetInstance();
  enum ParserType { kCsv, kArff, kRds };
  template <typename T>
  sp<lib_data::MlDataFrame<T>> ParseData(ParserType type, col_array<char>& raw_data);
  template <typename T>
  sp<lib_data::MlDataFrame<T>> ParseFile(ParserType type, string filepath);
};
}  // namespace lib_parsing
using ParsingLib = lib_parsing::ParsingInterface;
