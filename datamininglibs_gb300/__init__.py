"""GB300 random-forest / extremely-randomized-trees engine (drop-in for the
fit/predict path of novelari/DataminingLibs' lib_ensembles).

The engine is the C ABI in include/dml.h, implemented by the CUDA library
``libdml_gb300.so`` built in this directory (``datamininglibs_gb300.build``).
This package binds it with ctypes.  There is no CPU fallback: loading fails
loudly when the library is missing.
"""
from .ensembles import (  # noqa: F401
    DmlError, Forest, FitStats, OobStats, Server, accuracy, autotune, feature_importance, fit,
    fit_batched, fit_plain, lib, oob_estimate, tuning_for, ALGO_RF, ALGO_ERT, CLASSIFICATION, REGRESSION,
)
