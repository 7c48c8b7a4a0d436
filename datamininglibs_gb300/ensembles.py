"""ctypes binding of the engine's C ABI (include/dml.h), mirroring the
reference's lib_ensembles surface for the fit/predict path:

* ``fit(..., algo=ALGO_RF|ALGO_ERT)`` = ``EnsemblesInterface::CreateGpuRfAlgorithm
  / CreateGpuErtAlgorithm`` + ``MlAlgorithm<T>::Fit`` with the DteParams
  (lib_ensembles/include/ensembles_interface.h:23-38);
* ``Forest.predict`` = ``MlAlgorithm<T>::Predict``, returning the vote matrix that
  ``MlResultData::AddPredictions`` holds (lib_data/source/ml_resultdata_impl.cc:17-21);
* ``Forest.export`` = the model slots kNodeArray / kProbArray
  (lib_models/include/models_interface.h:9-19);
* ``accuracy`` = ``MlResultData::GetAccuracy`` (ml_resultdata_impl.cc:23-38).
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdml_gb300.so")

ALGO_RF, ALGO_ERT = 0, 1
CLASSIFICATION, REGRESSION = 0, 1
HOST, DEVICE = 0, 1

STATUS = {0: "DML_OK", 1: "DML_ERR_INVALID_ARG", 2: "DML_ERR_OOM", 3: "DML_ERR_CUDA",
          4: "DML_ERR_TIMEOUT", 5: "DML_ERR_BUDGET", 6: "DML_ERR_NOT_READY",
          7: "DML_ERR_INTERNAL"}


class DmlError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class FitDesc(ctypes.Structure):
    _fields_ = [("algo", ctypes.c_int32), ("task", ctypes.c_int32),
                ("n_trees", ctypes.c_int32), ("n_features_try", ctypes.c_int32),
                ("max_depth", ctypes.c_int32), ("min_node_size", ctypes.c_int32),
                ("min_leaf", ctypes.c_int32), ("n_classes", ctypes.c_int32),
                ("seed", ctypes.c_uint64), ("n_rows", ctypes.c_int64),
                ("n_features", ctypes.c_int32), ("memory", ctypes.c_int32),
                ("samples", ctypes.c_void_p), ("targets", ctypes.c_void_p),
                ("tree_offset", ctypes.c_int32), ("balanced", ctypes.c_int32)]


class Tuning(ctypes.Structure):
    _fields_ = [("warp_max", ctypes.c_int32), ("smem_cap", ctypes.c_int32),
                ("big_ctas_per_sm", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class OobStats(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_int64), ("pairs_correct", ctypes.c_int64),
                ("pairs_sq_err", ctypes.c_double), ("rows", ctypes.c_int64),
                ("rows_correct", ctypes.c_int64), ("rows_sq_err", ctypes.c_double)]


class ForestInfo(ctypes.Structure):
    _fields_ = [("task", ctypes.c_int32), ("n_trees", ctypes.c_int32),
                ("n_classes", ctypes.c_int32), ("n_features", ctypes.c_int32),
                ("n_nodes", ctypes.c_int64), ("n_probs", ctypes.c_int64),
                ("max_depth", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("fit_ms", ctypes.c_double)]


NUM_QUEUES = 11
# kernel that searches each node class (DML_Q_* in include/dml.h)
QUEUE_KERNELS = ["k_group_nodes<32>", "k_ert_cta", "k_rf_smem", "k_rf_big_items+k_rf_big_decide",
                 "k_warp_rf<2>", "k_warp_rf<4>", "k_warp_rf<8>", "k_group_nodes<16>",
                 "k_group_nodes<8>", "k_warp_rf<16>", "k_ert_warp<8>"]


class FitStats(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_int64), ("entries", ctypes.c_int64),
                ("weighted_rows", ctypes.c_int64), ("entry_tries", ctypes.c_int64),
                ("levels", ctypes.c_int32),
                ("launches", ctypes.c_int32), ("level_loop_ms", ctypes.c_double),
                ("search_ms", ctypes.c_double),
                ("queue_ms", ctypes.c_double * NUM_QUEUES),
                ("queue_entries", ctypes.c_int64 * NUM_QUEUES),
                ("queue_entry_tries", ctypes.c_int64 * NUM_QUEUES),
                ("queue_launches", ctypes.c_int32 * NUM_QUEUES), ("reserved", ctypes.c_int32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("max_batch_rows", ctypes.c_int32),
                ("n_streams", ctypes.c_int32), ("max_wait_us", ctypes.c_int32),
                ("small_rows", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_int64), ("rows", ctypes.c_int64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("mean_ms", ctypes.c_double), ("rows_per_s", ctypes.c_double),
                ("launches", ctypes.c_int64), ("rejected", ctypes.c_int64)]


_LIB = None

# every entry point of include/dml.h with its ctypes signature
_SIGS = {
    "dml_fit": (ctypes.c_int, [ctypes.POINTER(FitDesc), ctypes.POINTER(ctypes.c_void_p),
                               ctypes.c_void_p]),
    "dml_fit_batched": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(FitDesc),
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]),
    "dml_fit_plain": (ctypes.c_int, [ctypes.POINTER(FitDesc), ctypes.POINTER(ctypes.c_void_p),
                                     ctypes.c_void_p]),
    "dml_last_fit_stats": (ctypes.c_int, [ctypes.POINTER(FitStats)]),
    "dml_autotune": (ctypes.c_int, [ctypes.POINTER(FitDesc), ctypes.c_int32,
                                    ctypes.POINTER(Tuning), ctypes.c_void_p]),
    "dml_tuning_get": (ctypes.c_int, [ctypes.POINTER(FitDesc), ctypes.POINTER(Tuning)]),
    "dml_oob_estimate": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FitDesc), ctypes.c_int32,
                                        ctypes.POINTER(OobStats), ctypes.c_void_p]),
    "dml_fit_noalloc": (ctypes.c_int, [ctypes.POINTER(FitDesc), ctypes.c_void_p, ctypes.c_int64,
                                       ctypes.c_void_p, ctypes.c_int64,
                                       ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p]),
    "dml_predict": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                   ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "dml_predict_plain": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                         ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "dml_forest_info_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ForestInfo)]),
    "dml_forest_export": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "dml_forest_gains": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                        ctypes.c_void_p]),
    "dml_forest_import": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64,
                                         ctypes.c_void_p, ctypes.c_int64,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "dml_forest_free": (None, [ctypes.c_void_p]),
    "dml_forest_save": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "dml_forest_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    "dml_device_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int32)]),
    "dml_set_device": (ctypes.c_int, [ctypes.c_int32]),
    "dml_last_error": (ctypes.c_char_p, []),
    "dml_server_create": (ctypes.c_int, [ctypes.POINTER(ServerConfig),
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "dml_server_add_forest": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_int32)]),
    "dml_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                         ctypes.c_int64, ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_int64)]),
    "dml_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64,
                                       ctypes.POINTER(ctypes.c_double)]),
    "dml_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64,
                                       ctypes.POINTER(ctypes.c_double)]),
    "dml_server_stats_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ServerStats)]),
    "dml_server_destroy": (None, [ctypes.c_void_p]),
}


def lib():
    """The loaded engine library; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libdml_gb300.so is not built (run __graft_entry__.build() or "
                              "python datamininglibs_gb300/build.py)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def _check(status):
    if status != 0:
        msg = lib().dml_last_error()
        raise DmlError(status, msg.decode() if msg else "")


def _ptr(a):
    """(pointer, memory kind) of a numpy array or a CUDA torch tensor."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data, HOST
    if hasattr(a, "data_ptr"):
        return a.data_ptr(), DEVICE if a.is_cuda else HOST
    raise TypeError("expected a numpy array or a torch tensor")


def _stream(stream):
    if stream is None:
        return None
    return getattr(stream, "cuda_stream", stream)


class Forest:
    """A device-resident fitted forest (opaque ``dml_forest*``)."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)

    @property
    def handle(self):
        return self._h

    def info(self):
        i = ForestInfo()
        _check(lib().dml_forest_info_get(self._h, ctypes.byref(i)))
        return i

    def export(self, nodes=None, probs=None):
        """(nodes int32 [n, 5] in the Classify layout, probs float32), written
        into the given host arrays when passed (e.g. pinned buffers reused
        across fits; their shapes must match the forest's)."""
        i = self.info()
        if nodes is None:
            nodes = np.zeros((i.n_nodes, 5), np.int32)
        if probs is None:
            probs = np.zeros(i.n_probs, np.float32)
        if (nodes.shape != (i.n_nodes, 5) or nodes.dtype != np.int32 or probs.shape != (i.n_probs,)
                or probs.dtype != np.float32 or not nodes.flags.c_contiguous
                or not probs.flags.c_contiguous):
            raise ValueError("export buffers must be int32 [%d, 5] and float32 [%d], contiguous"
                             % (i.n_nodes, i.n_probs))
        _check(lib().dml_forest_export(self._h, nodes.ctypes.data, probs.ctypes.data))
        return nodes, probs

    def gains(self):
        """float32 [n_nodes]: the FP32 gain of every node's chosen split as the
        engine computed it on the device (NaN for leaves), in node-array order."""
        i = self.info()
        g = np.zeros(i.n_nodes, np.float32)
        _check(lib().dml_forest_gains(self._h, g.ctypes.data, HOST, None))
        return g

    def predict(self, X, out=None, stream=None):
        """X feature-major [F, N] (numpy or CUDA tensor).  Returns the
        [N, C] vote counts (classification) or [N, 1] sums (regression)."""
        return self._predict(lib().dml_predict, X, out, stream)

    def predict_plain(self, X, out=None, stream=None):
        """The same votes through the reference's launch structure
        (dml_predict_plain): the baseline of the serving speed-up."""
        return self._predict(lib().dml_predict_plain, X, out, stream)

    def _predict(self, fn, X, out, stream):
        i = self.info()
        width = i.n_classes if i.task == CLASSIFICATION else 1
        n = X.shape[1]
        xp, mem = _ptr(X)
        if out is None:
            if mem == HOST:
                out = np.zeros((n, width), np.float32)
            else:
                import torch
                out = torch.empty((n, width), dtype=torch.float32, device=X.device)
        op, omem = _ptr(out)
        if omem != mem:
            raise ValueError("X and out must both be host or both device memory")
        _check(fn(self._h, xp, n, op, mem, _stream(stream)))
        return out

    def save(self, path):
        """dml_forest_save: the forest as a file (reference node layout + hash)."""
        _check(lib().dml_forest_save(self._h, os.fsencode(path)))

    @staticmethod
    def load(path):
        """dml_forest_load: a device-resident forest from a dml_forest_save file."""
        h = ctypes.c_void_p()
        _check(lib().dml_forest_load(os.fsencode(path), ctypes.byref(h)))
        return Forest(h.value)

    def free(self):
        if self._h and self._h.value:
            lib().dml_forest_free(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @staticmethod
    def from_model(nodes, probs, *, task, n_trees, n_classes, n_features):
        nodes = np.ascontiguousarray(nodes, np.int32)
        probs = np.ascontiguousarray(probs, np.float32)
        h = ctypes.c_void_p()
        _check(lib().dml_forest_import(task, n_trees, n_classes, n_features, nodes.ctypes.data,
                                       nodes.shape[0], probs.ctypes.data, probs.size,
                                       ctypes.byref(h)))
        return Forest(h.value)


def _desc(X, y, algo, task, n_trees, K, max_depth, min_node_size, min_leaf, n_classes, seed,
          tree_offset=0, balanced=0):
    xp, mem = _ptr(X)
    yp, ymem = _ptr(y)
    if mem != ymem:
        raise ValueError("samples and targets must both be host or both device memory")
    F, N = X.shape
    return FitDesc(algo, task, n_trees, K, max_depth, min_node_size, min_leaf,
                   n_classes if task == CLASSIFICATION else 1, seed, N, F, mem, xp, yp,
                   tree_offset, balanced)


def fit(X, y, *, algo, task=CLASSIFICATION, n_trees=100, K=0, max_depth=1000,
        min_node_size=5, min_leaf=1, n_classes=2, seed=0, tree_offset=0, balanced=0,
        stream=None):
    """Defaults are the reference's param pack (ensembles_interface.cc:28-58);
    balanced=1 is kEasyEnsemble (RF classification)."""
    d = _desc(X, y, algo, task, n_trees, K, max_depth, min_node_size, min_leaf, n_classes, seed,
              tree_offset, balanced)
    h = ctypes.c_void_p()
    _check(lib().dml_fit(ctypes.byref(d), ctypes.byref(h), _stream(stream)))
    return Forest(h.value)


def fit_plain(X, y, *, algo, task=CLASSIFICATION, n_trees=100, K=0, max_depth=1000,
              min_node_size=5, min_leaf=1, n_classes=2, seed=0, stream=None):
    d = _desc(X, y, algo, task, n_trees, K, max_depth, min_node_size, min_leaf, n_classes, seed)
    h = ctypes.c_void_p()
    _check(lib().dml_fit_plain(ctypes.byref(d), ctypes.byref(h), _stream(stream)))
    return Forest(h.value)


def fit_noalloc(X, y, nodes_out, probs_out, *, algo, task=CLASSIFICATION, n_trees=100, K=0,
                max_depth=1000, min_node_size=5, min_leaf=1, n_classes=2, seed=0, stream=None):
    """dml_fit_noalloc: X, y and the two output buffers are CUDA tensors; the
    fit allocates no device memory.  Returns (n_nodes, n_probs) written."""
    d = _desc(X, y, algo, task, n_trees, K, max_depth, min_node_size, min_leaf, n_classes, seed)
    nn, npb = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().dml_fit_noalloc(ctypes.byref(d), nodes_out.data_ptr(), nodes_out.shape[0],
                                 probs_out.data_ptr(), probs_out.numel(), ctypes.byref(nn),
                                 ctypes.byref(npb), _stream(stream)))
    return nn.value, npb.value


def fit_batched(problems, stream=None):
    """problems: list of dicts with the keyword arguments of fit() plus X, y."""
    descs = (FitDesc * len(problems))()
    keep = []
    for i, p in enumerate(problems):
        p = dict(p)
        X, y = p.pop("X"), p.pop("y")
        keep.append((X, y))
        kw = dict(task=CLASSIFICATION, n_trees=100, K=0, max_depth=1000, min_node_size=5,
                  min_leaf=1, n_classes=2, seed=0)
        kw.update(p)
        descs[i] = _desc(X, y, kw["algo"], kw["task"], kw["n_trees"], kw["K"], kw["max_depth"],
                         kw["min_node_size"], kw["min_leaf"], kw["n_classes"], kw["seed"])
    out = (ctypes.c_void_p * len(problems))()
    _check(lib().dml_fit_batched(len(problems), descs, out, _stream(stream)))
    return [Forest(out[i]) for i in range(len(problems))]


def autotune(X, y, *, algo, task=CLASSIFICATION, n_trees=100, K=0, max_depth=1000,
             min_node_size=5, min_leaf=1, n_classes=2, seed=0, sample_trees=8, stream=None):
    """dml_autotune: times the scheduling candidates on the first sample_trees
    trees of this problem and keeps the fastest for problems of its shape."""
    d = _desc(X, y, algo, task, n_trees, K, max_depth, min_node_size, min_leaf, n_classes, seed)
    t = Tuning()
    _check(lib().dml_autotune(ctypes.byref(d), sample_trees, ctypes.byref(t), _stream(stream)))
    return {"warp_max": t.warp_max, "smem_cap": t.smem_cap, "big_ctas_per_sm": t.big_ctas_per_sm}


def tuning_for(X, y, *, algo, task=CLASSIFICATION, n_trees=100, K=0, max_depth=1000,
               min_node_size=5, min_leaf=1, n_classes=2, seed=0):
    """dml_tuning_get: the scheduling a fit of this problem would use."""
    d = _desc(X, y, algo, task, n_trees, K, max_depth, min_node_size, min_leaf, n_classes, seed)
    t = Tuning()
    _check(lib().dml_tuning_get(ctypes.byref(d), ctypes.byref(t)))
    return {"warp_max": t.warp_max, "smem_cap": t.smem_cap, "big_ctas_per_sm": t.big_ctas_per_sm}


def oob_estimate(forest, X, y, *, seed=0, tree_offset=0, balanced=0, permuted_feature=-1,
                 stream=None):
    """dml_oob_estimate: out-of-bag sums of an RF forest fitted on (X, y) with
    this seed (the bags are drawn again); with permuted_feature >= 0 the
    permutation run of that feature."""
    i = forest.info()
    d = _desc(X, y, ALGO_RF, i.task, i.n_trees, 0, 0, 0, 1, i.n_classes, seed, tree_offset,
              balanced)
    st = OobStats()
    _check(lib().dml_oob_estimate(forest.handle, ctypes.byref(d), permuted_feature,
                                  ctypes.byref(st), _stream(stream)))
    return st


def feature_importance(forest, X, y, features=None, **kw):
    """Permutation importance per feature: the drop in out-of-bag pair
    accuracy (classification) or the rise in out-of-bag pair MSE (regression)
    when the feature's values come from random rows."""
    base = oob_estimate(forest, X, y, **kw)
    feats = range(X.shape[0]) if features is None else features
    out = []
    for f in feats:
        p = oob_estimate(forest, X, y, permuted_feature=int(f), **kw)
        if forest.info().task == CLASSIFICATION:
            out.append((base.pairs_correct - p.pairs_correct) / max(1, base.pairs))
        else:
            out.append((p.pairs_sq_err - base.pairs_sq_err) / max(1, base.pairs))
    return np.array(out)


def last_fit_stats():
    s = FitStats()
    _check(lib().dml_last_fit_stats(ctypes.byref(s)))
    return s


def accuracy(votes, targets):
    """MlResultData::GetAccuracy: argmax with strict '>' starting from 0 (ties
    and all-zero rows go to the lowest class), counted when |class - target|
    < 0.001, divided by the row count, all in float32."""
    votes = np.asarray(votes, np.float32)
    targets = np.asarray(targets, np.float32)
    acc = np.float32(0.0)
    for i in range(len(targets)):
        high = np.float32(0.0)
        cls = np.float32(0.0)
        for j in range(votes.shape[1]):
            if votes[i, j] > high:
                high = votes[i, j]
                cls = np.float32(j)
        if abs(cls - targets[i]) < 0.001:
            acc = np.float32(acc + np.float32(1.0))
    return np.float32(acc / np.float32(len(targets)))


class Server:
    """Resident-forest prediction server with continuous batching (dml_server_*)."""

    def __init__(self, hbm_budget_bytes=8 << 30, max_batch_rows=1 << 16, n_streams=4,
                 max_wait_us=100, small_rows=4096):
        cfg = ServerConfig(hbm_budget_bytes, max_batch_rows, n_streams, max_wait_us, small_rows)
        h = ctypes.c_void_p()
        _check(lib().dml_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._keep = {}
        self._inflight = {}  # request id -> (samples, out): alive until the request is done

    def add_forest(self, forest):
        fid = ctypes.c_int32()
        _check(lib().dml_server_add_forest(self._h, forest.handle, ctypes.byref(fid)))
        self._keep[fid.value] = forest
        return fid.value

    def submit(self, forest_id, X, out):
        """Queues X (feature-major [F, n], host) for prediction into out ([n, width],
        host).  The server reads X and writes out after submit returns; both
        are kept referenced here until poll or wait reports the request done."""
        rid = ctypes.c_int64()
        _check(lib().dml_server_submit(self._h, forest_id, X.ctypes.data, X.shape[1],
                                       out.ctypes.data, ctypes.byref(rid)))
        self._inflight[rid.value] = (X, out)
        return rid.value

    def poll(self, rid):
        lat = ctypes.c_double()
        st = lib().dml_server_poll(self._h, rid, ctypes.byref(lat))
        if st == 6:
            return None
        self._inflight.pop(rid, None)
        _check(st)
        return lat.value

    def wait(self, rid):
        lat = ctypes.c_double()
        st = lib().dml_server_wait(self._h, rid, ctypes.byref(lat))
        if st != 4:  # a timed-out request may still be read and written
            self._inflight.pop(rid, None)
        _check(st)
        return lat.value

    def stats(self):
        s = ServerStats()
        _check(lib().dml_server_stats_get(self._h, ctypes.byref(s)))
        return s

    def close(self):
        if self._h and self._h.value:
            lib().dml_server_destroy(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
