"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle is the checker for the CUDA engine and the timed CPU baseline.  Only
tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs import this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class OracleDesc(ctypes.Structure):
    _fields_ = [
        ("algo", ctypes.c_int32), ("task", ctypes.c_int32),
        ("n_trees", ctypes.c_int32), ("K", ctypes.c_int32),
        ("max_depth", ctypes.c_int32), ("min_node_size", ctypes.c_int32),
        ("min_leaf", ctypes.c_int32), ("n_classes", ctypes.c_int32),
        ("seed", ctypes.c_uint64), ("n_rows", ctypes.c_int64),
        ("n_features", ctypes.c_int32), ("threads", ctypes.c_int32),
        ("samples", ctypes.c_void_p), ("targets", ctypes.c_void_p),
        ("tree_offset", ctypes.c_int32), ("balanced", ctypes.c_int32),
    ]


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.oracle_fit.restype = ctypes.c_void_p
        L.oracle_fit.argtypes = [ctypes.POINTER(OracleDesc)]
        L.oracle_forest_sizes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                          ctypes.POINTER(ctypes.c_int64)]
        L.oracle_forest_export.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 5
        L.oracle_forest_free.argtypes = [ctypes.c_void_p]
        L.oracle_predict.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
                                     ctypes.c_void_p, ctypes.c_int]
        L.oracle_philox.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_nlogn_table.argtypes = [ctypes.c_int64, ctypes.c_void_p]
        L.oracle_entropy_gain.restype = ctypes.c_float
        L.oracle_entropy_gain.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_double)]
        L.oracle_variance_gain.restype = ctypes.c_float
        L.oracle_variance_gain.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                           ctypes.c_int64, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_double)]
        L.oracle_split_node.restype = ctypes.c_int
        L.oracle_split_node.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_oob.argtypes = [ctypes.POINTER(OracleDesc), ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_int, ctypes.c_void_p]
        L.oracle_quant_scale.restype = ctypes.c_int
        L.oracle_quant_scale.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        _LIB = L
    return _LIB


class Model:
    """A fitted forest in the reference's Classify layout.

    ``nodes`` is int32 [n_nodes, 5] = {child_start, child_count,
    probability_start, attribute, split_point (float bits)}; ``probs`` holds C
    floats per leaf (1 for regression)."""

    def __init__(self, nodes, probs, n_trees, n_classes, task, gains32=None, gains64=None,
                 depth=None):
        self.nodes = nodes
        self.probs = probs
        self.n_trees = n_trees
        self.n_classes = n_classes
        self.task = task
        self.gains32 = gains32
        self.gains64 = gains64
        self.depth = depth

    @property
    def split_points(self):
        return self.nodes[:, 4].view(np.float32)


def fit(X, y, *, algo, task=0, n_trees, K=0, max_depth=1000, min_node_size=5, min_leaf=1,
        n_classes=2, seed=0, threads=0, tree_offset=0, balanced=0):
    """X: float32 feature-major [F, N]; y: float32 [N]."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    F, N = X.shape
    d = OracleDesc(algo, task, n_trees, K, max_depth, min_node_size, min_leaf,
                   n_classes if task == 0 else 1, seed, N, F, threads,
                   X.ctypes.data, y.ctypes.data, tree_offset, balanced)
    L = lib()
    h = L.oracle_fit(ctypes.byref(d))
    nn, npb = ctypes.c_int64(), ctypes.c_int64()
    L.oracle_forest_sizes(h, ctypes.byref(nn), ctypes.byref(npb))
    nodes = np.zeros((nn.value, 5), np.int32)
    probs = np.zeros(npb.value, np.float32)
    g32 = np.zeros(nn.value, np.float32)
    g64 = np.zeros(nn.value, np.float64)
    dep = np.zeros(nn.value, np.int32)
    L.oracle_forest_export(h, nodes.ctypes.data, probs.ctypes.data, g32.ctypes.data,
                           g64.ctypes.data, dep.ctypes.data)
    L.oracle_forest_free(h)
    return Model(nodes, probs, n_trees, n_classes if task == 0 else 1, task, g32, g64, dep)


def oob(model, X, y, *, seed=0, tree_offset=0, balanced=0, permuted_feature=-1):
    """Out-of-bag sums of an RF model fitted on (X, y) with this seed:
    [pairs, correct pairs | squared error, rows, correct rows | squared error]."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    F, N = X.shape
    d = OracleDesc(0, model.task, model.n_trees, 0, 0, 0, 1, model.n_classes, seed, N, F, 0,
                   X.ctypes.data, y.ctypes.data, tree_offset, balanced)
    nodes = np.ascontiguousarray(model.nodes, dtype=np.int32)
    probs = np.ascontiguousarray(model.probs, dtype=np.float32)
    out = np.zeros(4, np.float64)
    lib().oracle_oob(ctypes.byref(d), nodes.ctypes.data, probs.ctypes.data, permuted_feature,
                     out.ctypes.data)
    return out


def predict(model, X, threads=0):
    X = np.ascontiguousarray(X, dtype=np.float32)
    F, N = X.shape
    width = model.n_classes if model.task == 0 else 1
    out = np.zeros((N, width), np.float32)
    nodes = np.ascontiguousarray(model.nodes, dtype=np.int32)
    probs = np.ascontiguousarray(model.probs, dtype=np.float32)
    lib().oracle_predict(nodes.ctypes.data, probs.ctypes.data, model.n_trees, model.n_classes,
                         model.task, X.ctypes.data, N, out.ctypes.data, threads)
    return out


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().oracle_philox(c.ctypes.data, k.ctypes.data, o.ctypes.data)
    return o


def nlogn_table(nmax):
    """H[n] = round(n ln n * 2^28) as int64, n = 0..nmax (the gain table)."""
    out = np.zeros(nmax + 1, np.int64)
    lib().oracle_nlogn_table(nmax, out.ctypes.data)
    return out


def entropy_gain(L, R):
    L = np.ascontiguousarray(L, np.int64)
    R = np.ascontiguousarray(R, np.int64)
    g64 = ctypes.c_double()
    g = lib().oracle_entropy_gain(L.ctypes.data, R.ctypes.data, len(L), ctypes.byref(g64))
    return g, g64.value


def variance_gain(nL, SL, nR, SR, S):
    g64 = ctypes.c_double()
    g = lib().oracle_variance_gain(nL, SL, nR, SR, S, ctypes.byref(g64))
    return g, g64.value


def split_node(X, y, C, attribute, thr, rows, depth, max_depth, min_node_size):
    """The oracle's leaf rule + stable partition for one node (unit weights)."""
    rows = np.ascontiguousarray(rows, np.int32)
    xf = np.ascontiguousarray(X[attribute], np.float32)
    y = np.ascontiguousarray(y, np.float32)
    out = np.zeros(len(rows), np.int32)
    cn = np.zeros(2, np.int64)
    counts = np.zeros(C, np.int64)
    leaf = lib().oracle_split_node(rows.ctypes.data, len(rows), xf.ctypes.data, float(thr),
                                   y.ctypes.data, C, depth, max_depth, min_node_size,
                                   out.ctypes.data, cn.ctypes.data, counts.ctypes.data)
    return bool(leaf), out, cn, counts


def quant_scale(y):
    y = np.ascontiguousarray(y, np.float32)
    return lib().oracle_quant_scale(y.ctypes.data, len(y))
