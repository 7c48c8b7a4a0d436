"""ctypes wrapper of the reference pinning harness (oracle/_ref/libref.so).

The harness runs the reference's own device functions (compiled as host code)
and host-side data classes.  It exists only where the reference tree exists; it
is used to generate golden vectors (tests/golden/make_golden.py) and, when
present, to re-check the oracle directly.  Test infrastructure only.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# The one place that says where the reference tree lies: DML_REFERENCE_ROOT, or
# the checkout this project was built against.
REF_ROOT = os.environ.get("DML_REFERENCE_ROOT", "/root/reference")
_LIB = None


def available():
    return os.path.isdir(os.path.join(REF_ROOT, "lib_ensembles"))


def build():
    subprocess.run(["make", "-s", "-C", _HERE, "-f", "ref.mk", "REF=" + REF_ROOT], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_ref", "libref.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.ref_entropy_gain_f.restype = ctypes.c_float
        L.ref_entropy_gain_f.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ref_entropy_gain_d.restype = ctypes.c_double
        L.ref_entropy_gain_d.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ref_perform_split_f.restype = ctypes.c_int
        L.ref_perform_split_f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_int, ctypes.c_float] + [ctypes.c_int] * 4 + \
                                         [ctypes.c_void_p] * 5
        L.ref_predict_f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.ref_parse_csv_f.restype = ctypes.c_int
        L.ref_parse_csv_f.argtypes = [ctypes.c_char_p] + [ctypes.POINTER(ctypes.c_int)] * 3 + \
                                     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.ref_accuracy_f.restype = ctypes.c_float
        L.ref_accuracy_f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        _LIB = L
    return _LIB


def entropy_gain(L, R):
    m32 = np.ascontiguousarray(np.stack([L, R]).astype(np.float32))
    m64 = np.ascontiguousarray(np.stack([L, R]).astype(np.float64))
    C = m32.shape[1]
    return (lib().ref_entropy_gain_f(m32.ctypes.data, C),
            lib().ref_entropy_gain_d(m64.ctypes.data, C))


def perform_split(X, y, C, attribute, split_point, rows, depth, max_depth, min_node_size):
    """Classification node; rows = expanded row ids of the node."""
    X = np.ascontiguousarray(X, np.float32)
    F, N = X.shape
    rows = np.ascontiguousarray(rows, np.int32)
    x = X[attribute, rows]
    left = (x == -np.finfo(np.float32).max) | (x < np.float32(split_point))
    hist = np.zeros((2, C), np.float32)
    for side, mask in ((0, left), (1, ~left)):
        np.add.at(hist[side], y[rows[mask]].astype(np.int64), 1.0)
    hist = np.ascontiguousarray(hist.reshape(-1))
    out = np.zeros(len(rows), np.int32)
    cc = np.zeros(2, np.int32)
    probs = np.zeros(C, np.float32)
    leaf = lib().ref_perform_split_f(C, N, X.ctypes.data, attribute, split_point, len(rows),
                                     depth, max_depth, min_node_size, rows.ctypes.data,
                                     hist.ctypes.data, out.ctypes.data, cc.ctypes.data,
                                     probs.ctypes.data)
    return bool(leaf), out, cc, probs


def predict(nodes, probs, n_trees, C, task, X):
    X = np.ascontiguousarray(X, np.float32)
    F, N = X.shape
    nodes = np.ascontiguousarray(nodes, np.int32)
    probs = np.ascontiguousarray(probs, np.float32)
    out = np.zeros((N, C if task == 0 else 1), np.float32)
    lib().ref_predict_f(nodes.ctypes.data, probs.ctypes.data, n_trees, C, task, X.ctypes.data,
                        N, out.ctypes.data)
    return out


def parse_csv(text, cap=1 << 20):
    n, f, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    s = np.zeros(cap, np.float32)
    y = np.zeros(cap, np.float32)
    rc = lib().ref_parse_csv_f(text.encode(), ctypes.byref(n), ctypes.byref(f), ctypes.byref(t),
                               s.ctypes.data, y.ctypes.data, cap)
    if rc != 0:
        raise ValueError("reference CSV parser failed (%d)" % rc)
    N, F = n.value, f.value
    return s[:N * F].reshape(F, N).copy(), y[:N].copy(), t.value


def accuracy(preds, targets):
    preds = np.ascontiguousarray(preds, np.float32)
    targets = np.ascontiguousarray(targets, np.float32)
    N, C = preds.shape
    return lib().ref_accuracy_f(preds.ctypes.data, N, C, targets.ctypes.data)
