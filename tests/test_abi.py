"""The C ABI without a GPU: the library loads and exports every entry point
include/dml.h declares, the ctypes mirror has the C layouts, and the checks
that run before any device work reject bad input."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "dml.h")


@pytest.fixture(scope="module")
def lib():
    from datamininglibs_gb300 import build, ensembles
    if not os.path.exists(build.LIB):
        build.build()
    return ensembles.lib()


def declared():
    text = open(HEADER).read()
    return re.findall(r"DML_API\s+[\w\s\*]+?\b(dml_\w+)\s*\(", text)


def test_every_declared_entry_point_is_exported(lib):
    names = declared()
    assert len(names) >= 20
    from datamininglibs_gb300 import ensembles
    for n in names:
        assert hasattr(lib, n), n
        assert n in ensembles._SIGS, "no ctypes signature for " + n


def test_struct_layouts_match_the_header(tmp_path):
    from datamininglibs_gb300 import ensembles as e
    structs = {"dml_fit_desc": e.FitDesc, "dml_forest_info": e.ForestInfo,
               "dml_fit_stats": e.FitStats, "dml_oob_stats": e.OobStats,
               "dml_server_config": e.ServerConfig, "dml_server_stats": e.ServerStats}
    src = tmp_path / "sizes.c"
    body = "".join('  printf("%s %%zu\\n", sizeof(%s));\n' % (k, k) for k in structs)
    src.write_text('#include <stdio.h>\n#include "dml.h"\nint main(void) {\n' + body +
                   "  return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c99", "-I" + os.path.dirname(HEADER), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    for line in out.split("\n"):
        if line:
            name, size = line.split()
            assert int(size) == ctypes.sizeof(structs[name]), name


def test_forest_file_checks_run_before_device_work(lib, tmp_path):
    """A file that is not a forest, a truncated one and one whose hash does not
    match are refused on the host with DML_ERR_INVALID_ARG."""
    h = ctypes.c_void_p()
    bad = tmp_path / "junk.dmlf"
    bad.write_bytes(b"not a forest file at all" * 4)
    assert lib.dml_forest_load(os.fsencode(str(bad)), ctypes.byref(h)) == 1
    assert b"not a valid forest file" in lib.dml_last_error()
    hdr = b"DMLF" + np.array([1], np.uint32).tobytes() + np.array([0, 1, 2, 3], np.int32).tobytes()
    hdr += np.array([1, 2], np.int64).tobytes()
    node = np.array([-1, 0, 0, -1, 0], np.int32).tobytes()
    probs = np.array([1.0, 0.0], np.float32).tobytes()
    trunc = tmp_path / "trunc.dmlf"
    trunc.write_bytes(hdr + node)
    assert lib.dml_forest_load(os.fsencode(str(trunc)), ctypes.byref(h)) == 1
    wrong = tmp_path / "hash.dmlf"
    wrong.write_bytes(hdr + node + probs + b"\0" * 8)
    assert lib.dml_forest_load(os.fsencode(str(wrong)), ctypes.byref(h)) == 1
    missing = tmp_path / "missing.dmlf"
    assert lib.dml_forest_load(os.fsencode(str(missing)), ctypes.byref(h)) == 1


def test_server_config_checked_before_device_work(lib):
    from datamininglibs_gb300 import ensembles as e
    h = ctypes.c_void_p()
    for cfg in (e.ServerConfig(0, 1024, 2, 0, 0), e.ServerConfig(1 << 30, 0, 2, 0, 0),
                e.ServerConfig(1 << 30, 1024, 0, 0, 0), e.ServerConfig(1 << 30, 1024, 2, -1, 0),
                e.ServerConfig(1 << 30, 1024, 2, 0, -5)):
        assert lib.dml_server_create(ctypes.byref(cfg), ctypes.byref(h)) == 1


def test_forest_import_structure_checked_before_device_work(lib):
    """dml_forest_import refuses on the host a node array whose internal nodes
    do not point forward to an adjacent child pair inside the array (the
    guarantee that a predict walk ends), whose split attribute is out of
    range, or whose leaves point outside the probability array."""
    def imp(nodes, probs, n_trees=1, n_classes=2, n_features=3, task=0):
        nodes = np.ascontiguousarray(nodes, np.int32)
        probs = np.ascontiguousarray(probs, np.float32)
        h = ctypes.c_void_p()
        return lib.dml_forest_import(task, n_trees, n_classes, n_features, nodes.ctypes.data,
                                     len(nodes), probs.ctypes.data, len(probs), ctypes.byref(h))

    thr = int(np.array([0.5], np.float32).view(np.int32)[0])
    leaf = [-1, 0, 0, -1, -1]       # child_start, child_count, prob_start, attribute, split
    probs = np.array([1, 0, 0, 1], np.float32)

    def split(child, attr=0, count=2):
        return [child, count, -1, attr, thr]

    cases = {
        "child points backward (a cycle)": [split(0), leaf, [-1, 0, 2, -1, -1]],
        "child pair runs past the array": [split(2), leaf, [-1, 0, 2, -1, -1]],
        "one child": [split(1, count=1), leaf, [-1, 0, 2, -1, -1]],
        "attribute out of range": [split(1, attr=3), leaf, [-1, 0, 2, -1, -1]],
        "negative attribute": [split(1, attr=-2), leaf, [-1, 0, 2, -1, -1]],
        "leaf past the probabilities": [split(1), leaf, [-1, 0, 3, -1, -1]],
        "leaf before the probabilities": [split(1), leaf, [-1, 0, -1, -1, -1]],
    }
    for what, nodes in cases.items():
        assert imp(nodes, probs) == 1, what
        assert b"malformed" in lib.dml_last_error() or b"outside" in lib.dml_last_error(), what
    # bad arguments: fewer nodes than trees, unknown task, classes out of range
    ok_nodes = [split(1), leaf, [-1, 0, 2, -1, -1]]
    assert imp(ok_nodes, probs, n_trees=4) == 1
    assert imp(ok_nodes, probs, task=7) == 1
    assert imp(ok_nodes, probs, n_classes=0) == 1


def test_fit_descriptors_checked_before_device_work(lib):
    """dml_fit and dml_fit_batched refuse bad descriptors on the host with
    DML_ERR_INVALID_ARG and a message naming the forest, before any device
    work (so this runs without a GPU)."""
    from datamininglibs_gb300 import ensembles as e
    X = np.zeros((4, 100), np.float32)
    y = np.zeros(100, np.float32)

    def desc(**kw):
        p = dict(algo=0, task=0, n_trees=2, K=0, max_depth=10, min_node_size=5, min_leaf=1,
                 n_classes=2, seed=0, balanced=0)
        p.update(kw)
        return e._desc(X, y, p["algo"], p["task"], p["n_trees"], p["K"], p["max_depth"],
                       p["min_node_size"], p["min_leaf"], p["n_classes"], p["seed"], 0,
                       p["balanced"])

    bad = [dict(n_trees=0), dict(n_classes=0), dict(n_classes=33), dict(algo=5), dict(task=3),
           dict(task=1, balanced=1), dict(algo=1, balanced=1), dict(max_depth=-1), dict(K=-1),
           dict(min_node_size=-1)]
    h = ctypes.c_void_p()
    for kw in bad:
        d = desc(**kw)
        assert lib.dml_fit(ctypes.byref(d), ctypes.byref(h), None) == 1, kw
        assert lib.dml_last_error().startswith(b"forest 0:"), kw
    arr = (e.FitDesc * 3)(desc(), desc(n_classes=2), desc(algo=7))
    outs = (ctypes.c_void_p * 3)()
    assert lib.dml_fit_batched(3, arr, outs, None) == 1
    assert lib.dml_last_error().startswith(b"forest 2:")


def test_noalloc_descriptors_checked_before_device_work(lib):
    """dml_fit_noalloc refuses, on the host and before it touches its device
    array, what dml_fit refuses (a negative tree_offset included) and problems
    larger than its array, with DML_ERR_INVALID_ARG."""
    from datamininglibs_gb300 import ensembles as e
    X = np.zeros((4, 100), np.float32)
    y = np.zeros(100, np.float32)

    def desc(tree_offset=0, n_rows=100, **kw):
        p = dict(algo=0, task=0, n_trees=2, K=0, max_depth=10, min_node_size=5, min_leaf=1,
                 n_classes=2, seed=0)
        p.update(kw)
        d = e._desc(X, y, p["algo"], p["task"], p["n_trees"], p["K"], p["max_depth"],
                    p["min_node_size"], p["min_leaf"], p["n_classes"], p["seed"], tree_offset, 0)
        d.memory = e.DEVICE  # never dereferenced: the checks come first
        d.n_rows = n_rows
        return d

    nn, npb = ctypes.c_int64(), ctypes.c_int64()
    fake = ctypes.c_void_p(4096)
    bad = [dict(tree_offset=-1), dict(n_trees=0), dict(max_depth=-1), dict(K=-1),
           dict(min_node_size=-1), dict(algo=4), dict(n_rows=4097), dict(n_classes=9),
           dict(n_trees=700)]
    for kw in bad:
        d = desc(**kw)
        assert lib.dml_fit_noalloc(ctypes.byref(d), fake, 1 << 30, fake, 1 << 30,
                                   ctypes.byref(nn), ctypes.byref(npb), None) == 1, kw
    host = desc()
    host.memory = e.HOST
    assert lib.dml_fit_noalloc(ctypes.byref(host), fake, 1 << 30, fake, 1 << 30, ctypes.byref(nn),
                               ctypes.byref(npb), None) == 1
    assert b"device pointers" in lib.dml_last_error()
