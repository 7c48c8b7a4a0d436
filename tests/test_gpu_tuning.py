"""Scheduling (dml_autotune / DML_TUNE_CACHE) changes which kernel searches a
node, never the split: fits under extreme tunings equal the oracle's."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from datamininglibs_gb300 import synth

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

KW = dict(algo=0, n_trees=4, K=4, max_depth=12, min_node_size=5, n_classes=3, seed=9)
CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import datamininglibs_gb300 as dml
from datamininglibs_gb300 import synth
X, y = synth.rf_multiclass(20000, 12, n_classes=3, n_int=3, seed=8)
kw = dict(algo=0, n_trees=4, K=4, max_depth=12, min_node_size=5, n_classes=3, seed=9)
print(dml.tuning_for(X, y, **kw))
f = dml.fit(X, y, **kw)
nodes, probs = f.export()
np.save(sys.argv[2], nodes)
"""


@pytest.mark.parametrize("tuning", [(64, 300, 1), (128, 2048, 2), (256, 4096, 2),
                                    (512, 1024, 3)])
def test_forced_tunings_give_the_oracle_forest(tmp_path, tuning):
    X, y = synth.rf_multiclass(20000, 12, n_classes=3, n_int=3, seed=8)
    m = oracle.fit(X, y, **KW)
    cache = tmp_path / "tune.jsonl"
    # the bucket of this problem: RF, classification, 3 classes (2 words), 2^14 rows
    key = "a0-t0-c2-n%d-f%d-k4" % (round(np.log2(20000)), round(np.log2(12)))
    cache.write_text(json.dumps({"key": key, "warp_max": tuning[0], "smem_cap": tuning[1],
                                 "big_ctas": tuning[2]}) + "\n")
    out = str(tmp_path / "nodes.npy")
    env = dict(os.environ, DML_TUNE_CACHE=str(cache))
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, out], env=env, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    assert "'warp_max': %d" % tuning[0] in r.stdout and "'smem_cap': %d" % tuning[1] in r.stdout
    assert np.array_equal(np.load(out), m.nodes)


REG_KW = dict(algo=0, task=1, n_trees=3, K=4, max_depth=10, min_node_size=5, min_leaf=2, seed=5)
REG_CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import datamininglibs_gb300 as dml
from datamininglibs_gb300 import synth
X, y = synth.rf_regression(12000, 8, seed=14)
kw = dict(algo=0, task=1, n_trees=3, K=4, max_depth=10, min_node_size=5, min_leaf=2, seed=5)
print(dml.tuning_for(X, y, **kw))
np.save(sys.argv[2], dml.fit(X, y, **kw).export()[0])
"""


@pytest.mark.parametrize("tuning", [(64, 300, 1), (512, 4096, 3)])
def test_forced_tunings_regression(tmp_path, tuning):
    """The regression scans (warp kernels, shared-memory kernel, big-node
    items) under extreme node-class boundaries give the oracle's forest."""
    X, y = synth.rf_regression(12000, 8, seed=14)
    m = oracle.fit(X, y, **REG_KW)
    cache = tmp_path / "tune.jsonl"
    key = "a0-t1-c1-n%d-f%d-k4" % (round(np.log2(12000)), round(np.log2(8)))
    cache.write_text(json.dumps({"key": key, "warp_max": tuning[0], "smem_cap": tuning[1],
                                 "big_ctas": tuning[2]}) + "\n")
    out = str(tmp_path / "nodes.npy")
    env = dict(os.environ, DML_TUNE_CACHE=str(cache))
    r = subprocess.run([sys.executable, "-c", REG_CHILD, ROOT, out], env=env,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "'warp_max': %d" % tuning[0] in r.stdout and "'smem_cap': %d" % tuning[1] in r.stdout
    assert np.array_equal(np.load(out), m.nodes)


def test_autotune_records_its_choice():
    import datamininglibs_gb300 as dml
    X, y = synth.rf_multiclass(30000, 16, n_classes=5, n_int=3, seed=12)
    kw = dict(algo=0, n_trees=6, K=4, max_depth=14, min_node_size=5, n_classes=5, seed=2)
    best = dml.autotune(X, y, sample_trees=2, **kw)
    assert best == dml.tuning_for(X, y, **kw)
    f = dml.fit(X, y, **kw)
    nodes, probs = f.export()
    m = oracle.fit(X, y, **kw)
    assert np.array_equal(nodes, m.nodes) and np.array_equal(probs, m.probs)
