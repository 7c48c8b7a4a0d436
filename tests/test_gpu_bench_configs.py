"""Parity at the benchmark configurations' own sizes.

The smaller parity cases (test_gpu_parity.py) cover the algorithm's branches;
these check the forests that bench.py times: the ERT binary workload at its
exact configuration, trees of the 128-tree RF multiclass forest, the RF
regression workload on its full 4,000,000 x 64 data, and the first trees of
every one of the 256 uneven forests fitted in one batch.  Trees are compared in
breadth-first form (datamininglibs_gb300.model.tree_arrays), so a tree of a
128-tree fit compares with the same tree of a shorter oracle fit.  Tolerances:
trees, leaf payloads and votes bit-exact; FP32 gains equal to the oracle's FP32
gains bit for bit and within 1e-6 relative + 1e-7 absolute of its FP64 gains;
regression predictions within 1e-5 relative (they are bit-exact: same trees,
same tree order)."""
import numpy as np
import pytest

import oracle
from datamininglibs_gb300 import model, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dml():
    import datamininglibs_gb300 as d
    d.lib()
    return d


def _check_gains(g, m_nodes, g32, g64, tag):
    split = m_nodes[:, 1] > 0
    assert np.array_equal(np.isnan(g), ~split), tag
    assert np.array_equal(g[split].view(np.uint32), g32[split].view(np.uint32)), tag
    err = np.abs(g[split].astype(np.float64) - g64[split])
    assert np.all(err <= 1e-6 * np.abs(g64[split]) + 1e-7), (tag, err.max())


def _check_trees(nodes, probs, gains, C, m, trees, tag):
    """Trees `trees` of an engine forest against trees 0.. of oracle model m."""
    for k, t in enumerate(trees):
        en, ep, eg = model.tree_arrays(nodes, probs, C, t, gains)
        on, op, og32 = model.tree_arrays(m.nodes, m.probs, C, k, m.gains32)
        og64 = model.tree_arrays(m.nodes, m.probs, C, k, m.gains64)[2]
        assert en.shape == on.shape, (tag, t, en.shape, on.shape)
        bad = np.nonzero(np.any(en != on, axis=1))[0]
        assert bad.size == 0, (tag, t, "first differing node", bad[:3], en[bad[:2]], on[bad[:2]])
        assert np.array_equal(ep, op), (tag, t)
        _check_gains(eg, on, og32, og64, "%s tree %d" % (tag, t))


def test_ert_binary_at_its_configuration(dml):
    """4601 x 57 zero-inflated lognormal, 64 trees, K = 7, depth 12, min node
    size 10, seed 0: the whole forest, its votes and its gains."""
    X, y = synth.ert_binary()
    kw = dict(algo=1, n_trees=64, K=7, max_depth=12, min_node_size=10, n_classes=2, seed=0)
    m = oracle.fit(X, y, **kw)
    f = dml.fit(X, y, **kw)
    nodes, probs = f.export()
    assert np.array_equal(nodes, m.nodes) and np.array_equal(probs, m.probs)
    _check_gains(f.gains(), m.nodes, m.gains32, m.gains64, "ert_binary")
    assert np.array_equal(f.predict(X), oracle.predict(m, X))


def test_rf_multiclass_trees_of_the_timed_forest(dml):
    """Trees 0 and 1 of the 128-tree fit of the 1,000,000 x 128, 10-class
    workload (K = 11, depth 20, min leaf 2) against a 2-tree oracle fit."""
    X, y = synth.rf_multiclass()
    kw = dict(algo=0, K=11, max_depth=20, min_node_size=5, min_leaf=2, n_classes=10, seed=0)
    f = dml.fit(X, y, n_trees=128, **kw)
    nodes, probs = f.export()
    gains = f.gains()
    f.free()
    m = oracle.fit(X, y, n_trees=2, **kw)
    _check_trees(nodes, probs, gains, 10, m, [0, 1], "rf_multiclass")


def test_rf_regression_full_size_two_trees(dml):
    """The 4,000,000 x 64 regression workload (K = 21, depth 24, min leaf 5):
    trees 0 and 1 fitted as two parts through tree_offset and as one 2-tree
    forest, against the oracle; predictions on 200,000 of the rows."""
    X, y = synth.rf_regression()
    kw = dict(algo=0, task=1, K=21, max_depth=24, min_node_size=5, min_leaf=5, seed=0)
    m = oracle.fit(X, y, n_trees=2, **kw)
    f2 = dml.fit(X, y, n_trees=2, **kw)
    nodes, probs = f2.export()
    _check_trees(nodes, probs, f2.gains(), 1, m, [0, 1], "rf_regression")
    for t in (0, 1):
        ft = dml.fit(X, y, n_trees=1, tree_offset=t, **kw)
        n1, p1 = ft.export()
        mt = model.tree_arrays(m.nodes, m.probs, 1, t)
        assert np.array_equal(n1, mt[0]) and np.array_equal(p1, mt[1]), t
        ft.free()
    Xs = np.ascontiguousarray(X[:, :200_000])
    pg = f2.predict(Xs)
    po = oracle.predict(m, Xs)
    assert np.all(np.abs(pg - po) <= 1e-5 * np.abs(po) + 1e-30)
    f2.free()


def test_uneven_forests_all_256_first_two_trees(dml):
    """The 256 uneven ERT problems (rows 200..50,000, features 8..256, 2..8
    classes) fitted in one batch of 16 trees each, depth 16, min node size 5:
    trees 0 and 1 of every forest against a 2-tree oracle fit."""
    probs = synth.uneven_problems(256, seed=0)
    specs = [dict(X=X, y=y, algo=1, n_trees=16, K=0, max_depth=16, min_node_size=5, n_classes=c,
                  seed=i) for i, (X, y, c) in enumerate(probs)]
    batch = dml.fit_batched(specs)
    for i, ((X, y, c), fb) in enumerate(zip(probs, batch)):
        nodes, pr = fb.export()
        g = fb.gains()
        fb.free()
        m = oracle.fit(X, y, algo=1, n_trees=2, K=0, max_depth=16, min_node_size=5, n_classes=c,
                       seed=i)
        _check_trees(nodes, pr, g, c, m, [0, 1], "uneven %d" % i)
