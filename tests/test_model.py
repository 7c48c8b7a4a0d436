"""Breadth-first tree extraction (datamininglibs_gb300.model.tree_arrays) on the
CPU: a tree of a forest fitted at once equals the same tree of a forest fitted
in parts, and a one-tree forest is already in breadth-first form."""
import numpy as np

import oracle
from datamininglibs_gb300 import model, synth


def test_trees_of_a_forest_equal_the_trees_of_its_parts():
    X, y = synth.rf_multiclass(3000, 12, n_classes=4, n_int=3, seed=3)
    kw = dict(algo=0, K=4, max_depth=10, min_node_size=5, n_classes=4, seed=7)
    whole = oracle.fit(X, y, n_trees=5, **kw)
    parts = [oracle.fit(X, y, n_trees=2, tree_offset=0, **kw),
             oracle.fit(X, y, n_trees=3, tree_offset=2, **kw)]
    for t in range(5):
        p, k = (parts[0], t) if t < 2 else (parts[1], t - 2)
        a = model.tree_arrays(whole.nodes, whole.probs, 4, t, whole.gains32)
        b = model.tree_arrays(p.nodes, p.probs, 4, k, p.gains32)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        assert np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32))
        # the extracted tree predicts like the whole forest's tree alone
        one = oracle.Model(a[0], a[1], 1, 4, 0)
        assert one.nodes[0, 1] in (0, 2)
    single = oracle.fit(X, y, n_trees=1, **kw)
    n, p = model.tree_arrays(single.nodes, single.probs, 4, 0)
    assert np.array_equal(n, single.nodes) and np.array_equal(p, single.probs)


def test_regression_tree_extraction_keeps_leaf_values():
    X, y = synth.rf_regression(2000, 8, seed=4)
    m = oracle.fit(X, y, algo=0, task=1, n_trees=3, K=3, max_depth=8, min_node_size=5, seed=1)
    total = 0.0
    Xs = X[:, :50]
    for t in range(3):
        n, p = model.tree_arrays(m.nodes, m.probs, 1, t)
        total = total + oracle.predict(oracle.Model(n, p, 1, 1, 1), Xs)
    assert np.array_equal(total, oracle.predict(m, Xs))
