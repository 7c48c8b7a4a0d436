"""Host-side helpers on models in the reference's Classify layout.

A model is the pair (kNodeArray, kProbArray) of lib_models
(models_interface.h:9-19): ``nodes`` int32 [n, 5] = {child_start, child_count,
probability_start, attribute, split_point as float bits} with the roots of the
trees at 0..n_trees-1 and the two children of an internal node adjacent;
``probs`` holds C floats per leaf (1 for regression).
"""
import numpy as np


def tree_arrays(nodes, probs, n_classes, tree, gains=None):
    """Tree ``tree`` of a forest as a model of its own, in breadth-first order
    (root first, each level in parent order, left child before right).

    Any two forests that hold the same tree give identical arrays, whatever the
    order in which their fits laid the trees out (one tree at a time, level by
    level over a whole forest, or a forest split into parts), so trees of a
    128-tree fit compare directly with the trees of a 16-tree fit.  Returns
    (nodes, probs) or (nodes, probs, gains) when ``gains`` (one per node of the
    forest) is given."""
    nodes = np.asarray(nodes, np.int32)
    C = max(1, int(n_classes))
    levels = []
    frontier = np.array([tree], np.int64)
    while frontier.size:
        levels.append(frontier)
        nd = nodes[frontier]
        ch = nd[nd[:, 1] > 0, 0].astype(np.int64)
        frontier = np.stack([ch, ch + 1], axis=1).reshape(-1)
    idx = np.concatenate(levels)
    sub = nodes[idx].copy()
    internal = sub[:, 1] > 0
    # in breadth-first order the children of the i-th internal node sit at
    # 1 + 2i and 2 + 2i; the j-th leaf owns probabilities [j*C, (j+1)*C)
    sub[internal, 0] = 1 + 2 * (np.cumsum(internal)[internal] - 1)
    leaf = ~internal
    old_p = sub[leaf, 2].astype(np.int64)
    sub[leaf, 2] = C * np.arange(old_p.size, dtype=np.int64)
    sub_probs = np.asarray(probs)[(old_p[:, None] + np.arange(C)[None, :]).reshape(-1)]
    if gains is None:
        return sub, sub_probs
    return sub, sub_probs, np.asarray(gains)[idx]


def node_depths(nodes, n_trees):
    """Depth of every node of a forest (roots 0..n_trees-1 at depth 0)."""
    nodes = np.asarray(nodes, np.int32)
    depth = np.full(nodes.shape[0], -1, np.int32)
    frontier = np.arange(n_trees, dtype=np.int64)
    d = 0
    while frontier.size:
        depth[frontier] = d
        nd = nodes[frontier]
        ch = nd[nd[:, 1] > 0, 0].astype(np.int64)
        frontier = np.stack([ch, ch + 1], axis=1).reshape(-1)
        d += 1
    return depth


def mean_path_nodes(nodes, probs, n_trees, n_classes):
    """Nodes a prediction walk loads per tree, averaged over the rows the
    forest was fitted on: each leaf's depth + 1 weighted by the training
    weight that reached it (its class counts' sum; a tree of a bootstrap fit
    holds as many draws as rows, so the weights estimate the rows' share)."""
    nodes = np.asarray(nodes, np.int32)
    depth = node_depths(nodes, n_trees)
    leaf = nodes[:, 1] == 0
    C = max(1, int(n_classes))
    ps = nodes[leaf, 2].astype(np.int64)
    w = np.asarray(probs, np.float64)[(ps[:, None] + np.arange(C)[None, :])].sum(axis=1)
    return float(((depth[leaf] + 1) * w).sum() / w.sum())
