"""The allocation-free fit (dml_fit_noalloc) against dml_fit, through the C ABI.

dml_fit_noalloc serves callers that cannot allocate device memory while they
fit: a process whose device memory belongs to its own allocator or budget, or a
service that keeps cudaMalloc / cudaFree (device synchronisation, failures under
fragmentation) out of its steady state.  Its working buffers are one static
device array shared by all calls, which keeps the last call's contents, so each
call here checks that stale contents left by the previous call do not leak into
the next: different fits in a row, each compared with dml_fit's model (trees
and leaf counts bit-exact, as in the other parity tests).  This file is
collected last, so that a run stopping at the first failure has run every other
test before it.
"""
import numpy as np
import pytest

from datamininglibs_gb300 import synth

pytestmark = pytest.mark.gpu


def _run(dml, torch, X, y, **kw):
    ref_nodes, ref_probs = dml.fit(X, y, **kw).export()
    n, T = X.shape[1], kw["n_trees"]
    C = kw.get("n_classes", 2) if kw.get("task", 0) == 0 else 1
    nodes = torch.full((T * (2 * n - 1), 5), -7, dtype=torch.int32, device="cuda")
    probs = torch.full((T * n * C,), -7.0, dtype=torch.float32, device="cuda")
    nn, npb = dml.ensembles.fit_noalloc(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda(),
                                        nodes, probs, **kw)
    torch.cuda.synchronize()
    got_nodes = nodes[:nn].cpu().numpy()
    got_probs = probs[:npb].cpu().numpy()
    assert got_nodes.shape == ref_nodes.shape
    assert np.array_equal(got_nodes, ref_nodes)
    assert np.array_equal(got_probs, ref_probs)


def test_noalloc_fit_matches_fit_twice_in_a_row():
    torch = pytest.importorskip("torch")
    import datamininglibs_gb300 as dml
    dml.lib()
    X1, y1 = synth.rf_multiclass(3000, 12, n_classes=5, n_int=2, seed=3)
    _run(dml, torch, X1, y1, algo=0, n_trees=16, K=4, max_depth=14, min_node_size=5,
         min_leaf=2, n_classes=5, seed=11)
    X2, y2 = synth.ert_binary(4096, 9, seed=4)
    _run(dml, torch, X2, y2, algo=1, n_trees=12, K=3, max_depth=10, min_node_size=6,
         n_classes=2, seed=12)
    X3, y3 = synth.rf_regression(2000, 7, seed=5)
    _run(dml, torch, X3, y3, algo=0, task=1, n_trees=8, K=3, max_depth=12, min_node_size=5,
         seed=13)


def test_noalloc_fit_rejects_problems_beyond_its_array():
    torch = pytest.importorskip("torch")
    import datamininglibs_gb300 as dml
    X, y = synth.ert_binary(5000, 4, seed=1)
    nodes = torch.zeros((10, 5), dtype=torch.int32, device="cuda")
    probs = torch.zeros(10, dtype=torch.float32, device="cuda")
    with pytest.raises(dml.DmlError) as e:
        dml.ensembles.fit_noalloc(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda(),
                                  nodes, probs, algo=1, n_trees=4, n_classes=2)
    assert e.value.status == 1 and "at most" in str(e.value)
