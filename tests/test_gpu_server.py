"""Prediction server (dml_server_*): continuous batching over resident forests.

Each request's result through the server, mixed with requests for other
forests in shared launches, equals the same rows predicted alone with
dml_predict (votes exact, regression sums bit-exact: same per-row tree order).
"""
import numpy as np
import pytest

from datamininglibs_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def forests():
    import datamininglibs_gb300 as dml
    out = []
    X, y = synth.ert_binary(3000, 12, seed=1)
    out.append((dml.fit(X, y, algo=1, n_trees=24, K=4, max_depth=10, min_node_size=5,
                        n_classes=2, seed=1), "ert_binary", 12))
    X, y = synth.rf_multiclass(4000, 20, n_classes=5, n_int=3, seed=2)
    out.append((dml.fit(X, y, algo=0, n_trees=16, K=5, max_depth=14, min_node_size=5,
                        n_classes=5, seed=2), "rf_multiclass", 20))
    X, y = synth.rf_regression(4000, 10, seed=3)
    out.append((dml.fit(X, y, algo=0, task=1, n_trees=12, K=4, max_depth=14,
                        min_node_size=5, seed=3), "rf_regression", 10))
    return out


def _mixed(forests, srv, rng, n_req, max_rows, alloc):
    ids = [srv.add_forest(f) for f, _, _ in forests]
    reqs = []
    for k in range(n_req):
        fi = int(rng.integers(len(forests)))
        f, kind, F = forests[fi]
        n = int(np.exp(rng.uniform(0, np.log(max_rows))))
        X = alloc((F, n))
        X[...] = synth.request_rows(rng, n, F, kind)
        width = f.info().n_classes
        out = alloc((n, width))
        out[...] = np.nan
        rid = srv.submit(ids[fi], X, out)
        reqs.append((rid, fi, X, out))
    lat = [srv.wait(rid) for rid, _, _, _ in reqs]
    for rid, fi, X, out in reqs:
        alone = forests[fi][0].predict(np.ascontiguousarray(X))
        assert np.array_equal(out, alone), rid
    return reqs, lat


def test_mixed_requests_equal_alone(forests):
    """Both lanes (small requests whole, with the trees of a row split over
    threads; large requests in slices of max_batch_rows) give each request the
    votes of dml_predict on the same rows."""
    import datamininglibs_gb300 as dml
    srv = dml.Server(hbm_budget_bytes=256 << 20, max_batch_rows=3000, n_streams=3,
                     max_wait_us=200, small_rows=700)
    rng = np.random.default_rng(7)
    reqs, lat = _mixed(forests, srv, rng, 300, 12000,
                       lambda shape: np.empty(shape, np.float32))
    st = srv.stats()
    assert st.completed == len(reqs)
    assert st.launches < len(reqs)  # requests shared launches
    assert 0 < st.p50_ms <= st.p99_ms
    assert all(x > 0 for x in lat)
    srv.close()


def test_pinned_buffers_copied_directly(forests):
    """Pinned request buffers take the DMA path (no staging); same results."""
    import torch
    import datamininglibs_gb300 as dml
    srv = dml.Server(hbm_budget_bytes=128 << 20, max_batch_rows=2048, n_streams=2,
                     max_wait_us=50, small_rows=512)
    rng = np.random.default_rng(11)
    keep = []

    def pinned(shape):
        t = torch.empty(shape, dtype=torch.float32, pin_memory=True)
        keep.append(t)
        return t.numpy()
    reqs, _ = _mixed(forests, srv, rng, 120, 9000, pinned)
    assert srv.stats().completed == len(reqs)
    srv.close()


def test_budget_admission(forests):
    """A large request is sliced to fit the budget; one whose single rows
    cannot fit is rejected with DML_ERR_BUDGET."""
    import datamininglibs_gb300 as dml
    srv = dml.Server(hbm_budget_bytes=1 << 20, max_batch_rows=1 << 16, n_streams=2,
                     max_wait_us=0)
    fid = srv.add_forest(forests[1][0])
    rng = np.random.default_rng(3)
    big = np.ascontiguousarray(synth.request_rows(rng, 20000, 20, "rf_multiclass"))
    out = np.zeros((20000, 5), np.float32)  # 1.6 MB of rows > the budget: sliced
    srv.wait(srv.submit(fid, big, out))
    assert np.array_equal(out, forests[1][0].predict(big))
    Xw, yw = synth.rf_multiclass(600, 700, n_classes=3, n_int=0, seed=4)
    wide = dml.fit(Xw, yw, algo=0, n_trees=2, K=5, max_depth=4, n_classes=3, seed=1)
    wid = srv.add_forest(wide)
    with pytest.raises(dml.DmlError) as e:  # 192 rows x 700 features > a slot's share
        srv.submit(wid, np.zeros((700, 5000), np.float32), np.zeros((5000, 3), np.float32))
    assert e.value.status == 5
    assert srv.stats().rejected == 1
    srv.close()
    wide.free()
