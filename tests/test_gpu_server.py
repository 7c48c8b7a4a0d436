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


def test_mixed_requests_equal_alone(forests):
    import datamininglibs_gb300 as dml
    srv = dml.Server(hbm_budget_bytes=256 << 20, max_batch_rows=1 << 16, n_streams=3,
                     max_wait_us=200)
    ids = [srv.add_forest(f) for f, _, _ in forests]
    rng = np.random.default_rng(7)
    reqs = []
    for k in range(300):
        fi = int(rng.integers(len(forests)))
        f, kind, F = forests[fi]
        n = int(np.exp(rng.uniform(0, np.log(5000))))
        X = np.ascontiguousarray(synth.request_rows(rng, n, F, kind))
        width = f.info().n_classes
        out = np.full((n, width), np.nan, np.float32)
        rid = srv.submit(ids[fi], X, out)
        reqs.append((rid, fi, X, out))
    lat = [srv.wait(rid) for rid, _, _, _ in reqs]
    for rid, fi, X, out in reqs:
        alone = forests[fi][0].predict(X)
        assert np.array_equal(out, alone), rid
    st = srv.stats()
    assert st.completed == len(reqs)
    assert st.launches < len(reqs)  # requests shared launches
    assert 0 < st.p50_ms <= st.p99_ms
    assert all(x > 0 for x in lat)
    srv.close()


def test_budget_admission(forests):
    import datamininglibs_gb300 as dml
    srv = dml.Server(hbm_budget_bytes=1 << 20, max_batch_rows=1 << 16, n_streams=2,
                     max_wait_us=0)
    fid = srv.add_forest(forests[1][0])
    big = np.zeros((20, 20000), np.float32)  # 1.6 MB of rows > the per-batch budget
    out = np.zeros((20000, 5), np.float32)
    with pytest.raises(dml.DmlError) as e:
        srv.submit(fid, big, out)
    assert e.value.status == 5
    small = np.zeros((20, 100), np.float32)
    out = np.zeros((100, 5), np.float32)
    srv.wait(srv.submit(fid, small, out))
    assert srv.stats().rejected == 1
    srv.close()
