"""Failure detection without a GPU fault: forced device-allocation failures.

With DML_FAIL_ALLOC=k in the environment, the k-th device allocation of one
call fails as out of memory, on the host, before the allocation is attempted
(no kernel is broken, nothing waits).  Every position k of a fit, a batched fit,
an out-of-bag estimate and a server creation is tried: each call either reports
DML_ERR_OOM with the injected message, or (where the engine has a fallback, as
the value ranks have) completes; completed fits equal the oracle's forest, and
a fit after every failure still does, so no failure leaves state behind."""
import numpy as np
import pytest

import oracle
from datamininglibs_gb300 import synth

pytestmark = pytest.mark.gpu
OOM = 2


@pytest.fixture(scope="module")
def dml():
    import datamininglibs_gb300 as d
    d.lib()
    return d


def _sweep(monkeypatch, call, check, max_k=400):
    """Runs call() with DML_FAIL_ALLOC = 1, 2, ... until thirty calls in a row
    complete (k past the call's allocations: the value ranks' temporaries fall
    back rather than fail, so a few completions can come between failures);
    returns the number of OOMs."""
    ooms, streak = 0, 0
    for k in range(1, max_k):
        monkeypatch.setenv("DML_FAIL_ALLOC", str(k))
        try:
            out = call()
        except Exception as e:  # noqa: BLE001 - checked below
            assert getattr(e, "status", None) == OOM, (k, e)
            assert "DML_FAIL_ALLOC" in str(e), (k, e)
            ooms += 1
            streak = 0
            continue
        finally:
            monkeypatch.delenv("DML_FAIL_ALLOC", raising=False)
        check(out)
        streak += 1
        if streak >= 30:
            break
    return ooms


def test_fit_survives_a_failure_at_every_allocation(dml, monkeypatch):
    # rows enough for big nodes (more entries than the shared-memory cap)
    X, y = synth.rf_multiclass(6000, 12, n_classes=3, n_int=2, seed=4)
    kw = dict(algo=0, n_trees=4, K=4, max_depth=10, min_node_size=5, n_classes=3, seed=1)
    m = oracle.fit(X, y, **kw)

    def check(f):
        nodes, probs = f.export()
        f.free()
        assert np.array_equal(nodes, m.nodes) and np.array_equal(probs, m.probs)

    ooms = _sweep(monkeypatch, lambda: dml.fit(X, y, **kw), check)
    assert ooms >= 15
    check(dml.fit(X, y, **kw))


def test_batched_fit_and_regression_survive_failures(dml, monkeypatch):
    probs = synth.uneven_problems(3, seed=8, n_range=(300, 3000), f_range=(6, 20))
    Xr, yr = synth.rf_regression(5000, 6, seed=9)
    specs = [dict(X=X, y=y, algo=1, n_trees=3, K=0, max_depth=8, min_node_size=5, n_classes=c,
                  seed=i) for i, (X, y, c) in enumerate(probs)]
    specs.append(dict(X=Xr, y=yr, algo=0, task=1, n_trees=3, K=3, max_depth=9, min_node_size=5,
                      seed=3))
    want = []
    for sp in specs:
        sp = dict(sp)
        X, y = sp.pop("X"), sp.pop("y")
        want.append(oracle.fit(X, y, **sp))

    def check(fs):
        for f, m in zip(fs, want):
            nodes, pr = f.export()
            f.free()
            assert np.array_equal(nodes, m.nodes) and np.array_equal(pr, m.probs)

    assert _sweep(monkeypatch, lambda: dml.fit_batched(specs), check) >= 15


def test_oob_estimate_survives_failures(dml, monkeypatch):
    X, y = synth.rf_multiclass(3000, 8, n_classes=3, n_int=2, seed=5)
    kw = dict(algo=0, n_trees=4, K=3, max_depth=9, min_node_size=5, n_classes=3, seed=2)
    f = dml.fit(X, y, **kw)
    want = dml.oob_estimate(f, X, y, seed=2)

    def check(st):
        assert (st.pairs, st.pairs_correct, st.rows, st.rows_correct) == (
            want.pairs, want.pairs_correct, want.rows, want.rows_correct)

    assert _sweep(monkeypatch, lambda: dml.oob_estimate(f, X, y, seed=2), check) >= 1


def test_server_creation_survives_failures(dml, monkeypatch):
    X, y = synth.ert_binary(1200, 10, seed=6)
    f = dml.fit(X, y, algo=1, n_trees=6, K=3, max_depth=8, n_classes=2, seed=1)
    want = f.predict(X[:, :300].copy())

    def make():
        return dml.Server(hbm_budget_bytes=64 << 20, max_batch_rows=4096, n_streams=2,
                          max_wait_us=0, small_rows=256)

    Xs = np.ascontiguousarray(X[:, :300])  # must stay valid until the request completes

    def check(srv):
        fid = srv.add_forest(f)
        out = np.zeros((300, 2), np.float32)
        srv.wait(srv.submit(fid, Xs, out))
        srv.close()
        assert np.array_equal(out, want)

    assert _sweep(monkeypatch, make, check) >= 4
