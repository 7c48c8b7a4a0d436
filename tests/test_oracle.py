"""The oracle pinned against the reference: published Philox vectors, and golden
vectors produced by the reference's own code (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

import oracle

FLT_MAX = np.finfo(np.float32).max


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10 (Salmon et al., SC'11)
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in kat:
        assert oracle.philox(ctr, key).tolist() == want


def test_nlogn_table_accuracy():
    """Fixed point 2^-28: every entry within half a unit (plus double rounding)
    of n ln n."""
    H = oracle.nlogn_table(100000)
    n = np.arange(2, 100001, dtype=np.float64)
    exact = n * np.log(n)
    got = H[2:].astype(np.float64) / 2.0 ** 28
    assert np.all(np.abs(got - exact) <= 2.0 ** -29 + 1e-15 * exact)
    assert H[0] == 0 and H[1] == 0


def test_entropy_against_reference(golden_dir):
    d = np.load(os.path.join(golden_dir, "ref_entropy.npz"))
    for L, R, C, gf, gd in zip(d["L"], d["R"], d["C"], d["gain_ref_f32"], d["gain_ref_f64"]):
        g32, g64 = oracle.entropy_gain(L[:C], R[:C])
        # FP64 shadow == the reference's double instantiation
        assert abs(g64 - gd) <= 1e-12 * max(abs(gd), 1.0), (L[:C], R[:C])
        # FP32 (fixed-point table) gain within 1e-6 relative of FP64 (+1e-7 bits floor)
        assert abs(g32 - gd) <= 1e-6 * abs(gd) + 1e-7, (L[:C], R[:C], g32, gd)


def test_split_step_against_reference(golden_dir):
    d = np.load(os.path.join(golden_dir, "ref_split.npz"))
    for i in range(int(d["n"])):
        g = lambda k: d["%d_%s" % (i, k)]  # noqa: E731
        X = g("xcol")[None, :]
        leaf, out, cn, counts = oracle.split_node(X, g("y"), int(g("C")), 0, g("thr"), g("rows"),
                                                  int(g("depth")), int(g("max_depth")),
                                                  int(g("min_node_size")))
        assert leaf == bool(g("leaf"))
        assert np.array_equal(counts.astype(np.float32), g("probs"))
        if not leaf:
            assert np.array_equal(out, g("out"))
            assert np.array_equal(cn, g("cc"))


def _model(nodes, probs, trees, C, task):
    return oracle.Model(nodes, probs, int(trees), int(C), task)


def test_predict_against_reference(golden_dir):
    d = np.load(os.path.join(golden_dir, "ref_predict.npz"))
    m = _model(d["cls_nodes"], d["cls_probs"], d["cls_trees"], d["cls_C"], 0)
    assert np.array_equal(oracle.predict(m, d["cls_X"]), d["cls_out"])
    m = _model(d["reg_nodes"], d["reg_probs"], d["reg_trees"], 1, 1)
    assert np.array_equal(oracle.predict(m, d["reg_X"]), d["reg_out"])


def test_accuracy_rule_against_reference(golden_dir):
    from datamininglibs_gb300 import ensembles
    d = np.load(os.path.join(golden_dir, "ref_accuracy.npz"))
    assert np.float32(ensembles.accuracy(d["votes"], d["targets"])) == d["accuracy"]


def test_oracle_self_fixtures(golden_dir):
    d = np.load(os.path.join(golden_dir, "oracle_fits.npz"))
    for name in ("ert_cls", "rf_cls", "rf_reg", "ert_reg"):
        kw = {k[len(name) + 4:]: d[k].item() for k in d.files if k.startswith(name + "_kw_")}
        m = oracle.fit(d[name + "_X"], d[name + "_y"], **kw)
        assert np.array_equal(m.nodes, d[name + "_nodes"]), name
        assert np.array_equal(m.probs, d[name + "_probs"]), name
        assert np.array_equal(oracle.predict(m, d[name + "_X"]), d[name + "_pred"]), name


def test_oracle_structure_invariants():
    from datamininglibs_gb300 import synth
    X, y = synth.rf_multiclass(2000, 16, n_classes=4, n_int=3, seed=5)
    m = oracle.fit(X, y, algo=0, n_trees=5, K=4, max_depth=12, min_node_size=5, min_leaf=2,
                   n_classes=4, seed=9)
    nodes = m.nodes
    internal = nodes[:, 1] == 2
    # children adjacent, after their parent; leaves hold C counts summing to >= 1
    assert np.all(nodes[internal, 0] > np.nonzero(internal)[0])
    leaves = ~internal
    assert np.all(nodes[leaves, 3] == -1)
    sums = m.probs.reshape(-1, 4).sum(1)
    assert np.all(sums >= 1)
    # every tree's leaves hold N bootstrap draws in total
    assert int(sums.sum()) == 5 * 2000
    # min_leaf: every leaf count >= 2 unless it is a root-level leaf
    assert sums.min() >= 2


def test_reference_csv_fixture_roundtrip(golden_dir):
    """Fit/predict on the reference's own inline CSV test data
    (lib_ensembles/test/test_resources.h:9-25, parsed by its CsvParser), as its
    tests test_gpuert.h:13-30 and test_gpurf.h:13-28 do."""
    d = np.load(os.path.join(golden_dir, "ref_csv.npz"))
    X, y = d["csv_data_fit_X"], d["csv_data_fit_y"]
    Xp, yp = d["csv_data_predict_X"], d["csv_data_predict_y"]
    for algo in (0, 1):
        m = oracle.fit(X, y, algo=algo, n_trees=200, K=0, max_depth=1000, min_node_size=5,
                       n_classes=int(d["csv_data_fit_ntargets"]), seed=0)
        votes = oracle.predict(m, Xp)
        assert votes.sum() == 200 * len(yp)


@pytest.mark.skipif(not __import__("ref").available(), reason="needs the reference tree")
def test_live_reference_harness():
    """Where the reference tree is present, re-run its code on fresh cases."""
    import ref
    rng = np.random.default_rng(99)
    for _ in range(200):
        C = int(rng.integers(2, 12))
        L = rng.integers(0, 5000, C)
        R = rng.integers(1, 5000, C)
        g32, g64 = oracle.entropy_gain(L, R)
        _, gd = ref.entropy_gain(L, R)
        assert abs(g64 - gd) <= 1e-12 * max(abs(gd), 1.0)
    from datamininglibs_gb300 import synth
    X, y = synth.ert_binary(300, 9, seed=17)
    m = oracle.fit(X, y, algo=0, n_trees=7, K=3, max_depth=6, min_node_size=4, n_classes=2, seed=2)
    assert np.array_equal(oracle.predict(m, X), ref.predict(m.nodes, m.probs, 7, 2, 0, X))


def test_oracle_bags_out_of_bag_share_and_balance():
    """Plain bootstrap leaves about e^-1 of the (tree, row) pairs out of the
    bag; the balanced bootstrap draws N/C rows per non-empty class, so a rare
    class's rows are almost always in the bag."""
    from datamininglibs_gb300 import synth
    X, y = synth.rf_multiclass(4000, 8, n_classes=3, n_int=2, seed=5)
    m = oracle.fit(X, y, algo=0, n_trees=12, K=3, max_depth=4, n_classes=3, seed=1)
    o = oracle.oob(m, X, y, seed=1)
    assert abs(o[0] / (12 * 4000) - np.exp(-1)) < 0.01
    y2 = y.copy()
    rare = np.nonzero(y2 == 2)[0][100:]
    y2[rare] = 0  # class 2 keeps 100 rows
    mb = oracle.fit(X, y2, algo=0, n_trees=12, K=3, max_depth=4, n_classes=3, seed=1,
                    balanced=1)
    ob = oracle.oob(mb, X, y2, seed=1, balanced=1)
    # class c (n_c rows) gets N // C draws: a row is out of a bag with
    # probability (1 - 1/n_c)^(N // C)
    m_draw = 4000 // 3
    expect = 12 * sum(n * (1 - 1 / n) ** m_draw for n in np.bincount(y2.astype(int)) if n)
    assert abs(ob[0] / expect - 1) < 0.03
