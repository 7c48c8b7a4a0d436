"""CUDA engine vs the oracle through the C ABI: trees, leaf payloads and votes
bit-exact, regression sums bit-exact (same tree order), on seeded inputs of the
benchmark distributions at sizes the oracle finishes in seconds, plus the edge
cases of the reference's path."""
import numpy as np
import pytest

import oracle
from datamininglibs_gb300 import synth

pytestmark = pytest.mark.gpu
FLT_MAX = np.finfo(np.float32).max


@pytest.fixture(scope="module")
def dml():
    import datamininglibs_gb300 as d
    d.lib()
    return d


def _fit_both(dml, X, y, **kw):
    m = oracle.fit(X, y, **kw)
    f = dml.fit(X, y, **kw)
    nodes, probs = f.export()
    return m, f, nodes, probs


def _assert_same_model(m, nodes, probs, tag=""):
    assert nodes.shape == m.nodes.shape, (tag, nodes.shape, m.nodes.shape)
    bad = np.nonzero(np.any(nodes != m.nodes, axis=1))[0]
    assert bad.size == 0, (tag, "first differing node", bad[:5], nodes[bad[:3]], m.nodes[bad[:3]])
    assert np.array_equal(probs, m.probs), tag


CASES = {
    "ert_cls": (lambda: synth.ert_binary(1500, 21, seed=1),
                dict(algo=1, n_trees=16, K=7, max_depth=12, min_node_size=10, n_classes=2, seed=0)),
    "rf_cls": (lambda: synth.rf_multiclass(3000, 24, n_classes=10, n_int=4, seed=2),
               dict(algo=0, n_trees=12, K=5, max_depth=20, min_node_size=5, min_leaf=2,
                    n_classes=10, seed=3)),
    "rf_reg": (lambda: synth.rf_regression(3000, 16, seed=4),
               dict(algo=0, task=1, n_trees=8, K=6, max_depth=24, min_node_size=5, min_leaf=5,
                    seed=5)),
    "ert_reg": (lambda: synth.rf_regression(2000, 12, seed=6),
                dict(algo=1, task=1, n_trees=8, K=4, max_depth=14, min_node_size=5, seed=7)),
    "rf_cls_big_nodes": (lambda: synth.rf_multiclass(20000, 12, n_classes=3, n_int=3, seed=8),
                         dict(algo=0, n_trees=3, K=4, max_depth=8, min_node_size=5,
                              n_classes=3, seed=9)),
    "rf_reg_big_nodes": (lambda: synth.rf_regression(12000, 10, seed=10),
                         dict(algo=0, task=1, n_trees=3, K=4, max_depth=6, min_node_size=5,
                              seed=11)),
    "ert_cls_multiclass": (lambda: synth.rf_multiclass(4000, 30, n_classes=7, n_int=5, seed=12),
                           dict(algo=1, n_trees=10, K=6, max_depth=16, min_node_size=5,
                                n_classes=7, seed=13)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fit_and_predict_bit_exact(dml, name):
    gen, kw = CASES[name]
    X, y = gen()
    m, f, nodes, probs = _fit_both(dml, X, y, **kw)
    _assert_same_model(m, nodes, probs, name)
    pg = f.predict(X)
    po = oracle.predict(m, X)
    assert np.array_equal(pg, po), name


GAIN_CASES = {
    "ert_binary": (lambda: synth.ert_binary(2500, 57, seed=3),
                   dict(algo=1, n_trees=16, K=7, max_depth=12, min_node_size=10, n_classes=2,
                        seed=4)),
    "rf_10_classes": (lambda: synth.rf_multiclass(20000, 32, n_classes=10, n_int=4, seed=21),
                      dict(algo=0, n_trees=6, K=6, max_depth=20, min_node_size=5, min_leaf=2,
                           n_classes=10, seed=2)),
    "rf_regression": (lambda: synth.rf_regression(12000, 16, seed=22),
                      dict(algo=0, task=1, n_trees=4, K=6, max_depth=24, min_node_size=5,
                           min_leaf=5, seed=3)),
    "ert_regression": (lambda: synth.rf_regression(3000, 12, seed=23),
                       dict(algo=1, task=1, n_trees=6, K=4, max_depth=14, min_node_size=5,
                            seed=4)),
}


@pytest.mark.parametrize("name", sorted(GAIN_CASES))
def test_gains_within_tolerance_of_fp64(dml, name):
    """The FP32 gain of every split as the engine computed it on the device
    (dml_forest_gains): bit for bit the oracle's FP32 gain, and within
    1e-6 relative + 1e-7 absolute of the oracle's FP64 gain.  Leaves hold NaN."""
    gen, kw = GAIN_CASES[name]
    X, y = gen()
    m, f, nodes, probs = _fit_both(dml, X, y, **kw)
    _assert_same_model(m, nodes, probs, name)
    g = f.gains()
    split = nodes[:, 1] > 0
    assert split.any(), name
    assert np.array_equal(np.isnan(g), ~split), name
    assert np.array_equal(g[split].view(np.uint32), m.gains32[split].view(np.uint32)), name
    err = np.abs(g[split].astype(np.float64) - m.gains64[split])
    assert np.all(err <= 1e-6 * np.abs(m.gains64[split]) + 1e-7), (name, err.max())


def test_imported_forest_has_no_gains(dml):
    X, y = synth.ert_binary(600, 8, seed=5)
    f = dml.fit(X, y, algo=1, n_trees=2, K=3, max_depth=6, n_classes=2, seed=1)
    nodes, probs = f.export()
    g = dml.Forest.from_model(nodes, probs, task=0, n_trees=2, n_classes=2, n_features=8)
    with pytest.raises(dml.DmlError):
        g.gains()


def test_plain_path_matches_level_path(dml):
    X, y = synth.rf_multiclass(4000, 20, n_classes=4, n_int=2, seed=31)
    kw = dict(algo=0, n_trees=6, K=5, max_depth=15, min_node_size=5, n_classes=4, seed=1)
    a = dml.fit(X, y, **kw).export()
    b = dml.fit_plain(X, y, **kw).export()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_batched_uneven_forests_match_single_fits(dml):
    probs = synth.uneven_problems(6, seed=5, n_range=(200, 3000), f_range=(8, 40))
    specs = []
    for i, (X, y, c) in enumerate(probs):
        specs.append(dict(X=X, y=y, algo=1 if i % 3 else 0, n_trees=4, K=0, max_depth=10,
                          min_node_size=5, n_classes=c, seed=100 + i))
    specs.append(dict(X=probs[0][0], y=synth.rf_regression(probs[0][0].shape[1], 3, seed=1)[1],
                      algo=0, task=1, n_trees=3, K=3, max_depth=9, min_node_size=5, seed=7))
    batch = dml.fit_batched(specs)
    for sp, fb in zip(specs, batch):
        sp = dict(sp)
        X, y = sp.pop("X"), sp.pop("y")
        m = oracle.fit(X, y, **sp)
        nodes, pr = fb.export()
        _assert_same_model(m, nodes, pr)


def test_batched_regression_big_nodes_beside_ten_classes(dml):
    """A regression problem with nodes above the shared-memory cap fitted in
    one batch with a 10-class problem: the regression scans run in the kernels
    of the widest class word and give each problem the oracle's forest."""
    Xc, yc = synth.rf_multiclass(3000, 10, n_classes=10, n_int=3, seed=71)
    Xr, yr = synth.rf_regression(7000, 6, seed=72)
    specs = [dict(X=Xc, y=yc, algo=0, n_trees=3, K=3, max_depth=10, min_node_size=5,
                  n_classes=10, seed=73),
             dict(X=Xr, y=yr, algo=0, task=1, n_trees=3, K=3, max_depth=9, min_node_size=5,
                  min_leaf=2, seed=74)]
    batch = dml.fit_batched(specs)
    for sp, fb in zip(specs, batch):
        sp = dict(sp)
        X, y = sp.pop("X"), sp.pop("y")
        m = oracle.fit(X, y, **sp)
        nodes, pr = fb.export()
        _assert_same_model(m, nodes, pr)
        assert np.array_equal(fb.predict(X), oracle.predict(m, X))


def test_export_into_given_buffers(dml):
    X, y = synth.ert_binary(800, 8, seed=3)
    f = dml.fit(X, y, algo=1, n_trees=3, K=3, max_depth=8, n_classes=2, seed=1)
    nodes, probs = f.export()
    n2, p2 = np.full_like(nodes, -7), np.full_like(probs, -7.0)
    out = f.export(n2, p2)
    assert out[0] is n2 and out[1] is p2
    assert np.array_equal(n2, nodes) and np.array_equal(p2, probs)
    with pytest.raises(ValueError):
        f.export(n2[:-1], p2)
    with pytest.raises(ValueError):
        f.export(n2, p2.astype(np.float64))


def test_pinned_host_buffers_copied_by_sms(dml):
    """Samples and labels in pinned host memory are uploaded, and a model
    exported into pinned buffers (and a prediction into a pinned result) is
    downloaded, by SM copies through the buffers' mapped pointers (the samples' and labels' sizes here, 156,052 and
    12,004 bytes, leave a 4-byte tail for the copy engines): the same forest,
    bit for bit, as from and into pageable arrays."""
    torch = pytest.importorskip("torch")
    X, y = synth.rf_multiclass(3001, 13, n_classes=5, n_int=2, seed=61)
    kw = dict(algo=0, n_trees=6, K=4, max_depth=12, min_node_size=5, n_classes=5, seed=2)
    ref = dml.fit(X, y, **kw)
    rn, rp = ref.export()
    Xp = torch.from_numpy(X).pin_memory().numpy()
    yp = torch.from_numpy(y).pin_memory().numpy()
    f = dml.fit(Xp, yp, **kw)
    info = f.info()
    nbuf = torch.empty((info.n_nodes, 5), dtype=torch.int32, pin_memory=True).numpy()
    pbuf = torch.empty(info.n_probs, dtype=torch.float32, pin_memory=True).numpy()
    nodes, probs = f.export(nbuf, pbuf)
    assert np.array_equal(nodes, rn) and np.array_equal(probs, rp)
    # predict from pinned rows into a pinned result
    out = torch.empty((X.shape[1], 5), dtype=torch.float32, pin_memory=True).numpy()
    assert np.array_equal(f.predict(Xp, out=out), ref.predict(X))


def test_forests_of_one_fit_free_independently(dml):
    """The forests of one fit share one device allocation: each stays whole
    (export and predict equal the oracle's) while the others are freed in any
    order, and freeing the last releases the block."""
    probs = synth.uneven_problems(5, seed=9, n_range=(300, 2000), f_range=(6, 20))
    specs = [dict(X=X, y=y, algo=i % 2, n_trees=3, K=0, max_depth=8, min_node_size=5,
                  n_classes=c, seed=40 + i) for i, (X, y, c) in enumerate(probs)]
    batch = dml.fit_batched(specs)
    models = []
    for sp in specs:
        sp = dict(sp)
        X, y = sp.pop("X"), sp.pop("y")
        models.append((oracle.fit(X, y, **sp), X))
    for i in (3, 0, 4, 1, 2):
        batch[i].free()
        for j in range(len(specs)):
            if j in (3, 0, 4, 1, 2)[: (3, 0, 4, 1, 2).index(i) + 1]:
                continue
            m, X = models[j]
            nodes, pr = batch[j].export()
            _assert_same_model(m, nodes, pr, tag="forest %d after freeing %d" % (j, i))
            assert np.array_equal(batch[j].predict(X), oracle.predict(m, X)), (j, i)


def test_repeated_fits_bitwise_identical(dml):
    X, y = synth.ert_binary(2500, 20, seed=41)
    kw = dict(algo=0, n_trees=8, K=5, max_depth=12, min_node_size=5, n_classes=2, seed=4)
    ref = dml.fit(X, y, **kw).export()
    for _ in range(2):
        again = dml.fit(X, y, **kw).export()
        assert np.array_equal(ref[0], again[0]) and np.array_equal(ref[1], again[1])


@pytest.mark.parametrize("name", ["rf_cls", "ert_cls"])
def test_overlapped_node_classes_equal_serial_ones(dml, monkeypatch, name):
    """Small fits launch a level's node classes on streams of their own; with
    DML_SERIAL_CLASSES=1 they run one after another.  Same forest, bit for
    bit, with every node class present (nodes from the root down to a few
    entries)."""
    gen, kw = CASES[name]
    X, y = gen()
    over = dml.fit(X, y, **kw)
    monkeypatch.setenv("DML_SERIAL_CLASSES", "1")
    serial = dml.fit(X, y, **kw)
    a, b = over.export(), serial.export()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(over.gains().view(np.uint32), serial.gains().view(np.uint32))


EDGE = {
    "root_leaf_depth0": dict(max_depth=0),
    "min_node_size_huge": dict(min_node_size=10 ** 6),
    "k_greater_than_f": dict(K=50),
    "k_equals_f": dict(K=6),
    "min_leaf_large": dict(min_leaf=40),
    "single_class": dict(n_classes=1),
}


@pytest.mark.parametrize("name", sorted(EDGE))
@pytest.mark.parametrize("algo", [0, 1])
def test_edge_parameters(dml, name, algo):
    X, y = synth.rf_multiclass(700, 6, n_classes=3, n_int=2, seed=51)
    kw = dict(algo=algo, n_trees=5, K=3, max_depth=9, min_node_size=4, n_classes=3, seed=8)
    kw.update(EDGE[name])
    if kw["n_classes"] == 1:
        y = np.zeros_like(y)
    m, f, nodes, probs = _fit_both(dml, X, y, **kw)
    _assert_same_model(m, nodes, probs, name)
    assert np.array_equal(f.predict(X), oracle.predict(m, X))


@pytest.mark.parametrize("algo", [0, 1])
def test_missing_values_and_constant_features(dml, algo):
    X, y = synth.rf_multiclass(1200, 8, n_classes=3, n_int=2, seed=61)
    X[2] = 1.5                     # constant feature: never splits
    X[:, ::5] = -FLT_MAX           # missing-value marker goes left
    X[4, ::3] = 0.0
    X[4, 1::3] = -0.0              # -0 and +0 are one value
    kw = dict(algo=algo, n_trees=6, K=4, max_depth=10, min_node_size=4, n_classes=3, seed=3)
    m, f, nodes, probs = _fit_both(dml, X, y, **kw)
    _assert_same_model(m, nodes, probs)
    Xq = X.copy()
    Xq[:, 1::7] = -FLT_MAX
    assert np.array_equal(f.predict(Xq), oracle.predict(m, Xq))


def test_big_nodes_with_signed_zeros_and_missing(dml):
    """Nodes above the shared-memory sort size: thresholds next to -0/+0 and the
    missing-value marker, classification and regression."""
    X, y = synth.rf_multiclass(12000, 6, n_classes=3, n_int=2, seed=17)
    X[1, ::3] = 0.0
    X[1, 1::3] = -0.0
    X[2, ::4] = -FLT_MAX
    X[3] = np.where(X[3] > 0, -0.0, X[3])
    for task in (0, 1):
        yy = y if task == 0 else (y * 0.5 - 0.3).astype(np.float32)
        kw = dict(algo=0, task=task, n_trees=3, K=4, max_depth=7, min_node_size=5,
                  n_classes=3, seed=5)
        m, f, nodes, probs = _fit_both(dml, X, yy, **kw)
        _assert_same_model(m, nodes, probs, task)


@pytest.mark.parametrize("n_rows", [1, 2, 3, 33, 65, 129, 257, 513, 1025, 2049, 4097])
def test_tiny_and_boundary_sizes(dml, n_rows):
    X, y = synth.rf_multiclass(n_rows, 5, n_classes=2, n_int=1, seed=n_rows)
    for algo in (0, 1):
        kw = dict(algo=algo, n_trees=3, K=2, max_depth=20, min_node_size=1, n_classes=2, seed=1)
        m, f, nodes, probs = _fit_both(dml, X, y, **kw)
        _assert_same_model(m, nodes, probs, (n_rows, algo))


def test_many_classes(dml):
    X, y = synth.rf_multiclass(3000, 10, n_classes=32, n_int=2, seed=71)
    for algo in (0, 1):
        kw = dict(algo=algo, n_trees=4, K=4, max_depth=12, min_node_size=5, n_classes=32, seed=2)
        m, f, nodes, probs = _fit_both(dml, X, y, **kw)
        _assert_same_model(m, nodes, probs, algo)
        assert np.array_equal(f.predict(X), oracle.predict(m, X))


def test_regression_negative_and_tiny_targets(dml):
    X, _ = synth.rf_regression(1500, 6, seed=81)
    rng = np.random.default_rng(0)
    y = (rng.standard_normal(1500) * 1e-3 - 5e-4).astype(np.float32)
    for algo in (0, 1):
        kw = dict(algo=algo, task=1, n_trees=4, K=3, max_depth=10, min_node_size=5, seed=2)
        m, f, nodes, probs = _fit_both(dml, X, y, **kw)
        _assert_same_model(m, nodes, probs, algo)
        pg, po = f.predict(X), oracle.predict(m, X)
        assert np.array_equal(pg, po)


@pytest.mark.parametrize("kind", ["discrete", "overflow", "large", "tiny"])
def test_regression_big_nodes_tied_and_extreme_targets(dml, kind):
    """Regression nodes above the shared-memory cap (the bounded boundary scan
    of the big items): targets of four values over features of 20 values make
    many exactly tied gains; targets near 1e30 make every gain +inf (ties at
    infinity), near 1e13 large finite gains, near 1e-12 gains near 1e-21 with
    the target scale at its upper clamp."""
    X, y = synth.rf_regression(7000, 6, seed=91)
    rng = np.random.default_rng(5)
    if kind == "discrete":
        X = (np.floor(X * 20.0) / 20.0).astype(np.float32)
        y = rng.integers(0, 4, size=y.shape[0]).astype(np.float32)
    else:
        scale = {"overflow": 3e29, "large": 3e12, "tiny": 1e-12}[kind]
        y = (y * np.float32(scale)).astype(np.float32)
    kw = dict(algo=0, task=1, n_trees=3, K=3, max_depth=9, min_node_size=5, min_leaf=2, seed=4)
    m, f, nodes, probs = _fit_both(dml, X, y, **kw)
    _assert_same_model(m, nodes, probs, kind)
    assert np.array_equal(f.predict(X), oracle.predict(m, X))


def test_invalid_inputs_rejected(dml):
    X, y = synth.ert_binary(200, 5, seed=1)
    Xn = X.copy()
    Xn[1, 3] = np.nan
    with pytest.raises(dml.DmlError) as e:
        dml.fit(Xn, y, algo=1, n_trees=2, n_classes=2)
    assert e.value.status == 1
    yb = y.copy()
    yb[0] = 2.0
    with pytest.raises(dml.DmlError):
        dml.fit(X, yb, algo=0, n_trees=2, n_classes=2)
    with pytest.raises(dml.DmlError):
        dml.fit(X, y, algo=0, n_trees=2, n_classes=64)
    # the context stays usable after rejected calls
    f = dml.fit(X, y, algo=1, n_trees=2, n_classes=2)
    assert f.info().n_trees == 2


def test_device_pointers_through_the_c_abi(dml):
    torch = pytest.importorskip("torch")
    X, y = synth.ert_binary(1000, 9, seed=91)
    kw = dict(algo=0, n_trees=5, K=3, max_depth=10, min_node_size=5, n_classes=2, seed=6)
    fh = dml.fit(X, y, **kw)
    fd = dml.fit(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda(), **kw)
    assert np.array_equal(fh.export()[0], fd.export()[0])
    out = fd.predict(torch.from_numpy(X).cuda())
    assert np.array_equal(out.cpu().numpy(), fh.predict(X))


def test_import_reference_layout_model(dml):
    """A model in the kNodeArray/kProbArray layout built elsewhere (here: the
    oracle) imports and predicts identically."""
    X, y = synth.ert_binary(800, 10, seed=3)
    m = oracle.fit(X, y, algo=1, n_trees=9, K=3, max_depth=8, min_node_size=5, n_classes=2,
                   seed=1)
    f = dml.Forest.from_model(m.nodes, m.probs, task=0, n_trees=9, n_classes=2, n_features=10)
    assert np.array_equal(f.predict(X), oracle.predict(m, X))


@pytest.mark.parametrize("algo", [0, 1])
def test_tree_offset_parts_equal_the_whole_forest(dml, algo):
    """A forest fitted as parts (tree keys offset by the part's first tree, as
    SplitParameterPack hands them out) votes exactly as the forest fitted in one
    call, and each part equals the oracle's fit with the same offset."""
    X, y = synth.rf_multiclass(2500, 18, n_classes=4, n_int=3, seed=31)
    kw = dict(algo=algo, K=5, max_depth=12, min_node_size=5, n_classes=4, seed=17)
    whole = dml.fit(X, y, n_trees=10, **kw).predict(X)
    acc = np.zeros_like(whole)
    for t0, k in ((0, 3), (3, 3), (6, 4)):
        m = oracle.fit(X, y, n_trees=k, tree_offset=t0, **kw)
        f = dml.fit(X, y, n_trees=k, tree_offset=t0, **kw)
        nodes, probs = f.export()
        _assert_same_model(m, nodes, probs, f"part at {t0}")
        acc += f.predict(X)
    assert np.array_equal(acc, whole)


@pytest.mark.parametrize("name", ["rf_cls", "rf_reg"])
def test_plain_predict_matches_predict(dml, name):
    """The reference-structured predict (one thread per (tree, row), 65,536 per
    launch) gives dml_predict's votes and sums bit for bit."""
    gen, kw = CASES[name]
    X, y = gen()
    f = dml.fit(X, y, **kw)
    assert np.array_equal(f.predict_plain(X), f.predict(X))


def test_balanced_bootstrap_matches_oracle(dml):
    """kEasyEnsemble (balanced per-class bootstrap) on imbalanced classes, one
    class empty: trees and votes bit-exact."""
    X, y = synth.rf_multiclass(3000, 16, n_classes=5, n_int=3, seed=41)
    y = np.where(y == 4, 1, y).astype(np.float32)  # class 4 empty
    y[:2500] = np.where(y[:2500] == 3, 0, y[:2500])  # class 3 rare
    kw = dict(algo=0, n_trees=10, K=5, max_depth=14, min_node_size=5, n_classes=5, seed=8,
              balanced=1)
    m, f, nodes, probs = _fit_both(dml, X, y, **kw)
    _assert_same_model(m, nodes, probs, "balanced")
    assert np.array_equal(f.predict(X), oracle.predict(m, X))
    plain = oracle.fit(X, y, **dict(kw, balanced=0))
    assert plain.nodes.shape != m.nodes.shape or not np.array_equal(plain.nodes, m.nodes)


@pytest.mark.parametrize("task", [0, 1])
@pytest.mark.parametrize("balanced", [0, 1])
def test_oob_and_permutation_runs_match_oracle(dml, task, balanced):
    """dml_oob_estimate equals the oracle's restatement bit for bit (counts and
    fixed-order double sums), for the plain estimate and permutation runs."""
    if task == 1 and balanced:
        pytest.skip("balanced sampling is for classification")
    if task == 0:
        X, y = synth.rf_multiclass(5000, 14, n_classes=4, n_int=3, seed=51)
        kw = dict(algo=0, n_trees=9, K=4, max_depth=12, n_classes=4, seed=6, balanced=balanced)
    else:
        X, y = synth.rf_regression(5000, 10, seed=52)
        kw = dict(algo=0, task=1, n_trees=9, K=4, max_depth=12, min_leaf=3, seed=6)
    m = oracle.fit(X, y, **kw)
    f = dml.fit(X, y, **kw)
    for pf in (-1, 0, 5):
        o = oracle.oob(m, X, y, seed=6, balanced=balanced, permuted_feature=pf)
        g = dml.oob_estimate(f, X, y, seed=6, balanced=balanced, permuted_feature=pf)
        assert (g.pairs, g.rows) == (int(o[0]), int(o[2])), pf
        if task == 0:
            assert (g.pairs_correct, g.rows_correct) == (int(o[1]), int(o[3])), pf
        else:
            assert (g.pairs_sq_err, g.rows_sq_err) == (o[1], o[3]), pf
    imp = dml.feature_importance(f, X, y, seed=6, balanced=balanced)
    assert imp.shape == (X.shape[0],) and np.isfinite(imp).all()


def test_oob_rejects_ert_and_mismatched_descriptors(dml):
    X, y = synth.ert_binary(800, 9, seed=3)
    f = dml.fit(X, y, algo=1, n_trees=4, K=3, max_depth=6, n_classes=2)
    with pytest.raises(dml.DmlError):
        dml.ensembles.lib()  # loaded
        d = dml.ensembles._desc(X, y, 1, 0, 4, 0, 0, 0, 1, 2, 0)
        st = dml.OobStats()
        dml.ensembles._check(dml.lib().dml_oob_estimate(f.handle, d, -1, st, None))
    g = dml.fit(X, y, algo=0, n_trees=4, K=3, max_depth=6, n_classes=2)
    with pytest.raises(dml.DmlError):
        dml.oob_estimate(g, X[:5], y, seed=0)  # feature count differs from the forest's
    with pytest.raises(dml.DmlError):
        dml.oob_estimate(g, X, y, permuted_feature=9)


def test_forest_file_roundtrip(dml, tmp_path):
    """dml_forest_save / dml_forest_load keep the reference-layout arrays and
    the votes bit for bit; a flipped byte is refused."""
    gen, kw = CASES["rf_cls"]
    X, y = gen()
    f = dml.fit(X, y, **kw)
    path = str(tmp_path / "forest.dmlf")
    f.save(path)
    g = dml.Forest.load(path)
    n1, p1 = f.export()
    n2, p2 = g.export()
    assert np.array_equal(n1, n2) and np.array_equal(p1, p2)
    assert np.array_equal(f.predict(X), g.predict(X))
    raw = bytearray(open(path, "rb").read())
    raw[100] ^= 0x40
    bad = str(tmp_path / "bad.dmlf")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(dml.DmlError):
        dml.Forest.load(bad)


@pytest.mark.parametrize("task", [0, 1])
@pytest.mark.parametrize("pass_mb", [None, "1"])
def test_bulk_predict_in_tree_passes_matches_oracle(dml, monkeypatch, task, pass_mb):
    """Predictions of 70,000 rows (the bulk path: passes over blocks of trees,
    votes and regression sums carried between passes) equal the oracle's, bit
    for bit, over the compact 8-byte node layout and, with DML_PREDICT_NODE16
    set, over the 16-byte one; DML_PREDICT_PASS_MB=1 forces a pass per few
    trees."""
    if pass_mb:
        monkeypatch.setenv("DML_PREDICT_PASS_MB", pass_mb)
    if task == 0:
        X, y = synth.rf_multiclass(70000, 24, n_classes=7, n_int=4, seed=41)
        kw = dict(algo=0, n_trees=40, K=5, max_depth=14, min_node_size=5, n_classes=7, seed=5)
    else:
        X, y = synth.rf_regression(70000, 12, seed=42)
        kw = dict(algo=0, task=1, n_trees=37, K=4, max_depth=12, min_node_size=5, min_leaf=3,
                  seed=6)
    m = oracle.fit(X, y, **kw)
    f = dml.fit(X, y, **kw)
    nodes, probs = f.export()
    _assert_same_model(m, nodes, probs)
    want = oracle.predict(m, X)
    assert np.array_equal(f.predict(X), want)
    monkeypatch.setenv("DML_PREDICT_NODE16", "1")
    assert np.array_equal(f.predict(X), want)


def _large_node_case(kind):
    rng = np.random.default_rng(77)
    if kind == "cls_10":
        X, y = synth.rf_multiclass(40000, 12, n_classes=10, n_int=3, seed=78)
        return X, y, dict(algo=0, n_trees=4, K=4, max_depth=10, min_node_size=5, min_leaf=2,
                          n_classes=10, seed=4)
    if kind == "cls_ties_missing":
        X, y = synth.rf_multiclass(36000, 10, n_classes=3, n_int=2, seed=79)
        X[0] = np.round(X[0], 1)                       # many ties
        X[1, rng.random(X.shape[1]) < 0.2] = -FLT_MAX  # missing values, go left
        X[2, rng.random(X.shape[1]) < 0.3] = -0.0      # signed zeros beside +0
        X[2, rng.random(X.shape[1]) < 0.3] = 0.0
        return X, y, dict(algo=0, n_trees=3, K=10, max_depth=9, min_node_size=5,
                          n_classes=3, seed=5)
    if kind == "cls_balanced_rare_class":
        X, y = synth.rf_multiclass(40000, 8, n_classes=3, n_int=2, seed=80)
        y = np.where(y == 2, 1, y).astype(np.float32)
        y[rng.choice(y.size, 25, replace=False)] = 2   # 25 rows of class 2: weights far above 15
        return X, y, dict(algo=0, n_trees=3, K=4, max_depth=8, min_node_size=5, n_classes=3,
                          seed=6, balanced=1)
    X, y = synth.rf_regression(40000, 10, seed=81)
    X[3] = np.round(X[3], 2)
    return X, y, dict(algo=0, task=1, n_trees=3, K=5, max_depth=12, min_node_size=5,
                      min_leaf=3, seed=7)


@pytest.mark.parametrize("kind", ["cls_10", "cls_ties_missing", "cls_balanced_rare_class",
                                  "reg_ties"])
def test_large_node_edge_cases_match_oracle(dml, kind):
    """Nodes of tens of thousands of entries (far above the shared-memory cap,
    searched as per-try items) with many ties, missing values, signed zeros,
    ten classes, regression, and bootstrap weights far above 15 (a balanced
    bootstrap with a 25-row class): trees, payloads, gains and votes equal the
    oracle's."""
    X, y, kw = _large_node_case(kind)
    m, f, nodes, probs = _fit_both(dml, X, y, **kw)
    _assert_same_model(m, nodes, probs, kind)
    g = f.gains()
    split = nodes[:, 1] > 0
    assert np.array_equal(g[split].view(np.uint32), m.gains32[split].view(np.uint32)), kind
    assert np.array_equal(f.predict(X), oracle.predict(m, X)), kind
