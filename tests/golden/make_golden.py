"""Generate the golden fixtures under tests/golden/.

Two kinds of vectors are written:

* ``ref_*.npz``: outputs of the reference's own code, run through the pinning
  harness (oracle/ref_harness.cc compiled from the reference sources by
  oracle/ref.mk): entropy (gpudte.cu:70-117), the node split step
  (gpudte.cu:156-309), predict/vote (gpudte.cu:311-359), GetAccuracy
  (ml_resultdata_impl.cc:23-38) and the CSV parser (csv_parser.cc:36-104) on the
  reference's inline test fixtures (lib_ensembles/test/test_resources.h:9-25).
* ``oracle_*.npz``: the oracle's own fits on small seeded problems, so that a
  later change of the oracle (or a different host) is caught.

Run from the repository root where the reference tree exists:
    python tests/golden/make_golden.py
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import ref  # noqa: E402
from datamininglibs_gb300 import synth  # noqa: E402


def reference_csv_fixtures():
    path = os.path.join(ref.REF_ROOT, "lib_ensembles", "test", "test_resources.h")
    src = open(path).read()
    out = {}
    for name in ("csv_data_fit", "csv_data_predict"):
        m = re.search(r"char\s+%s\[\]\s*=\s*\{(.*?)\};" % name, src, re.S)
        lits = re.findall(r'"((?:[^"\\]|\\.)*)"', m.group(1))
        out[name] = "".join(lits).encode().decode("unicode_escape")
    return out


def entropy_cases(rng, n=600):
    Ls, Rs, Cs, gf, gd = [], [], [], [], []
    scales = [3, 20, 500, 20000, 400000]
    while len(Cs) < n:
        C = int(rng.integers(2, 21))
        L = rng.integers(0, scales[rng.integers(len(scales))], C)
        R = rng.integers(0, scales[rng.integers(len(scales))], C)
        if rng.random() < 0.15:
            R = L.copy()  # zero-gain tables
        if L.sum() == 0 or R.sum() == 0:
            continue
        f, d = ref.entropy_gain(L, R)
        Ls.append(np.pad(L, (0, 20 - C)))
        Rs.append(np.pad(R, (0, 20 - C)))
        Cs.append(C)
        gf.append(f)
        gd.append(d)
    return dict(L=np.array(Ls, np.int64), R=np.array(Rs, np.int64), C=np.array(Cs, np.int32),
                gain_ref_f32=np.array(gf, np.float32), gain_ref_f64=np.array(gd, np.float64))


def split_cases(rng, n=300):
    cases = []
    for _ in range(n):
        N = int(rng.integers(8, 160))
        F = 4
        C = int(rng.integers(2, 6))
        X = rng.standard_normal((F, N)).astype(np.float32)
        X[rng.random((F, N)) < 0.1] = -np.finfo(np.float32).max  # missing values
        y = rng.integers(0, C, N).astype(np.float32)
        m = int(rng.integers(1, N + 1))
        rows = np.sort(rng.choice(N, m, replace=False)).astype(np.int32)
        a = int(rng.integers(0, F))
        thr = np.float32(rng.standard_normal() * 0.8)
        depth = int(rng.integers(0, 6))
        max_depth = int(rng.integers(0, 6))
        mns = int(rng.integers(0, 12))
        leaf, out, cc, probs = ref.perform_split(X, y, C, a, thr, rows, depth, max_depth, mns)
        cases.append(dict(xcol=X[a], y=y, C=C, rows=rows, thr=thr, depth=depth,
                          max_depth=max_depth, min_node_size=mns, leaf=leaf, out=out, cc=cc,
                          probs=probs))
    return cases


def main():
    if not ref.available():
        raise SystemExit("the reference tree is needed to generate the golden vectors")
    ref.build()
    oracle.build()
    rng = np.random.default_rng(20261203)

    np.savez_compressed(os.path.join(HERE, "ref_entropy.npz"), **entropy_cases(rng))

    cases = split_cases(rng)
    flat = {}
    for i, c in enumerate(cases):
        for k, v in c.items():
            flat["%d_%s" % (i, k)] = np.asarray(v)
    flat["n"] = np.array(len(cases))
    np.savez_compressed(os.path.join(HERE, "ref_split.npz"), **flat)

    # predict/vote through the reference's gpudte_predict on oracle models
    pred = {}
    X, y = synth.ert_binary(600, 11, seed=7)
    m = oracle.fit(X, y, algo=1, n_trees=12, K=4, max_depth=7, min_node_size=6,
                   n_classes=2, seed=11)
    Xq = X.copy()
    Xq[:, ::7] = -np.finfo(np.float32).max
    pred.update(cls_nodes=m.nodes, cls_probs=m.probs, cls_X=Xq, cls_trees=12, cls_C=2,
                cls_out=ref.predict(m.nodes, m.probs, 12, 2, 0, Xq))
    Xr, yr = synth.rf_regression(700, 12, seed=8)
    mr = oracle.fit(Xr, yr, algo=0, task=1, n_trees=9, K=5, max_depth=8, min_node_size=5,
                    seed=12)
    pred.update(reg_nodes=mr.nodes, reg_probs=mr.probs, reg_X=Xr, reg_trees=9,
                reg_out=ref.predict(mr.nodes, mr.probs, 9, 1, 1, Xr))
    np.savez_compressed(os.path.join(HERE, "ref_predict.npz"), **pred)

    # GetAccuracy (argmax with strict '>' from 0, ties to the lowest class)
    votes = rng.integers(0, 4, (300, 5)).astype(np.float32)
    targets = rng.integers(0, 5, 300).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "ref_accuracy.npz"), votes=votes, targets=targets,
                        accuracy=np.float32(ref.accuracy(votes, targets)))

    # the reference's inline CSV fixtures parsed by its own CsvParser
    fx = reference_csv_fixtures()
    csv = {}
    for key, text in fx.items():
        Xc, yc, nt = ref.parse_csv(text)
        csv[key + "_text"] = np.array(text)
        csv[key + "_X"] = Xc
        csv[key + "_y"] = yc
        csv[key + "_ntargets"] = np.array(nt)
    np.savez_compressed(os.path.join(HERE, "ref_csv.npz"), **csv)

    # oracle self-fixtures: small seeded fits of every algorithm/task pair
    orc = {}
    specs = {
        "ert_cls": (synth.ert_binary(900, 14, seed=21), dict(algo=1, n_trees=10, K=5,
                    max_depth=9, min_node_size=8, n_classes=2, seed=3)),
        "rf_cls": (synth.rf_multiclass(1200, 20, n_classes=5, n_int=4, seed=22),
                   dict(algo=0, n_trees=8, K=5, max_depth=10, min_node_size=5, min_leaf=2,
                        n_classes=5, seed=4)),
        "rf_reg": (synth.rf_regression(1500, 12, seed=23), dict(algo=0, task=1, n_trees=6,
                   K=6, max_depth=11, min_node_size=5, min_leaf=5, seed=5)),
        "ert_reg": (synth.rf_regression(800, 10, seed=24), dict(algo=1, task=1, n_trees=6,
                    K=4, max_depth=8, min_node_size=5, seed=6)),
    }
    for name, ((Xs, ys), kw) in specs.items():
        mo = oracle.fit(Xs, ys, **kw)
        orc[name + "_X"] = Xs
        orc[name + "_y"] = ys
        orc[name + "_nodes"] = mo.nodes
        orc[name + "_probs"] = mo.probs
        orc[name + "_gains32"] = mo.gains32
        orc[name + "_pred"] = oracle.predict(mo, Xs)
        for k, v in kw.items():
            orc[name + "_kw_" + k] = np.array(v)
    np.savez_compressed(os.path.join(HERE, "oracle_fits.npz"), **orc)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
