"""The C++ drop-in (datamininglibs_gb300/shim) through a test program written
against the reference's public API."""
import os
import subprocess

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "datamininglibs_gb300")


@pytest.fixture(scope="session")
def shim_test(tmp_path_factory):
    from datamininglibs_gb300 import build
    if not (os.path.exists(build.LIB) and os.path.exists(build.SHIM_LIB)):
        build.build()
    exe = str(tmp_path_factory.mktemp("shim") / "shim_test")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(PKG, "shim", "include"),
                    os.path.join(HERE, "cpp", "shim_test.cc"), "-o", exe, "-L" + PKG,
                    "-ldml_gb300_shim", "-ldml_gb300", "-Wl,-rpath," + PKG], check=True)
    return exe


def _read(f):
    n = int(np.frombuffer(f.read(8), np.int64)[0])
    return n


def test_csv_parser_matches_the_reference(shim_test, golden_dir, tmp_path):
    """ParsingInterface::ParseFile on the reference's own test fixtures
    (lib_ensembles/test/test_resources.h:9-25) equals what the reference's
    CsvParser produced (tests/golden/ref_csv.npz)."""
    d = np.load(os.path.join(golden_dir, "ref_csv.npz"))
    for key in ("csv_data_fit", "csv_data_predict"):
        src = tmp_path / (key + ".csv")
        src.write_text(str(d[key + "_text"]))
        out = tmp_path / (key + ".bin")
        subprocess.run([shim_test, "parse", str(src), str(out)], check=True)
        with open(out, "rb") as f:
            N, F, T = np.frombuffer(f.read(12), np.int32)
            ns = _read(f)
            X = np.frombuffer(f.read(4 * ns), np.float32)
            ny = _read(f)
            y = np.frombuffer(f.read(4 * ny), np.float32)
        assert (N, F) == (d[key + "_X"].shape[1], d[key + "_X"].shape[0])
        assert T == int(d[key + "_ntargets"])
        assert np.array_equal(X.reshape(F, N), d[key + "_X"])
        assert np.array_equal(y, d[key + "_y"])


def test_csv_parser_rejects_ragged_rows(shim_test, tmp_path):
    src = tmp_path / "bad.csv"
    src.write_text("a,b,c\n1,2,0\n3,4\n")
    r = subprocess.run([shim_test, "parse", str(src), str(tmp_path / "o.bin")])
    assert r.returncode == 3


def test_shim_host_parts(shim_test):
    """Param-pack defaults, SplitParameterPack keeping every user value with
    tree offsets, SplitModel / AggregateModels round trips, AggregateResults
    and the accuracy rule, all on the host (no GPU)."""
    r = subprocess.run([shim_test, "host"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "host ok" in r.stdout


@pytest.mark.gpu
def test_shim_fit_predict_split_aggregate(shim_test, tmp_path):
    from datamininglibs_gb300 import synth
    X, y = synth.rf_multiclass(2500, 14, n_classes=4, n_int=3, seed=9)
    with open(tmp_path / "data.bin", "wb") as f:
        f.write(np.array([X.shape[1], X.shape[0], 4], np.int32).tobytes())
        f.write(X.tobytes())
        f.write(y.tobytes())
    r = subprocess.run([shim_test, "fit", str(tmp_path / "data.bin"), str(tmp_path)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "shim ok" in r.stdout

    def load(name):
        with open(tmp_path / name, "rb") as f:
            n = _read(f)
            nodes = np.frombuffer(f.read(4 * n), np.int32).reshape(-1, 5)
            n = _read(f)
            probs = np.frombuffer(f.read(4 * n), np.float32)
            n = _read(f)
            votes = np.frombuffer(f.read(4 * n), np.float32)
        return nodes, probs, votes

    nodes, probs, votes = load("model.bin")
    m = oracle.fit(X, y, algo=0, n_trees=12, K=5, max_depth=14, min_node_size=5, min_leaf=2,
                   n_classes=4, seed=3)
    assert np.array_equal(nodes, m.nodes) and np.array_equal(probs, m.probs)
    assert np.array_equal(votes.reshape(-1, 4), oracle.predict(m, X))
    nodes, probs, votes = load("ert.bin")
    m = oracle.fit(X, y, algo=1, n_trees=100, K=0, max_depth=1000, min_node_size=5,
                   n_classes=4, seed=0)
    assert np.array_equal(nodes, m.nodes) and np.array_equal(probs, m.probs)


@pytest.fixture(scope="session")
def reference_style_test(tmp_path_factory, shim_test):
    exe = str(tmp_path_factory.mktemp("refstyle") / "reference_style_test")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I" + os.path.join(PKG, "shim", "include"),
                    os.path.join(HERE, "cpp", "reference_style_test.cc"), "-o", exe, "-L" + PKG,
                    "-ldml_gb300_shim", "-ldml_gb300", "-Wl,-rpath," + PKG], check=True)
    return exe


def test_reference_style_classes_on_the_host(reference_style_test):
    """A pack class and a model class written as the reference writes them
    (SetParam / GetParam, AddData / GetData only) compile against the drop-in;
    SplitParameterPack through AlgorithmsInterface::CreateGpuAlgorithm copies
    such a pack (no GPU)."""
    r = subprocess.run([reference_style_test, "host"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "host ok" in r.stdout


@pytest.mark.gpu
def test_reference_style_program_fits(reference_style_test, tmp_path):
    """The ensembles_interface.cc:14-26 pattern (a single-device algorithm
    wrapped by CreateGpuAlgorithm<T>) fitted with a reference-style pack gives
    the library factory's forest; a reference-style model predicts alike; a
    double frame of float values gives the float forest, one with a value no
    float equals is refused, and double predictions equal a double walk of the
    model on the host."""
    from datamininglibs_gb300 import synth
    X, y = synth.rf_multiclass(2000, 10, n_classes=3, n_int=2, seed=12)
    with open(tmp_path / "data.bin", "wb") as f:
        f.write(np.array([X.shape[1], X.shape[0], 3], np.int32).tobytes())
        f.write(X.tobytes())
        f.write(y.tobytes())
    r = subprocess.run([reference_style_test, "fit", str(tmp_path / "data.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "reference style ok" in r.stdout
