"""The scheduling lookup without a GPU (dml_tuning_get, csrc/tuning.cu): the
defaults per class-count width, a DML_TUNE_CACHE line taken for its problem's
shape bucket only, the persistent CTAs clamped to what the kernel's registers
allow, and invalid lines ignored.  The cache is read once per process, so each
case runs in a child process."""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import datamininglibs_gb300 as dml
out = {}
for name, rows, feats, kw in json.loads(sys.argv[2]):
    X = np.zeros((feats, rows), np.float32)
    y = np.zeros(rows, np.float32)
    out[name] = dml.tuning_for(X, y, **kw)
print(json.dumps(out))
"""

PROBLEMS = [
    ("rf10", 1000, 12, dict(algo=0, n_classes=10, K=4)),
    ("rf10_near", 1100, 12, dict(algo=0, n_classes=10, K=4)),   # same log2 buckets
    ("rf10_big", 4000, 12, dict(algo=0, n_classes=10, K=4)),    # another row bucket
    ("reg", 1000, 12, dict(algo=0, task=1, K=4)),
    ("rf32", 1000, 12, dict(algo=0, n_classes=32, K=4)),
]


@pytest.fixture(scope="module")
def built():
    from datamininglibs_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()


def _run(cache_lines, tmp_path):
    env = dict(os.environ)
    env.pop("DML_TUNE_CACHE", None)
    if cache_lines is not None:
        path = tmp_path / "tune.jsonl"
        path.write_text("".join(line + "\n" for line in cache_lines))
        env["DML_TUNE_CACHE"] = str(path)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, json.dumps(PROBLEMS)], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def _t(w, s, b):
    return {"warp_max": w, "smem_cap": s, "big_ctas_per_sm": b}


def test_defaults_per_class_width(built, tmp_path):
    got = _run(None, tmp_path)
    # three persistent big-item CTAs for one packed class word (regression,
    # two classes), four up to 16 classes, two above
    assert got["rf10"] == _t(512, 2048, 4)
    assert got["reg"] == _t(512, 2048, 3)
    assert got["rf32"] == _t(512, 2048, 2)


def test_cache_line_applies_to_its_bucket_only(built, tmp_path):
    # key: algorithm, task, class-count width, log2 rows, log2 features, K
    lines = [json.dumps({"key": "a0-t0-c5-n10-f4-k4", "warp_max": 128, "smem_cap": 1024,
                         "big_ctas": 2}),
             json.dumps({"key": "a0-t1-c1-n10-f4-k4", "warp_max": 64, "smem_cap": 4096,
                         "big_ctas": 4})]
    got = _run(lines, tmp_path)
    assert got["rf10"] == _t(128, 1024, 2)
    assert got["rf10_near"] == _t(128, 1024, 2)
    assert got["rf10_big"] == _t(512, 2048, 4)
    # four CTAs asked for, three allowed for one class word
    assert got["reg"] == _t(64, 4096, 3)
    assert got["rf32"] == _t(512, 2048, 2)


def test_invalid_cache_lines_are_ignored(built, tmp_path):
    lines = ["not json at all",
             json.dumps({"key": "a0-t0-c5-n10-f4-k4", "warp_max": 100, "smem_cap": 1024,
                         "big_ctas": 2}),
             json.dumps({"key": "a0-t1-c1-n10-f4-k4", "warp_max": 256, "smem_cap": 8192,
                         "big_ctas": 2}),
             json.dumps({"key": "a0-t0-c16-n10-f4-k4", "warp_max": 256, "smem_cap": 1024,
                         "big_ctas": 0})]
    got = _run(lines, tmp_path)
    assert got["rf10"] == _t(512, 2048, 4)
    assert got["reg"] == _t(512, 2048, 3)
    assert got["rf32"] == _t(512, 2048, 2)
