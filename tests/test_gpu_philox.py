"""The engine's Philox4x32-10 against cuRAND's Philox4_32_10 on the GPU (the
counter-based generator that replaces the reference's cuRAND MRG32k3a draws)."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "datamininglibs_gb300", "csrc")


def test_philox_matches_curand(tmp_path):
    exe = str(tmp_path / "philox_vs_curand")
    subprocess.run(["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I" + CSRC, os.path.join(HERE, "cuda", "philox_vs_curand.cu"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatching words: 0" in r.stdout
