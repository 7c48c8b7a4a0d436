"""The bench's roofline `traffic` comes from the committed ncu summary of the
split-search kernels: DRAM bytes per tried entry, scaled by the tried entries
of a launch.  These checks keep that link intact without a GPU."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_every_rf_classification_class_has_a_traffic_figure(bench):
    # the classes that can dominate the headline RF fit
    for kernel in ("k_rf_big_items+k_rf_big_decide", "k_rf_smem", "k_warp_rf<16>",
                   "k_group_nodes<8>"):
        t = bench.traffic_from_profile(kernel)
        assert t is not None and 0.0 < t < 1000.0, kernel


def test_traffic_names_match_the_engine_queue_names(bench):
    from datamininglibs_gb300 import ensembles
    path = os.path.join(ROOT, "profiles", "search_kernels_rf_multiclass.md")
    names = [line.split(":")[0][len("dram_bytes_per_entry_try "):]
             for line in open(path) if line.startswith("dram_bytes_per_entry_try ")]
    assert names and all(n in ensembles.QUEUE_KERNELS for n in names)


def test_unknown_kernel_has_no_traffic(bench):
    assert bench.traffic_from_profile("k_not_a_kernel") is None
