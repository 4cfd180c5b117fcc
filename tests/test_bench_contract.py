"""The bench line's inputs that do not need a GPU: the figures it reads from
the committed ncu summaries (the list build's DRAM traffic and its issue-bound
figures) and the workload configuration both arms print."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_contract", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_list_build_traffic_is_read_from_its_profile(bench):
    traffic = bench.traffic_from_profile("k_knn_first_gauss3d_1e7")
    assert traffic is not None and traffic > 0
    # DRAM bytes of one 10^7-point launch: at least the algorithmic 101 B per point
    assert traffic >= bench.KNN_BYTES_PER_POINT * 10_000_000


def test_list_build_issue_figures_are_read_from_its_profile(bench):
    issue = bench.issue_from_profile("k_knn_first")
    assert issue is not None
    assert 0.0 < issue["issue_slots_busy"] <= 1.0
    assert issue["warp_instructions_per_32_queries"] > 0
    assert 0.0 < issue["active_lanes_per_instruction"] <= 32.0


def test_missing_profile_gives_null(bench):
    assert bench.traffic_from_profile("no_such_kernel_no_such_workload") is None
    assert bench.issue_from_profile("no_such_kernel") is None


def test_both_arms_name_the_same_workload(bench):
    a = bench.workload_config("gauss3d_1e7", 10_000_000, 3)
    b = bench.workload_config("gauss3d_1e7", 10_000_000, 3)
    assert a == b
    assert a["workload"] == "gauss3d_1e7" and a["n"] == 10_000_000 and a["dim"] == 3
    assert "l2" in a
