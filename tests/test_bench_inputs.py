"""The committed ncu summaries that bench.py reads for its roofline object: every top kernel's file
parses, with its DRAM bytes per launch and pipe utilisations, and names the command that made it."""
import os

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("kernel", ["k_probes", "k_visibility", "k_neighbors", "k_probe_jobs", "k_probe_neighbors"])
def test_profile_summaries(kernel):
    p = bench.profiled(kernel)
    assert p["traffic"] > 0
    assert 0 < p["issue_active"] <= 1 and 0 < p["alu_pipe"] <= 1 and 0 < p["fma_pipe"] <= 1
    assert 1 <= p["threads_per_instruction"] <= 32
    text = open(os.path.join(ROOT, "profiles", f"{kernel}_assembly100k.txt")).read()
    assert "ncu --set full --clock-control none" in text and "python bench.py" in text


def test_launch_list_summary():
    text = open(os.path.join(ROOT, "profiles", "launches_assembly100k_full.md")).read()
    assert "--clock-control none" in text
    rows = [ln for ln in text.splitlines() if ln.startswith("| k_")]
    names = {ln.split("|")[1].strip().split("<")[0] for ln in rows}
    assert {"k_probes", "k_visibility", "k_neighbors"} <= names
