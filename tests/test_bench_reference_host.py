"""The CPU reference timing of bench.py (the oracle port of upstream's algorithm), on CPU:
the one-core sample of the GPU line's cpu_baseline and the all-cores form of
``bench.py --impl reference`` (spawned oracle processes), each with a small time budget."""

import multiprocessing
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_cpu_baseline_one_core():
    line = bench.cpu_baseline(0.5)
    assert line["cores"] == 1 and line["kind"] == "port" and line["unit"] == "s"
    assert line["value"] > 0
    parts = line["parts_s"]
    assert parts["gs_s"] > 0 and parts["xas_s"] > 0 and parts["rixs_s"] > 0
    assert "1 core" in line["sample"]


@pytest.mark.timeout(300)
def test_reference_time_on_worker_pool():
    procs = 2
    with multiprocessing.get_context("spawn").Pool(procs, initializer=bench._ref_worker_init) as pool:
        total, sample, parts = bench.cpu_reference_time(0.3, pool=pool, procs=procs)
    assert total > 0 and all(v > 0 for v in parts.values())
    assert "2 cores" in sample and "750 RIXS units" in sample
