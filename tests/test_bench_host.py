"""Host-side figures bench.py reports beside its timings (no GPU): the DRAM
traffic it reads from the committed capture summary, and the FLOPs of the
tensor-core backprojector's MMAs it divides by that kernel's time."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


@pytest.fixture(scope="module")
def bench():
    """bench.py, imported without leaving its CUDA module-loading default in
    this process's environment."""
    had = os.environ.get("CUDA_MODULE_LOADING")
    import bench as b

    if had is None:
        os.environ.pop("CUDA_MODULE_LOADING", None)
    return b


def test_traffic_of_every_form_comes_from_the_capture(bench):
    for form in ("f32", "f16", "f16t"):
        traffic, source = bench.bp_traffic(form)
        assert source == bench.TRAFFIC_CAPTURE
        # a launch writes the 1.26 GB volume and reads part of the staged rows
        assert 1.26e9 < traffic < 1.26e9 + 2.56e9, form
    assert bench.bp_traffic("f64")[0] is None


def test_tensor_core_flops_of_the_workload(bench):
    rows, flops = bench.tc_mma_flops()
    assert rows == 256  # every 16 x 8 tile reaches at most two of the ten slabs
    slots = flops / (2 * 2 * 128 * rows * 16)
    tiles = (1024 // 16) * ((300 + 7) // 8) * (1024 // rows)
    # between one and two slabs per (tile, tilt): 1.12 on average
    assert tiles * 61 <= slots <= 2 * tiles * 61
    assert abs(slots / (tiles * 61) - 1.1246) < 1e-3


def test_job_throughput_counts_every_replica(bench):
    one = bench.job_throughput(bench.voxel_tilts(), 10, 1, 80.0)
    assert np.isclose(bench.job_throughput(bench.voxel_tilts(), 10, 4, 80.0), 4 * one)
    assert np.isclose(one, 1024 * 300 * 1024 * 61 * 10 / 80e-3 / 1e9)
