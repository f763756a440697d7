"""Host-side logic of bench.py without a GPU: the roofline figure of the
dominant kernel group (algorithmic bytes x launches that did work / event
time, against the measured peak, DRAM traffic scaled per cell) and the
parsing of a GPU's local CPU list."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_roofline_of_the_vcycle_group(monkeypatch):
    monkeypatch.setattr(bench, "measured_peaks", lambda: (6800.0, "measured"))
    N = 192 ** 3
    res = {"precision": "mixed", "N": N,
           "stats": [{"pressure_iterations": 40, "velocity_sweeps": 59}] * 5,
           # group -> (launches that ran, total ms); the V-cycle dominates
           "prof": {"mg_vcycle": (200, 92.0), "cg_spmv": (200, 15.0), "mom_sweep": (800, 35.0)}}
    r = bench.roofline(res)
    per_cell = bench.ALG_BYTES_PER_CELL_FP32["mg_vcycle"]
    assert r["kernel"] == "mg_vcycle" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["bytes_per_launch"] == per_cell * N
    achieved = per_cell * N * 200 / 0.092 / 1e9
    assert abs(r["achieved"] - achieved) < 0.1
    assert abs(r["frac"] - achieved / 6800.0) < 1e-4
    assert abs(r["avg_launch_us"] - 460.0) < 1e-6
    assert r["traffic"] == round(bench.TRAFFIC_PER_CELL["mg_vcycle"] * N)


def test_roofline_counts_sweeps_and_iterations(monkeypatch):
    monkeypatch.setattr(bench, "measured_peaks", lambda: (6800.0, "measured"))
    res = {"precision": "fp64", "N": 1000,
           "stats": [{"pressure_iterations": 7, "velocity_sweeps": 3}] * 2,
           "prof": {"cg_spmv": (30, 10.0)}}
    r = bench.roofline(res)
    # queued launches past convergence do not count: the iterations do
    assert r["effective_launches"] == 14 and r["launches"] == 30


def test_gpu_local_cpus_without_a_device():
    import pytest
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        cpus = bench.gpu_local_cpus(0)
        assert cpus is None or (cpus and all(isinstance(c, int) for c in cpus))
    else:
        # no CUDA device: the helper says it does not know
        assert bench.gpu_local_cpus(0) is None
