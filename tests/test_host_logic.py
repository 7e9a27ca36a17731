"""Host-side logic without a GPU: the seeded benchmark workloads (the shapes
and value ranges the benchmark configurations are quoted on, identical on
every run) and the reference arm's JSON line (the oracle on the host cores)."""
import json
import os
import sys
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "cuda-sipg-matrix-free_gb300"))
sys.path.insert(0, ROOT)

import workloads  # noqa: E402


def test_workloads_are_deterministic_in_their_seed():
    assert workloads.request_stream(count=50, seed=3) == workloads.request_stream(count=50, seed=3)
    assert workloads.request_stream(count=50, seed=3) != workloads.request_stream(count=50, seed=4)
    assert workloads.uneven_problems(count=20, seed=2) == workloads.uneven_problems(count=20, seed=2)
    assert workloads.shared_mesh_rhs(count=8, seed=1) == workloads.shared_mesh_rhs(count=8, seed=1)


def test_request_stream_ranges():
    reqs = workloads.request_stream(count=2000, rate=5.0, seed=3)
    t = np.array([r[0] for r in reqs])
    assert np.all(np.diff(t) >= 0) and t[0] >= 0  # Poisson arrivals in order
    assert abs(len(t) / t[-1] - 5.0) < 0.5  # the requested rate
    for _, dim, p, pen, modes, tol in reqs:
        assert 8 <= dim <= 512 and 2 <= p <= 8 and pen == float(p * p)
        assert tol in (1e-8, 1e-10)
        amps, ks, ls = modes
        assert len(amps) == len(ks) == len(ls) == 4 and all(1 <= k <= 8 for k in ks + ls)


def test_shared_mesh_and_uneven_batches():
    a = workloads.shared_mesh_rhs(count=64, dim=256, degree=4, seed=1)
    assert len(a) == 64 and all(r[0] == 256 and r[1] == 4 for r in a)
    assert sum(workloads.ndof(r[0], r[1]) for r in a) == 64 * 1638400  # 104.9 M DoF in all
    b = workloads.uneven_problems(count=200, seed=2)
    assert len(b) == 200 and all(16 <= r[0] <= 256 and 2 <= r[1] <= 8 for r in b)


def test_reference_arm_line_keys(capsys):
    # the reference arm: the oracle's apply of the 1024^2, p = 4 workload on
    # the host cores, one JSON line with the keys the benchmark contract names
    import bench

    args = types.SimpleNamespace(steps=1, warmup=0, gpus=1)
    for var in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(var, None)
    assert bench.run_reference(args) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GDoF/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "GDoF/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["metric"] == bench.METRIC and line["higher_is_better"] is True
