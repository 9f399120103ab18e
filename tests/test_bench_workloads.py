"""The benchmark's two arms build the same inputs.

The GPU arm builds its tissues with the product's host model (clDPM); the
reference arm builds them with the oracle and must not load the product at
all.  Both builders must give the same bits, so that the two arms time the
same workload."""
import argparse
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert x.keys() == y.keys()
        for k in x:
            assert np.array_equal(np.asarray(x[k]), np.asarray(y[k])), k


def test_builders_give_the_same_bits():
    import bench
    pg, og = bench.ProductGeometry(), bench.OracleGeometry()
    same(bench.workload_batched(pg, ntissues=24), bench.workload_batched(og, ntissues=24))
    same(bench.workload_c1(pg), bench.workload_c1(og))
    same(bench.workload_c0(pg), bench.workload_c0(og))


def test_reference_arm_loads_no_product():
    code = r"""
import argparse, json, sys
sys.path.insert(0, %r)
import bench
orig = bench.workload_batched
bench.workload_batched = lambda geo, seed=bench.SWEEP_SEED: orig(geo, seed, ntissues=32)
bench.SIM_STEPS = 1
line = bench.run_reference(argparse.Namespace(steps=1, warmup=1, gpus=1))
assert "opencl_dpm_gb300" not in sys.modules, "the reference arm imported the product"
print(json.dumps(line))
""" % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    import json
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["workload"] and line["cpu_baseline"]["kind"] == "port"


def test_roofline_rows_of_the_committed_profile():
    """The bench line's roofline takes the step kernel's DRAM traffic, warp
    instructions per launch and the captured build from the committed ncu
    summary; the rows must parse, and the traffic must be close to the
    algorithmic bytes of one step of the sweep (16 B per vertex and 28 B per
    cell: no re-reads)."""
    import bench
    rows = bench.profile_rows("k2d_step_batched512")
    assert rows["build"] and rows["traffic"] and rows["warp_inst"]
    V, N = 1940768, 66116
    algorithmic = 16.0 * V + 28.0 * N
    assert 0.9 <= rows["traffic"] / algorithmic <= 1.2
    assert 1e7 < rows["warp_inst"] < 1e9


def test_launches_per_call_counts_each_class_and_rebuild():
    """gpu_launches: per rebuild period one bin-preparation, three per radix
    pass and one neighbour-list launch; per simulation step one step launch
    per vertex-slot class."""
    import bench

    class FakeBatch:
        ntissues = 512

        def bins(self):
            return 9, None, None, None

    tissues = [{"nv": np.full(4, nv)} for nv in (16, 24, 32, 48)]
    assert bench.slot_classes(tissues) == 2
    passes = (9 + 9 + 7) // 8
    assert bench.launches_per_call(FakeBatch(), tissues, 32, 32) == (1 + 3 * passes + 1) + 64
