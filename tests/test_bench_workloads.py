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
