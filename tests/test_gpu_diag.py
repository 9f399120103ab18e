"""Device diagnostics (dpm2d_diagnostics, dpm3d_diagnostics) against the
oracle's FP64 host diagnostics, and the ensemble statistics of long runs.

Diagnostics are computed in double from the same float positions on both
sides; only the summation order differs (relative tolerance 1e-9).  Long
runs are judged by ensemble statistics over seeds -- packing fraction, mean
shape index P/sqrt(4 pi A) and mean energy -- because trajectories that
differ by float rounding drift apart (tolerance in tests/ensemble.py)."""
import numpy as np
import pytest

from cases import gpu_batch2d, gpu_batch3d, make_tissue2d, make_tissue3d, perturb, port

pytestmark = pytest.mark.gpu

DT = 0.005


@pytest.fixture(scope="module")
def ctx():
    from opencl_dpm_gb300.abi import Context
    return Context(0)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-12)))


def test_diag2d_matches_oracle(ctx):
    states = [perturb(make_tissue2d(n, nv, calA=1.15, Kb=kb, phi=0.8, seed=50 + n), 0.02, n)
              for n, nv, kb in ((12, 16, 0.0), (30, 32, 0.05), (7, 48, 0.01))]
    b = gpu_batch2d(ctx, states)
    d = b.diagnostics()
    off = 0
    for t, s in enumerate(states):
        a, p, e = port().diag2d(s)
        n = len(s.nv)
        assert rel(d["area"][off:off + n], a) <= 1e-9
        assert rel(d["perimeter"][off:off + n], p) <= 1e-9
        assert rel(d["energy"][off:off + n], e) <= 1e-9
        assert rel(d["packing_fraction"][t], a.sum() / (s.L * s.L)) <= 1e-9
        assert rel(d["shape_index"][t], np.mean(p / np.sqrt(4 * np.pi * a))) <= 1e-9
        off += n


def test_diag3d_matches_oracle(ctx):
    for kb in (None, 0.05):
        s = make_tissue3d(5, level=2, phi0=0.5, seed=8, Kb=kb)
        s.xyz[:, 2] *= np.float32(0.93)  # off the sphere: non-zero strains and bending
        b = gpu_batch3d(ctx, [s])
        d = b.diagnostics()
        v, a, e = port().diag3d(s)
        assert rel(d["volume"], v) <= 1e-9
        assert rel(d["surface_area"], a) <= 1e-9
        assert rel(d["energy"], e) <= 1e-9


def test_ensemble_statistics_c0(ctx):
    """The plain 2D workload's long run as an ensemble: 16 seeds of 16 cells
    x 32 vertices (calA0 = 1, ka = kl = kc = 1, kb = 0, packing fraction 0.6,
    dt = 0.005) for its full 10,000 steps, all seeds in one batch on the GPU
    and one by one on the oracle.  Ensemble means of packing fraction, shape
    index and energy agree within four standard errors of the paired
    difference plus 1e-3 relative (tests/ensemble.py)."""
    from ensemble import compare_ensembles
    states = [make_tissue2d(16, 32, calA=1.0, Kb=0.0, phi=0.6, seed=300 + k) for k in range(16)]
    b = gpu_batch2d(ctx, states)
    b.step(10000, DT)
    d = b.diagnostics()
    gpu = {"packing_fraction": d["packing_fraction"], "shape_index": d["shape_index"],
           "energy": d["energy"].reshape(16, 16).mean(axis=1)}
    orc = {"packing_fraction": [], "shape_index": [], "energy": []}
    for s in states:
        r = s.copy()
        port().run2d(r, 10000, DT)
        a, p, e = port().diag2d(r)
        orc["packing_fraction"].append(a.sum() / (r.L * r.L))
        orc["shape_index"].append(np.mean(p / np.sqrt(4 * np.pi * a)))
        orc["energy"].append(np.mean(e))
    report = compare_ensembles(gpu, orc)
    assert report["ok"], report
