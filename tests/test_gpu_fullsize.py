"""The benchmark's full-size batched workloads, checked through properties
that hold at any size, so that no oracle run of the whole workload is
needed:

* the batched 2D sweep (512 tissues, N ~ U{8..256}, NV in {16, 24, 32, 48}:
  66,116 cells, 1,940,768 vertices) and the batched 3D monolayers (48
  tissues, N ~ U{8..64} cells x 642 vertices);
* a rerun of the same input gives the same bits;
* sampled tissues run alone give the batch's bits (positions and forces);
* from the batch's state after the run, one step of sampled tissues matches
  the oracle: forces within 1e-5 of the oracle's norm, 2D containment flags
  identical.
"""
import numpy as np
import pytest

from cases import port, rel_norm_err

pytestmark = pytest.mark.gpu

F_TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    from opencl_dpm_gb300.abi import Context
    return Context(0)


def tissue_state2d(t, xy):
    from oracle.oracle import Tissue2DState
    return Tissue2DState(nv=t["nv"], xy=np.asarray(xy, np.float32).copy(), Ka=t["Ka"],
                         Kl=t["Kl"], Kb=t["Kb"], a0=t["a0"], l0=t["l0"], r0=t["r0"],
                         L=float(t["L"]), Kre=float(t["Kre"]), Kat=float(t["Kat"]), pbc=1)


def test_sweep_2d_full_size(ctx):
    import bench
    tissues = bench.workload_batched(bench.ProductGeometry(), seed=1000)
    nsteps = 64
    runs = []
    for _ in range(2):
        b, _ = bench.make_batch(ctx, tissues)
        assert b.nverts == 1940768 and b.ncells == 66116
        b.step(nsteps, bench.DT)
        runs.append(b.download())
    (x1, F1), (x2, F2) = runs
    assert np.array_equal(x1, x2) and np.array_equal(F1, F2)
    assert np.all(np.isfinite(x1))

    off = np.concatenate([[0], np.cumsum([len(t["xy"]) for t in tissues])])
    sample = list(range(0, len(tissues), 64)) + [int(np.argmax([len(t["nv"]) for t in tissues]))]
    for t in sample:
        lo, hi = off[t], off[t + 1]
        a, _ = bench.make_batch(ctx, [tissues[t]])
        a.step(nsteps, bench.DT)
        xa, Fa = a.download()
        assert np.array_equal(xa, x1[lo:hi]) and np.array_equal(Fa, F1[lo:hi]), t

        # one step from the batch's state, against the oracle
        s = tissue_state2d(tissues[t], x1[lo:hi])
        a.upload(s.xy)
        a.step(1, bench.DT)
        _, F = a.download()
        flags = a.contained()
        rF, rflags = port().run2d(s, 1, bench.DT)
        assert rel_norm_err(F, rF) <= F_TOL, t
        assert np.array_equal(flags, rflags), t


def test_monolayers_3d_full_size(ctx):
    import bench
    from opencl_dpm_gb300 import clDPM
    from opencl_dpm_gb300.abi import Batch3D
    from oracle.oracle import Tissue3DState
    rng = np.random.default_rng(5)
    ts = [bench.build_monolayer(clDPM, rng, int(rng.integers(8, 65)), 3) for _ in range(48)]
    nsteps = 16

    def batch(group):
        cat = lambda k: np.concatenate([t[k] for t in group])
        b = Batch3D(ctx, [len(t["Kv"]) for t in group], group[0]["faces"], group[0]["nv"])
        b.set_cells(cat("Kv"), cat("Ka"), cat("Ks"), cat("v0"), cat("a0"), cat("l0"),
                    cat("Kb"), cat("adh"))
        b.set_tissues([t["L"] for t in group], [1.0] * len(group), [1] * len(group))
        b.upload(cat("xyz"))
        return b

    runs = []
    for _ in range(2):
        b = batch(ts)
        b.step(nsteps, bench.DT3)
        runs.append(b.download())
    (x1, F1), (x2, F2) = runs
    assert np.array_equal(x1, x2) and np.array_equal(F1, F2)
    assert np.all(np.isfinite(x1))

    off = np.concatenate([[0], np.cumsum([len(t["xyz"]) for t in ts])])
    # the oracle's repulsion is all pairs: its step is checked on the two
    # smallest monolayers, the bits on those and three more
    small = sorted(range(len(ts)), key=lambda t: len(ts[t]["Kv"]))[:2]
    for t in [0, 17, 47] + small:
        lo, hi = off[t], off[t + 1]
        a = batch([ts[t]])
        a.step(nsteps, bench.DT3)
        xa, Fa = a.download()
        assert np.array_equal(xa, x1[lo:hi]) and np.array_equal(Fa, F1[lo:hi]), t
        if t not in small:
            continue

        m = ts[t]
        s = Tissue3DState(nv=m["nv"], faces=m["faces"], xyz=x1[lo:hi].copy(), Kv=m["Kv"],
                          Ka=m["Ka"], Ks=m["Ks"], v0=m["v0"], a0=m["a0"], l0=m["l0"],
                          L=float(m["L"]), Kre=1.0, pbc=1, Kb=m["Kb"], adh=m["adh"])
        a.upload(s.xyz)
        a.step(1, bench.DT3)
        _, F = a.download()
        rF, _ = port().run3d(s, 1, bench.DT3)
        assert rel_norm_err(F, rF) <= F_TOL, t
