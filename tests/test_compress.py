"""The compression protocol of the 2D jamming workload (1,024 bidisperse
cells compressed from packing fraction 0.6 to 0.85 in steps of 0.002 with
500 relaxation steps per stage).

The reference fixes the box at construction (src/Tissue2D.cpp:31), so the
box update is an extension: the host Tissue2D.SetPackingFraction and the
device dpm2d_set_packing_fraction.  Both must give the bits of the numpy
restatement `cases.rescale_packing`.  A compression run is chaotic, so the
GPU run is compared with the oracle's run of the same protocol through
ensemble statistics over seeds (packing fraction, shape index, energy)."""
import numpy as np
import pytest

from cases import gpu_batch2d, make_tissue2d, perturb, port, rescale_packing
from ensemble import compare_ensembles

DT = 0.005


def bidisperse(n, seed, phi=0.6, nv=32):
    """n cells, half r0 = 1.0 and half r0 = 1.4 (shuffled), calA0 ~ U[1, 1.2],
    kb = 0.01, at seeded uniform centres in the box of true packing fraction
    phi."""
    rng = np.random.default_rng(seed)
    r0 = rng.permutation(np.r_[np.full(n // 2, 1.0), np.full(n - n // 2, 1.4)])
    calA = rng.uniform(1.0, 1.2, n)
    return make_tissue2d(n, nv, r0=r0, calA=calA, Kb=0.01, phi=phi, seed=seed + 1000)


def test_rescale_restatement_matches_host_class():
    from opencl_dpm_gb300 import clDPM
    s = perturb(bidisperse(12, 3), 0.05, 1)
    cells = []
    for c in range(len(s.nv)):
        o = int(s.off[c])
        cell = clDPM.Cell2D(0.0, 0.0, 1.0, int(s.nv[c]), float(s.r0[c]))
        cell.Verts = s.xy[o:o + int(s.nv[c])].tolist()
        cells.append(cell)
    T = clDPM.Tissue2D(cells, 1.0)
    s.L = float(T.L)
    for phi in (0.62, 0.71, 0.5):
        T.SetPackingFraction(phi)
        s = rescale_packing(s, phi)
        got = np.concatenate([np.asarray(c.Verts, np.float32) for c in T.Cells])
        assert np.float32(T.L) == np.float32(s.L)
        assert np.array_equal(got, s.xy)


@pytest.mark.gpu
def test_device_rescale_bit_exact():
    from opencl_dpm_gb300.abi import Context
    ctx = Context(0)
    states = [perturb(bidisperse(n, 10 + n), 0.03, n) for n in (9, 40, 17)]
    states.append(perturb(make_tissue2d(11, 24, calA=1.1, phi=0.7, seed=4), 0.02, 5))
    b = gpu_batch2d(ctx, states)
    phis = [0.652, 0.0, 0.8, 0.55]
    b.set_packing_fraction(phis)
    xy, _ = b.download()
    exp = [rescale_packing(s, p) if p > 0 else s for s, p in zip(states, phis)]
    assert np.array_equal(xy, np.concatenate([e.xy for e in exp]))
    d = b.diagnostics()
    for t, (e, p) in enumerate(zip(exp, phis)):
        if p > 0:
            assert abs(d["packing_fraction"][t] - p) < 1e-5
    # the rescaled batch steps on like one built at the new box directly
    b.step(40, DT)
    b2 = gpu_batch2d(ctx, exp)
    b2.step(40, DT)
    x1, f1 = b.download()
    x2, f2 = b2.download()
    assert np.array_equal(x1, x2) and np.array_equal(f1, f2)
    with pytest.raises(Exception):
        b.set_packing_fraction([0.5, -1.0, 0.5, 0.5])


def compress(stages, relax, phi0, dphi, gpu=None, oracle_state=None):
    """Runs the protocol: at each stage the box goes to phi0 + k*dphi, then
    `relax` steps.  gpu: a Batch2D (all its tissues together); oracle_state:
    a Tissue2DState stepped by the oracle."""
    for k in range(1, stages + 1):
        phi = phi0 + k * dphi
        if gpu is not None:
            gpu.set_packing_fraction(phi)
            gpu.step(relax, DT)
        else:
            oracle_state = rescale_packing(oracle_state, phi)
            port().run2d(oracle_state, relax, DT)
    return oracle_state


@pytest.mark.gpu
def test_compression_ensemble_matches_oracle():
    """16 seeds of a reduced compression: 32 bidisperse cells, packing
    fraction 0.6 -> 0.75 in steps of 0.002, 50 relaxation steps each (3,750
    steps).  Ensemble means of packing fraction, shape index and energy on
    the GPU and on the oracle agree within the tolerance of `ensemble`."""
    from opencl_dpm_gb300.abi import Context
    ctx = Context(0)
    seeds = range(16)
    states = [bidisperse(32, 200 + k) for k in seeds]
    b = gpu_batch2d(ctx, states)
    compress(75, 50, 0.6, 0.002, gpu=b)
    d = b.diagnostics()
    gpu_stats = {"packing_fraction": d["packing_fraction"], "shape_index": d["shape_index"],
                 "energy": np.add.reduceat(d["energy"], np.arange(0, 32 * len(states), 32)) / 32}
    orc = {"packing_fraction": [], "shape_index": [], "energy": []}
    for s in states:
        r = compress(75, 50, 0.6, 0.002, oracle_state=s.copy())
        a, p, e = port().diag2d(r)
        orc["packing_fraction"].append(a.sum() / (r.L * r.L))
        orc["shape_index"].append(np.mean(p / np.sqrt(4 * np.pi * a)))
        orc["energy"].append(np.mean(e))
    report = compare_ensembles(gpu_stats, orc)
    assert report["ok"], report
    # the box reached the protocol's last stage; the cells' areas shrink
    # under the compression, so sum(A)/L^2 ends a few percent below it
    assert np.all((d["packing_fraction"] > 0.65) & (d["packing_fraction"] < 0.76))
