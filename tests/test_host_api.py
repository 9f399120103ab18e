"""The clDPM module: the reference's Python API over the GB300 library.

CPU tests pin the host model (geometry, box size, dispersion) bit for bit to
the reference's own outputs (tests/golden); GPU tests step tissues through
Tissue2D/Tissue3D.CLEulerUpdate and compare with the same golden runs.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


@pytest.fixture(scope="module")
def clDPM():
    from opencl_dpm_gb300 import clDPM as m
    return m


def test_api_surface(clDPM):
    c = clDPM.Cell2D(0.0, 0.0, 1.0, 32, 1.0)
    for a in ("Ka", "Kl", "Kb", "Verts", "Forces"):
        assert hasattr(c, a)
    t = clDPM.Tissue2D([c, c], 0.8)
    for a in ("Cells", "NCELLS", "L", "PBC", "Kre", "Kat", "CLEulerUpdate", "Disperse"):
        assert hasattr(t, a)
    c3 = clDPM.Cell3D([0.0, 0.0, 0.0], 1.0, 1.0)
    for a in ("Kv", "Ka", "Ks", "Verts", "GetVolume", "GetPositions", "GetVesselPositions",
              "GetFaces", "GetForces"):
        assert hasattr(c3, a)
    t3 = clDPM.Tissue3D([c3], 0.5)
    for a in ("Kre", "Kat", "Cells", "NCELLS", "L", "PBC", "CLEulerUpdate", "Disperse2D"):
        assert hasattr(t3, a)
    assert len(c3.GetPositions()) == 3 and len(c3.GetPositions()[0]) == 162
    assert len(c3.GetFaces()) == 320
    # read-only attributes stay read-only
    with pytest.raises(AttributeError):
        t.L = 3.0
    with pytest.raises(AttributeError):
        t3.NCELLS = 2


def test_cell2d_geometry(clDPM):
    g = load("cell2d")
    off = 0
    for i, nv in enumerate(g["nv"]):
        c = clDPM.Cell2D(0.25, -1.5, float(g["calA"][i]), int(nv), float(g["r0"][i]))
        assert np.array_equal(np.array(c.Verts, np.float32), g["xy"][off:off + nv])
        assert np.float32(c.a0) == g["a0"][i] and np.float32(c.l0) == g["l0"][i]
        assert np.float32(c.calA0) == g["calA0"][i]
        off += nv


def test_cell3d_geometry(clDPM):
    g = load("cell3d")
    c = clDPM.Cell3D(list(map(float, g["start"])), float(g["calA"]), float(g["r0"]))
    assert np.array_equal(np.array(c.Verts, np.float32), g["xyz"])
    assert np.array_equal(np.array(c.GetFaces(), np.uint32), g["faces"])
    assert np.float32(c.v0) == g["v0"] and np.float32(c.a0) == g["a0"]
    assert np.float32(c.GetVolume()) == g["volume"]
    assert np.float32(c.GetSurfaceArea()) == g["surface"]
    c3 = clDPM.Cell3D([0.0, 0.0, 0.0], 1.0, 1.0, 3)
    assert c3.NV == 642 and c3.NF == 1280


def tissue2d_from_golden(clDPM, g):
    cells = []
    for i in range(len(g["nv"])):
        c = clDPM.Cell2D(float(g["x0"][i]), float(g["y0"][i]), float(g["calA"][i]),
                         int(g["nv"][i]), float(g["r0"][i]))
        c.Ka, c.Kl, c.Kb = float(g["Ka"][i]), float(g["Kl"][i]), float(g["Kb"][i])
        cells.append(c)
    T = clDPM.Tissue2D(cells, float(g["phi0"]))
    T.Kre = float(g["Kre"])
    T.Kat = float(g["Kat"])
    return T


def test_tissue2d_box(clDPM):
    g = load("c0_2d")
    T = tissue2d_from_golden(clDPM, g)
    assert np.float32(T.L) == g["L"] and T.NCELLS == 16 and T.PBC


def check_disperse(clDPM, device):
    g = load("disperse_2d")
    cells = [clDPM.Cell2D(0.0, 0.0, 1.0, int(nv), float(r)) for nv, r in zip(g["nv"], g["r0"])]
    T = clDPM.Tissue2D(cells, float(g["phi0"]))
    assert np.float32(T.L) == g["L"]
    clDPM.srand48(int(g["seed"]))
    T.Disperse(device=device)
    xy = np.concatenate([np.array(c.Verts, np.float32) for c in T.Cells])
    assert np.array_equal(xy, g["xy"])
    g3 = load("disperse_3d")
    c3 = [clDPM.Cell3D([0.0, 0.0, 0.0], 1.0, 1.0) for _ in range(6)]
    T3 = clDPM.Tissue3D(c3, float(g3["phi0"]))
    assert np.float32(T3.L) == g3["L"]
    clDPM.srand48(int(g3["seed"]))
    T3.Disperse2D(device=device)
    x3 = np.concatenate([np.array(c.Verts, np.float32) for c in T3.Cells])
    assert np.array_equal(x3, g3["xyz"])


def test_disperse_host(clDPM):
    """The host loop reproduces the reference build's dispersion bit for bit."""
    check_disperse(clDPM, device=False)


@pytest.mark.gpu
def test_disperse_device(clDPM):
    """The device relaxation reproduces the same bits."""
    check_disperse(clDPM, device=True)


@pytest.mark.gpu
def test_disperse_device_batched(clDPM):
    """Many systems in one launch, each equal to the host loop; sizes span
    the list overflow (dense) and the skin rebuilds (sparse)."""
    from opencl_dpm_gb300.abi import Context, disperse
    rng = np.random.default_rng(9)
    systems = []
    for n in (1, 2, 17, 64, 200):
        r = rng.choice([1.0, 1.4], n).astype(np.float32)
        # box for true packing fraction phi: L = sqrt(sum pi r^2 / phi)
        L = np.float32(np.sqrt(np.sum(np.pi * r.astype(np.float64) ** 2) / rng.uniform(0.3, 0.9)))
        systems.append((r, L, 1000 + n))
    X0, Y0 = [], []
    for r, L, seed in systems:
        x, y = clDPM.drand48_centres(seed, len(r), float(L))
        X0.append(np.asarray(x, np.float32))
        Y0.append(np.asarray(y, np.float32))
    ctx = Context(0)
    X, Y, it = disperse(ctx, [len(s[0]) for s in systems], np.concatenate([s[0] for s in systems]),
                        [s[1] for s in systems], np.concatenate(X0), np.concatenate(Y0))
    off = 0
    for (r, L, seed), k in zip(systems, it):
        n = len(r)
        hx, hy, hk = clDPM.relax_centres(list(map(float, r)), float(L), seed, False)
        assert np.array_equal(X[off:off + n], np.asarray(hx, np.float32))
        assert np.array_equal(Y[off:off + n], np.asarray(hy, np.float32))
        assert k == hk
        off += n


def test_tissue3d_validation(clDPM):
    c = clDPM.Cell3D([0.0, 0.0, 1.0], 1.0, 1.0)
    c.Kv, c.Ka, c.Ks = 1.0, 1.0, 1.0
    T = clDPM.Tissue3D([c], 0.5)
    with pytest.raises(ValueError):
        T.CLEulerUpdate(0, 0.01)
    with pytest.raises(ValueError):
        T.CLEulerUpdate(1, 0.5)
    c.Ks = 0.0
    T = clDPM.Tissue3D([c], 0.5)
    with pytest.raises(RuntimeError):
        T.CLEulerUpdate(1, 0.01)


def test_packing_fraction_extension(clDPM):
    cells = [clDPM.Cell2D(float(x), float(y), 1.0, 32, 1.0) for x, y in [(1, 1), (4, 2), (2, 5)]]
    T = clDPM.Tissue2D(cells, 0.8)
    T.SetPackingFraction(0.7)
    assert abs(T.GetPackingFraction() - 0.7) < 1e-5
    si = T.GetShapeIndices()
    assert len(si) == 3 and all(1.0 < s < 1.01 for s in si)


@pytest.mark.gpu
def test_tissue2d_steps_match_reference(clDPM):
    g = load("c0_2d")
    for k in (1, 100):
        T = tissue2d_from_golden(clDPM, g)
        T.CLEulerUpdate(k, float(g["dt"]))
        xy = np.concatenate([np.array(c.Verts, np.float32) for c in T.Cells])
        F = np.concatenate([np.array(c.Forces, np.float32) for c in T.Cells])
        ref = g[f"xy_{k}"]
        assert np.max(np.abs(xy - ref) / np.maximum(np.abs(ref), 1.0)) <= 1e-4
        if k == 1:
            rF = g["F_1"]
            assert np.linalg.norm(F - rF) <= 1e-5 * np.linalg.norm(rF)


@pytest.mark.gpu
def test_tissue2d_repeated_calls(clDPM):
    # k calls of n steps == one call of k*n steps (state lives in Cells)
    g = load("ragged_2d")
    T1 = tissue2d_from_golden(clDPM, g)
    for _ in range(5):
        T1.CLEulerUpdate(10, float(g["dt"]))
    xy = np.concatenate([np.array(c.Verts, np.float32) for c in T1.Cells])
    ref = g["xy_50"]
    assert np.max(np.abs(xy - ref) / np.maximum(np.abs(ref), 1.0)) <= 1e-4


@pytest.mark.gpu
def test_tissue3d_steps_match_reference(clDPM):
    g = load("run_3d")
    for k in (1, 20):
        cells = []
        for i in range(len(g["Kv"])):
            c = clDPM.Cell3D(list(map(float, g["start"][i])), float(g["calA"][i]),
                             float(g["r0"][i]))
            c.Kv, c.Ka, c.Ks = float(g["Kv"][i]), float(g["Ka"][i]), float(g["Ks"][i])
            cells.append(c)
        T = clDPM.Tissue3D(cells, float(g["phi0"]))
        T.Kre = float(g["Kre"])
        T.CLEulerUpdate(k, float(g["dt"]))
        x = np.concatenate([np.array(c.Verts, np.float32) for c in T.Cells])
        ref = g[f"xyz_{k}"]
        assert np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1.0)) <= 1e-4
        if k == 1:
            F = np.concatenate([np.array(c.GetForces(), np.float32).T for c in T.Cells])
            rF = g["F_1"]
            assert np.linalg.norm(F - rF) <= 1e-5 * np.linalg.norm(rF)
