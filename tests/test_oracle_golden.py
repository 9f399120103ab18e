"""The oracle restatement pinned against the reference's own outputs.

tests/golden/*.npz were produced by the reference's host code and kernel
text (tests/golden/make_golden.py); the oracle must reproduce them bit for
bit.  Where the reference build itself is present (oracle/_ref), extra seeded
cases are compared live.
"""
import os

import numpy as np
import pytest

from cases import port
from oracle.oracle import Ref, Tissue2DState, Tissue3DState, ref_available

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def state2d_from_golden(g):
    P = port()
    xs, a0s, l0s, areas = [], [], [], []
    for i in range(len(g["nv"])):
        xy, a0, l0, _ = P.cell2d(g["x0"][i], g["y0"][i], g["calA"][i], int(g["nv"][i]),
                                 g["r0"][i])
        xs.append(xy)
        a0s.append(a0)
        l0s.append(l0)
        areas.append(P.area2d(xy))
    L = P.box2d(areas, float(g["phi0"]))
    return Tissue2DState(nv=g["nv"], xy=np.concatenate(xs), Ka=g["Ka"], Kl=g["Kl"], Kb=g["Kb"],
                         a0=np.array(a0s, np.float32), l0=np.array(l0s, np.float32), r0=g["r0"],
                         L=L, Kre=float(g["Kre"]), Kat=float(g["Kat"]), pbc=1)


@pytest.mark.parametrize("name", ["c0_2d", "ragged_2d"])
def test_2d_runs_bit_exact(name):
    g = load(name)
    s = state2d_from_golden(g)
    assert np.float32(s.L) == g["L"]
    assert np.array_equal(s.xy, g["xy0"])
    steps = sorted(int(k.split("_")[1]) for k in g if k.startswith("xy_"))
    for k in steps:
        t = s.copy()
        F, _ = port().run2d(t, k, float(g["dt"]), nthreads=4)
        assert np.array_equal(t.xy, g[f"xy_{k}"]), f"positions after {k} steps"
        assert np.array_equal(F, g[f"F_{k}"]), f"forces of step {k}"


def test_cell2d_geometry_bit_exact():
    g = load("cell2d")
    off = 0
    for i, nv in enumerate(g["nv"]):
        xy, a0, l0, c0 = port().cell2d(0.25, -1.5, g["calA"][i], int(nv), g["r0"][i])
        assert np.array_equal(xy, g["xy"][off:off + nv])
        assert np.float32(a0) == g["a0"][i] and np.float32(l0) == g["l0"][i]
        assert np.float32(c0) == g["calA0"][i]
        off += nv


def test_cell3d_geometry_bit_exact():
    g = load("cell3d")
    xyz, faces, v0, sa0, a0 = port().cell3d(g["start"], float(g["calA"]), float(g["r0"]), 2)
    assert np.array_equal(xyz, g["xyz"]) and np.array_equal(faces, g["faces"])
    assert np.float32(v0) == g["v0"] and np.float32(sa0) == g["sa0"]
    assert np.float32(a0) == g["a0"]
    assert np.float32(port().volume3d(xyz, faces)) == g["volume"]
    assert np.float32(port().surface3d(xyz, faces)) == g["surface"]


def test_3d_run_bit_exact():
    g = load("run_3d")
    P = port()
    n = len(g["Kv"])
    xs, v0s, a0s = [], [], []
    for i in range(n):
        xyz, faces, v0, sa0, a0 = P.cell3d(g["start"][i], float(g["calA"][i]), float(g["r0"][i]))
        xs.append(xyz)
        v0s.append(v0)
        a0s.append(a0)
    v0s, a0s = np.array(v0s, np.float32), np.array(a0s, np.float32)
    L = P.box3d(v0s, float(g["phi0"]))
    assert np.float32(L) == g["L"]
    l0 = np.array([P.l0_3d(a) for a in a0s], np.float32)
    s = Tissue3DState(nv=len(xs[0]), faces=faces, xyz=np.concatenate(xs), Kv=g["Kv"], Ka=g["Ka"],
                      Ks=g["Ks"], v0=v0s, a0=a0s, l0=l0, L=L, Kre=float(g["Kre"]))
    for k in (1, 20):
        t = s.copy()
        F, _ = P.run3d(t, k, float(g["dt"]), nthreads=4)
        assert np.array_equal(t.xyz, g[f"xyz_{k}"])
        assert np.array_equal(F, g[f"F_{k}"])
        vol = np.array([P.volume3d(t.xyz[i * s.nv:(i + 1) * s.nv], faces) for i in range(n)],
                       np.float32)
        assert np.array_equal(vol, g[f"volume_{k}"])


def test_disperse_bit_exact():
    g = load("disperse_2d")
    xy = port().disperse2d(g["nv"], g["r0"], float(g["L"]), int(g["seed"]))
    assert np.array_equal(xy, g["xy"])
    g3 = load("disperse_3d")
    xs = np.concatenate([port().cell3d([0, 0, 0], 1.0, 1.0)[0] for _ in range(6)])
    x3 = port().disperse3d(xs, 162, np.ones(6, np.float32), float(g3["L"]), int(g3["seed"]))
    assert np.array_equal(x3, g3["xyz"])


def test_analytic_identities():
    # regular polygon: area NV/2 r^2 sin(2 pi/NV); calA=1 -> l0 = 2 r sin(pi/NV)
    P = port()
    for nv, r in [(16, 1.0), (32, 1.4), (100, 2.0)]:
        xy, a0, l0, _ = P.cell2d(0.0, 0.0, 1.0, nv, r)
        assert abs(a0 - nv / 2 * r * r * np.sin(2 * np.pi / nv)) < 1e-5 * a0
        assert abs(l0 - 2 * r * np.sin(np.pi / nv)) < 1e-5 * l0
    # icosphere counts 12/20 -> 42/80 -> 162/320 -> 642/1280
    assert [P.icosphere_counts(k) for k in range(4)] == [(12, 20), (42, 80), (162, 320),
                                                         (642, 1280)]
    # a regular polygon with Kb only: by symmetry the bending force
    # Kb (2 s_i - s_{i-1} - s_{i+1}) has the same magnitude at every vertex
    # and points along the radius, |F| = Kb |s| (2 - 2 cos(2 pi / NV))
    from cases import make_tissue2d
    nv = 32
    s = make_tissue2d(1, nv, Ka=0.0, Kl=0.0, Kb=1.0, phi=0.1, seed=0)
    x0 = s.xy.copy()
    F, _ = P.run2d(s, 1, 0.005)
    mag = np.linalg.norm(F, axis=1)
    th = 2 * np.pi / nv
    side = 2.0 * np.sin(th / 2)
    smag = 2 * side * np.sin(th / 2)
    assert np.allclose(mag, smag * (2 - 2 * np.cos(th)), rtol=1e-3)
    rad = x0 - x0.mean(axis=0)
    cosang = np.sum(F * rad, axis=1) / (mag * np.linalg.norm(rad, axis=1))
    assert np.all(np.abs(np.abs(cosang) - 1) < 1e-4)


@pytest.mark.skipif(not ref_available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("seed", [11, 12])
def test_port_matches_reference_live(seed):
    R = Ref()
    rng = np.random.default_rng(seed)
    n = 12
    nv = rng.choice([16, 24, 32], n).astype(np.uint32)
    r0 = rng.uniform(0.8, 1.3, n).astype(np.float32)
    cal = rng.uniform(1.0, 1.2, n).astype(np.float32)
    one = np.ones(n, np.float32)
    _, _, L = R.run2d(one * 0, one * 0, cal, nv, r0, one, one, one * 0.02, phi0=0.9, nsteps=0)
    c = rng.uniform(0, L, (n, 2)).astype(np.float32)
    xo, fo, L2 = R.run2d(c[:, 0], c[:, 1], cal, nv, r0, one, one, one * 0.02, phi0=0.9,
                         Kre=1.0, Kat=0.3, nsteps=30, dt=0.005)
    g = dict(nv=nv, r0=r0, calA=cal, Ka=one, Kl=one, Kb=one * 0.02, x0=c[:, 0], y0=c[:, 1],
             phi0=np.float32(0.9), Kre=np.float32(1.0), Kat=np.float32(0.3))
    s = state2d_from_golden(g)
    F, _ = port().run2d(s, 30, 0.005)
    assert np.array_equal(s.xy, xo) and np.array_equal(F, fo)


def test_attraction_3d_golden():
    """AllVertAttraction (never enqueued by the reference's step loop): the
    oracle gathers each vertex's pairs in cell and vertex order, the
    reference scatters them with float atomics, so the sums agree to
    rounding (relative 1e-6), term by term the same arithmetic."""
    g = load("attraction_3d")
    F = port().attraction3d(g["xyz"], 162, g["l0"], float(g["L"]), int(g["pbc"]),
                            float(g["Kat"]))
    ref = g["F"]
    assert np.count_nonzero(np.abs(ref).sum(1)) > 100
    assert np.array_equal(np.abs(F).sum(1) == 0, np.abs(ref).sum(1) == 0)
    assert np.linalg.norm(F - ref) <= 1e-6 * np.linalg.norm(ref)


@pytest.mark.skipif(not ref_available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("pbc", [0, 1])
def test_attraction_3d_live(pbc):
    from cases import make_tissue3d
    s = make_tissue3d(6, level=2, phi0=0.5, seed=3)
    l0 = s.l0 * np.float32(1.5)  # a longer range: more pairs
    ref = Ref().attraction3d(s.xyz, l0, s.L, pbc, 0.7)
    F = port().attraction3d(s.xyz, s.nv, l0, s.L, pbc, 0.7)
    assert np.count_nonzero(np.abs(ref).sum(1)) > 100
    assert np.linalg.norm(F - ref) <= 1e-6 * np.linalg.norm(ref)


def test_attraction_in_the_oracle_step():
    """The oracle's 3D step adds AllVertAttraction after the other forces when
    Kat != 0: one step's forces with and without it differ by the
    attraction alone (up to the rounding of adding it to the other terms)."""
    from cases import make_tissue3d
    s = make_tissue3d(5, level=2, phi0=0.5, seed=8)
    s.Kat = 0.5
    on, off = s.copy(), s.copy()
    off.Kat = 0.0
    Fon, _ = port().run3d(on, 1, 0.005)
    Foff, _ = port().run3d(off, 1, 0.005)
    att = port().attraction3d(s.xyz, s.nv, s.l0, s.L, s.pbc, s.Kat)
    assert np.linalg.norm(att) > 0.1 * np.linalg.norm(Foff)
    scale = np.abs(Fon).max()
    assert np.max(np.abs((Fon - Foff) - att)) <= 1e-5 * scale
