"""Generates tests/golden/*.npz from the reference itself.

The reference's own host code and kernel text, compiled for the CPU by
oracle/build_ref.py (oracle/_ref/libdpm_ref.so), are driven through their
public C++ API (Cell2D/Cell3D constructors, Tissue2D/Tissue3D, Disperse,
CLEulerUpdate) on small seeded cases.  The outputs pin the oracle
restatement and the product's host geometry, and travel with the repository
to machines where the reference tree is absent.

Run: python tests/golden/make_golden.py   (needs oracle/_ref built)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Ref  # noqa: E402


def case2d(R, name, n, nv, r0, calA, Ka, Kl, Kb, phi0, Kre, Kat, seed, steps, dt=0.005,
           spread=1.0):
    rng = np.random.default_rng(seed)
    nv = np.broadcast_to(np.asarray(nv, np.uint32), (n,)).copy()
    r0 = np.broadcast_to(np.asarray(r0, np.float32), (n,)).copy()
    calA = np.broadcast_to(np.asarray(calA, np.float32), (n,)).copy()
    f = lambda v: np.broadcast_to(np.asarray(v, np.float32), (n,)).copy()
    # box of the tissue, then centres uniform in it (the reference's L rule)
    _, _, L = R.run2d(np.zeros(n, np.float32), np.zeros(n, np.float32), calA, nv, r0,
                      f(Ka), f(Kl), f(Kb), phi0=phi0, nsteps=0)
    cen = rng.uniform(0.0, L * spread, size=(n, 2)).astype(np.float32)
    out = dict(nv=nv, r0=r0, calA=calA, Ka=f(Ka), Kl=f(Kl), Kb=f(Kb), x0=cen[:, 0],
               y0=cen[:, 1], phi0=np.float32(phi0), Kre=np.float32(Kre), Kat=np.float32(Kat),
               dt=np.float32(dt))
    x_init, _, L = R.run2d(cen[:, 0], cen[:, 1], calA, nv, r0, f(Ka), f(Kl), f(Kb), phi0=phi0,
                           Kre=Kre, Kat=Kat, nsteps=0)
    out["xy0"] = x_init
    out["L"] = np.float32(L)
    for k in steps:
        xy, F, _ = R.run2d(cen[:, 0], cen[:, 1], calA, nv, r0, f(Ka), f(Kl), f(Kb), phi0=phi0,
                           Kre=Kre, Kat=Kat, nsteps=k, dt=dt)
        out[f"xy_{k}"] = xy
        out[f"F_{k}"] = F
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def main():
    R = Ref()
    # 2D, the 16-cell workload at true packing fraction 0.6 (phi0 = sqrt 0.6)
    case2d(R, "c0_2d", 16, 32, 1.0, 1.0, 1.0, 1.0, 0.0, np.sqrt(0.6), 1.0, 0.0, 0, [1, 100])
    # dense, bending, ragged vertex counts and attraction
    rng = np.random.default_rng(1)
    n = 24
    case2d(R, "ragged_2d", n, rng.choice([16, 24, 32, 48], n), rng.uniform(0.8, 1.4, n),
           rng.uniform(1.0, 1.2, n), 1.0, 1.0, 0.02, np.sqrt(0.85), 1.0, 0.5, 2, [1, 50])
    # geometry of Cell2D
    geo = []
    for nv_, cal, r in [(32, 1.0, 1.0), (25, 1.2, 1.0), (22, 1.2, 1.3), (48, 1.1, 1.4),
                        (16, 1.3, 0.7)]:
        xy, a0, l0, c0 = R.cell2d(0.25, -1.5, cal, nv_, r)
        geo.append((nv_, cal, r, xy, a0, l0, c0))
    np.savez_compressed(os.path.join(HERE, "cell2d.npz"),
                        nv=np.array([g[0] for g in geo], np.uint32),
                        calA=np.array([g[1] for g in geo], np.float32),
                        r0=np.array([g[2] for g in geo], np.float32),
                        xy=np.concatenate([g[3] for g in geo]),
                        a0=np.array([g[4] for g in geo], np.float32),
                        l0=np.array([g[5] for g in geo], np.float32),
                        calA0=np.array([g[6] for g in geo], np.float32))
    # Disperse (drand48 seeded with srand48(seed) before the call)
    nvd = np.full(20, 32, np.uint32)
    rd = np.linspace(0.8, 1.3, 20).astype(np.float32)
    ones = np.ones(20, np.float32)
    xyd, _, Ld = R.run2d(np.zeros(20, np.float32), np.zeros(20, np.float32), ones, nvd, rd, ones,
                         ones, ones * 0, phi0=0.8, disperse=True, seed=7, nsteps=0)
    np.savez_compressed(os.path.join(HERE, "disperse_2d.npz"), nv=nvd, r0=rd, xy=xyd,
                        L=np.float32(Ld), seed=np.int64(7), phi0=np.float32(0.8))
    # 3D: Cell3D geometry and a 5-cell run
    xyz, faces, v0, sa0, a0, vol, sa = R.cell3d([0.5, -0.25, 1.0], 1.05, 1.3)
    np.savez_compressed(os.path.join(HERE, "cell3d.npz"), start=np.float32([0.5, -0.25, 1.0]),
                        calA=np.float32(1.05), r0=np.float32(1.3), xyz=xyz, faces=faces,
                        v0=np.float32(v0), sa0=np.float32(sa0), a0=np.float32(a0),
                        volume=np.float32(vol), surface=np.float32(sa))
    starts = np.array([[0, 0, 1.0], [1.8, 0.2, 1.0], [0.9, 1.6, 1.1], [3.0, 1.5, 0.9],
                       [-1.5, 0.5, 1.0]], np.float32)
    n3 = len(starts)
    c = lambda v: np.full(n3, v, np.float32)
    out = dict(start=starts, calA=c(1.05), r0=c(1.0), Kv=c(1.0), Ka=c(0.5), Ks=c(0.1),
               phi0=np.float32(0.5), Kre=np.float32(1.0), dt=np.float32(0.005))
    for k in (1, 20):
        x3, F3, v3, s3, L3 = R.run3d(starts, c(1.05), c(1.0), c(1.0), c(0.5), c(0.1), phi0=0.5,
                                     Kre=1.0, nsteps=k, dt=0.005)
        out[f"xyz_{k}"] = x3
        out[f"F_{k}"] = F3
        out[f"volume_{k}"] = v3
        out[f"surface_{k}"] = s3
        out["L"] = np.float32(L3)
    np.savez_compressed(os.path.join(HERE, "run_3d.npz"), **out)
    # Disperse2D
    st = np.zeros((6, 3), np.float32)
    o6 = np.ones(6, np.float32)
    x6, _, _, _, L6 = R.run3d(st, o6, o6, o6, o6, o6, phi0=0.35, disperse=True, seed=3,
                              nsteps=0)
    np.savez_compressed(os.path.join(HERE, "disperse_3d.npz"), xyz=x6, L=np.float32(L6),
                        seed=np.int64(3), phi0=np.float32(0.35))
    attraction_case(R, out)
    print("golden vectors written to", HERE)


def attraction_case(R, run3d_out):
    """The reference's AllVertAttraction kernel (never enqueued by its step
    loop) on the 20-step state of run_3d, cells in contact, with the rest
    edge of the reference's 3D tissue as l0."""
    from oracle.oracle import Port
    xyz = run3d_out["xyz_20"]
    n = len(run3d_out["start"])
    _, _, _, _, a0, _, _ = R.cell3d([0.0, 0.0, 0.0], 1.05, 1.0)
    l0 = np.full(n, Port().l0_3d(a0), np.float32)
    L = np.float32(run3d_out["L"])
    Kat = np.float32(0.3)
    F = R.attraction3d(xyz, l0, L, 1, Kat)
    np.savez_compressed(os.path.join(HERE, "attraction_3d.npz"), xyz=xyz, l0=l0, L=L, Kat=Kat,
                        pbc=np.int32(1), F=F)


if __name__ == "__main__":
    main()
