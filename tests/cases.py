"""Seeded tissue builders and comparison helpers shared by the tests.

Inputs are synthetic and seeded (numpy PCG64); they follow the shapes of the
workloads the library is measured on: regular polygons of radius r0 placed
uniformly in a periodic box sized for a packing fraction, the box side from
the reference's rule L = sqrt(sum of areas) / phi0 with phi0 = sqrt(phi) so
that the true packing fraction is phi.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle.oracle import Port, Tissue2DState, Tissue3DState  # noqa: E402

_port = None


def port() -> Port:
    global _port
    if _port is None:
        _port = Port()
    return _port


def make_tissue2d(ncells=16, nv=32, r0=1.0, calA=1.0, Ka=1.0, Kl=1.0, Kb=0.0, phi=0.6,
                  Kre=1.0, Kat=0.0, seed=0, centers=None, pbc=1) -> Tissue2DState:
    """Regular polygons (Cell2D ctor geometry) at seeded uniform centres."""
    P = port()
    rng = np.random.default_rng(seed)
    nv = np.broadcast_to(np.asarray(nv, dtype=np.uint32), (ncells,)).copy()
    r0 = np.broadcast_to(np.asarray(r0, dtype=np.float32), (ncells,)).copy()
    calA = np.broadcast_to(np.asarray(calA, dtype=np.float32), (ncells,)).copy()
    xs, a0s, l0s, areas = [], [], [], []
    for i in range(ncells):
        xy, a0, l0, _ = P.cell2d(0.0, 0.0, float(calA[i]), int(nv[i]), float(r0[i]))
        xs.append(xy)
        a0s.append(a0)
        l0s.append(l0)
        areas.append(P.area2d(xy))
    phi0 = float(np.sqrt(phi))
    L = P.box2d(areas, phi0)
    if centers is None:
        centers = rng.uniform(0.0, L, size=(ncells, 2)).astype(np.float32)
    xy = np.concatenate([xs[i] + centers[i].astype(np.float32) for i in range(ncells)])
    f = lambda v: np.broadcast_to(np.asarray(v, dtype=np.float32), (ncells,)).copy()
    return Tissue2DState(nv=nv, xy=xy.astype(np.float32), Ka=f(Ka), Kl=f(Kl), Kb=f(Kb),
                         a0=np.array(a0s, np.float32), l0=np.array(l0s, np.float32), r0=r0,
                         L=float(L), Kre=float(Kre), Kat=float(Kat), pbc=pbc)


def rescale_packing(state: Tissue2DState, phi: float) -> Tissue2DState:
    """The host Tissue2D.SetPackingFraction restated with numpy, operation by
    operation (float32 where it rounds to float, float64 where it promotes):
    per cell the float shoelace area with a double accumulator, summed in
    double in cell order; L' = sqrt(sum / phi); each cell shifted by its
    double vertex-mean centroid times (L'/L - 1).  Returns a new state."""
    s = state.copy()
    f32, f64 = np.float32, np.float64
    off = s.off
    nv = s.nv.astype(np.int64)
    xy = s.xy.astype(f32)
    areas = np.zeros(len(nv), f32)
    cents = np.zeros((len(nv), 2), f64)
    for n in np.unique(nv):
        cells = np.nonzero(nv == n)[0]
        idx = off[cells][:, None].astype(np.int64) + np.arange(n)[None, :]
        x, y = xy[idx, 0], xy[idx, 1]
        a = np.zeros(len(cells), f32)
        j = n - 1
        for i in range(n):
            sm = x[:, j] + x[:, i]
            d = y[:, j] - y[:, i]
            a = (a.astype(f64) + 0.5 * (sm * d).astype(f64)).astype(f32)
            j = i
        areas[cells] = np.abs(a)
        # sequential double sums over each ring (accumulate is in order)
        cents[cells, 0] = np.add.accumulate(x.astype(f64), axis=1)[:, -1] / f64(n)
        cents[cells, 1] = np.add.accumulate(y.astype(f64), axis=1)[:, -1] / f64(n)
    total = float(np.add.accumulate(areas.astype(f64))[-1])
    Lnew = np.sqrt(total / f64(f32(phi)))
    sm1 = Lnew / f64(f32(s.L)) - 1.0
    shift = cents * sm1
    rep = np.repeat(shift, nv, axis=0)
    s.xy = (xy.astype(f64) + rep).astype(f32)
    s.L = float(f32(Lnew))
    return s


def perturb(state: Tissue2DState, scale: float, seed: int) -> Tissue2DState:
    s = state.copy()
    rng = np.random.default_rng(seed)
    s.xy = (s.xy + rng.normal(0.0, scale, size=s.xy.shape)).astype(np.float32)
    return s


def rel_norm_err(a, b, floor=0.0) -> float:
    """||a - b|| / max(||b||, floor)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = max(np.linalg.norm(b), floor, 1e-30)
    return float(np.linalg.norm(a - b) / den)


def make_tissue3d(ncells=4, level=2, r0=1.0, calA=1.05, Kv=1.0, Ka=0.5, Ks=0.1, Kre=1.0,
                  phi0=0.5, seed=0, Kb=None, adh=None, centers=None, pbc=1) -> Tissue3DState:
    """Icospheres (Cell3D ctor geometry) resting on z = 0 (centres at z = r0),
    seeded uniform x, y in the reference's box L = cbrt(sum v0) / phi0."""
    P = port()
    rng = np.random.default_rng(seed)
    xyz0, faces, v0, sa0, a0 = P.cell3d([0.0, 0.0, 0.0], calA, r0, level)
    nv = len(xyz0)
    v0s = np.full(ncells, v0, np.float32)
    L = P.box3d(v0s, phi0)
    if centers is None:
        centers = np.column_stack([rng.uniform(0.0, L, size=(ncells, 2)),
                                   np.full(ncells, r0)]).astype(np.float32)
    xyz = np.concatenate([P.cell3d(centers[i], calA, r0, level)[0] for i in range(ncells)])
    f = lambda v: np.broadcast_to(np.asarray(v, dtype=np.float32), (ncells,)).copy()
    a0s = f(a0)
    l0s = np.array([P.l0_3d(x) for x in a0s], np.float32)
    return Tissue3DState(nv=nv, faces=faces, xyz=xyz.astype(np.float32), Kv=f(Kv), Ka=f(Ka),
                         Ks=f(Ks), v0=v0s, a0=a0s, l0=l0s, L=float(L), Kre=float(Kre), pbc=pbc,
                         Kb=None if Kb is None else f(Kb), adh=None if adh is None else f(adh))


def gpu_batch3d(ctx, states, tuning=None):
    """A Batch3D (C ABI) holding the given 3D tissues (one mesh), uploaded."""
    from opencl_dpm_gb300.abi import Batch3D
    s0 = states[0]
    b = Batch3D(ctx, [s.ncells for s in states], s0.faces, s0.nv)
    cat = lambda k: np.concatenate([getattr(s, k) for s in states])
    kb = None
    if any(s.Kb is not None for s in states):
        kb = np.concatenate([s.Kb if s.Kb is not None else np.zeros(s.ncells, np.float32)
                             for s in states])
    adh = None
    if any(s.adh is not None for s in states):
        adh = np.concatenate([s.adh if s.adh is not None else 2.0 * s.l0 for s in states])
    b.set_cells(cat("Kv"), cat("Ka"), cat("Ks"), cat("v0"), cat("a0"), cat("l0"), kb, adh)
    b.set_tissues([s.L for s in states], [s.Kre for s in states], [s.pbc for s in states])
    if any(s.Kat != 0.0 for s in states):
        b.set_attraction([s.Kat for s in states])
    if tuning:
        b.set_tuning(**tuning)
    b.upload(np.concatenate([s.xyz for s in states]))
    return b


def gpu_batch2d(ctx, states, tuning=None):
    """A Batch2D (C ABI) holding the given tissues, uploaded."""
    from opencl_dpm_gb300.abi import Batch2D
    ncells = [len(s.nv) for s in states]
    nv = np.concatenate([s.nv for s in states])
    b = Batch2D(ctx, ncells, nv)
    cat = lambda k: np.concatenate([getattr(s, k) for s in states])
    b.set_cells(cat("Ka"), cat("Kl"), cat("Kb"), cat("a0"), cat("l0"), cat("r0"))
    b.set_tissues([s.L for s in states], [s.Kre for s in states], [s.Kat for s in states],
                  [s.pbc for s in states])
    if tuning:
        b.set_tuning(**tuning)
    b.upload(np.concatenate([s.xy for s in states]))
    return b
