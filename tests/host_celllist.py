"""Host rebuild of the 2D cell list, for the bit-exact check of the device one.

Every float operation is an IEEE float32 operation in the same order as the
device code (which rounds each operation separately on that path), so keys,
sorted order and neighbour lists must agree exactly.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32
MAXNB = 96
NBBUF = 128


def roundf(x):
    """C roundf: halves away from zero."""
    x = f32(x)
    a = np.abs(x)
    r = np.floor(a)
    frac = f32(a - r)
    r = f32(r + (f32(1) if frac >= f32(0.5) else f32(0)))
    return f32(np.copysign(r, x))


def wrap(x, L):
    return f32(x - f32(L * np.floor(f32(x / L))))


def bin_of(x, L, inv, nb):
    b = int(np.floor(f32(wrap(x, L) * inv)))
    return max(0, min(b, nb - 1))


def rebuild_margin(gi, gj, L):
    mag = f32(f32(f32(f32(abs(gi[0]) + abs(gi[1])) + abs(gj[0])) + abs(gj[1])) + L)
    return f32(f32(f32(1e-3) * f32(gi[2] + gj[2])) + f32(f32(1e-4) * mag))


def pair_near(gi, gj, T, l0):
    dx, dy = f32(gi[0] - gj[0]), f32(gi[1] - gj[1])
    m = rebuild_margin(gi, gj, T["L"])
    r = f32(f32(f32(gi[2] + gj[2]) + T["skin"]) + m)
    if f32(f32(dx * dx) + f32(dy * dy)) <= f32(r * r):
        return True
    if T["Kat"] != 0:
        ex, ey = dx, dy
        if T["pbc"]:
            ex = f32(ex - f32(T["L"] * roundf(f32(ex / T["L"]))))
            ey = f32(ey - f32(T["L"] * roundf(f32(ey / T["L"]))))
        ra = f32(r + max(f32(l0), T["l0max"]))
        if f32(f32(ex * ex) + f32(ey * ey)) <= f32(ra * ra):
            return True
    return False


def pair_far(gi, gj, T):
    if not T["pbc"]:
        return False
    lim = f32(f32(T["L"] - T["skin"]) - rebuild_margin(gi, gj, T["L"]))
    # geom columns: cx cy R area minx maxx miny maxy
    return (f32(gi[5] - gj[4]) >= lim or f32(gj[5] - gi[4]) >= lim or
            f32(gi[7] - gj[6]) >= lim or f32(gj[7] - gi[6]) >= lim)


def on_boundary(gi, T):
    if not T["pbc"]:
        return False
    ext = f32(f32(f32(abs(T["gminx"]) + abs(T["gmaxx"])) + abs(T["gminy"])) + abs(T["gmaxy"]))
    own = f32(f32(abs(gi[0]) + abs(gi[1])) + T["L"])
    m = f32(f32(f32(f32(2e-3) * f32(gi[2] + T["binw"])) + f32(f32(1e-4) * own)) +
            f32(f32(2e-4) * ext))
    lim = f32(f32(T["L"] - T["skin"]) - m)
    return (f32(gi[5] - T["gminx"]) >= lim or f32(T["gmaxx"] - gi[4]) >= lim or
            f32(gi[7] - T["gminy"]) >= lim or f32(T["gmaxy"] - gi[6]) >= lim)


def host_rebuild(geom, tissue_of, tissues, l0, local_bits):
    """geom: (n, 8) float32 device geometry; tissues: list of dicts with
    L, skin, Kat, pbc, l0max, cap, begin, end.  Returns (keys, ids, nn, nbr, nbins)."""
    geom = np.asarray(geom, dtype=np.float32)
    n = len(geom)
    keys = np.zeros(n, np.uint32)
    nbins = []
    for t, T in enumerate(tissues):
        g = geom[T["begin"]:T["end"]]
        dmax = f32(np.max(f32(2) * g[:, 2]))
        T["gminx"], T["gmaxx"] = f32(g[:, 4].min()), f32(g[:, 5].max())
        T["gminy"], T["gmaxy"] = f32(g[:, 6].min()), f32(g[:, 7].max())
        w = f32(dmax + T["skin"])
        w = f32(w + f32(f32(f32(1e-3) * dmax) + f32(f32(1e-5) * T["L"])))
        if T["Kat"] != 0:
            w = f32(w + T["l0max"])
        nb = int(np.floor(f32(T["L"] / w)))
        nb = max(1, min(nb, T["cap"]))
        T["binw"], T["nb"] = w, nb
        nbins.append(nb)
        inv = f32(f32(nb) / T["L"])
        for c in range(T["begin"], T["end"]):
            bx = bin_of(geom[c, 0], T["L"], inv, nb)
            by = bin_of(geom[c, 1], T["L"], inv, nb)
            keys[c] = (t << local_bits) | (by * nb + bx)
    order = np.argsort(keys, kind="stable").astype(np.uint32)
    skeys = keys[order]
    nn = np.zeros(n, np.int32)
    nbr = np.full((n, MAXNB), -1, np.int32)
    for c in range(n):
        t = tissue_of[c]
        T = tissues[t]
        gi = geom[c]
        nb = T["nb"]
        inv = f32(f32(nb) / T["L"])
        bx, by = bin_of(gi[0], T["L"], inv, nb), bin_of(gi[1], T["L"], inv, nb)
        offs = [-1, 0, 1] if nb >= 3 else list(range(nb))
        buf = []
        for oy in offs:
            yy = (by + oy + nb) % nb
            for ox in offs:
                xx = (bx + ox + nb) % nb
                key = (t << local_bits) | (yy * nb + xx)
                lo = T["begin"] + int(np.searchsorted(skeys[T["begin"]:T["end"]], key, "left"))
                hi = T["begin"] + int(np.searchsorted(skeys[T["begin"]:T["end"]], key, "right"))
                for q in range(lo, hi):
                    j = int(order[q])
                    if j != c and pair_near(gi, geom[j], T, l0[c]):
                        buf.append(j)
        if on_boundary(gi, T):
            for j in range(T["begin"], T["end"]):
                if j != c and pair_far(gi, geom[j], T):
                    buf.append(j)
        uniq = sorted(set(buf))
        if len(buf) > NBBUF or len(uniq) > MAXNB:
            nn[c] = -1
        else:
            nn[c] = len(uniq)
            nbr[c, :len(uniq)] = uniq
    return skeys, order, nn, nbr, np.array(nbins)
