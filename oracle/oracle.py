"""Python access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Two libraries sit behind this module:

* ``Port``: ``oracle/libdpm_oracle.so``, the project's plain-C restatement of
  the reference algorithm (``oracle/dpm_oracle.c``).  It builds anywhere gcc
  is present (this container and the GPU machines).
* ``Ref``: ``oracle/_ref/libdpm_ref.so``, the reference's own host code and
  kernel text compiled for the CPU by ``oracle/build_ref.py``.  It exists only
  where the reference tree was available at build time.

Only the tests, the smoke check and the benchmark's CPU-baseline leg may use
this module, and only as the checker or the CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libdpm_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdpm_ref.so")

_f32p = ctypes.POINTER(ctypes.c_float)
_u32p = ctypes.POINTER(ctypes.c_uint)
_u8p = ctypes.POINTER(ctypes.c_ubyte)
_f64p = ctypes.POINTER(ctypes.c_double)


def build_port(force: bool = False) -> str:
    """Compile the oracle restatement (gcc, OpenMP, no contraction)."""
    src = os.path.join(HERE, "dpm_oracle.c")
    if not force and os.path.exists(PORT_SO) and os.path.getmtime(PORT_SO) >= os.path.getmtime(src):
        return PORT_SO
    tmp = PORT_SO + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-std=c11", "-D_DEFAULT_SOURCE", "-fopenmp", "-ffp-contract=off",
           "-fno-strict-aliasing", "-fPIC", "-shared", src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, PORT_SO)
    return PORT_SO


def _p(a, t=_f32p):
    return None if a is None else a.ctypes.data_as(t)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


class _Tissue2D(ctypes.Structure):
    _fields_ = [("ncells", ctypes.c_int), ("nv", _u32p), ("off", _u32p),
                ("Ka", _f32p), ("Kl", _f32p), ("Kb", _f32p), ("a0", _f32p), ("l0", _f32p),
                ("r0", _f32p), ("pbc", ctypes.c_int), ("L", ctypes.c_float),
                ("Kre", ctypes.c_float), ("Kat", ctypes.c_float)]


class _Tissue3D(ctypes.Structure):
    _fields_ = [("ncells", ctypes.c_int), ("nv", ctypes.c_int), ("nf", ctypes.c_int),
                ("faces", _u32p), ("Kv", _f32p), ("Ka", _f32p), ("Ks", _f32p), ("v0", _f32p),
                ("a0", _f32p), ("l0", _f32p), ("Kb", _f32p), ("adh", _f32p),
                ("pbc", ctypes.c_int), ("L", ctypes.c_float), ("Kre", ctypes.c_float),
                ("Kat", ctypes.c_float)]


@dataclass
class Tissue2DState:
    """A 2D tissue in the oracle's layout (ragged, cell-major, xy interleaved)."""
    nv: np.ndarray
    xy: np.ndarray  # [sum(nv), 2] float32
    Ka: np.ndarray
    Kl: np.ndarray
    Kb: np.ndarray
    a0: np.ndarray
    l0: np.ndarray
    r0: np.ndarray
    L: float
    Kre: float = 1.0
    Kat: float = 0.0
    pbc: int = 1

    @property
    def off(self) -> np.ndarray:
        o = np.zeros(len(self.nv), np.uint32)
        o[1:] = np.cumsum(self.nv[:-1])
        return o

    def copy(self) -> "Tissue2DState":
        return Tissue2DState(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                                for k, v in self.__dict__.items()})


@dataclass
class Tissue3DState:
    """A 3D tissue: cells share one face table; xyz is [ncells*nv, 3]."""
    nv: int
    faces: np.ndarray  # [nf, 3] uint32
    xyz: np.ndarray
    Kv: np.ndarray
    Ka: np.ndarray
    Ks: np.ndarray
    v0: np.ndarray
    a0: np.ndarray
    l0: np.ndarray
    L: float
    Kre: float = 1.0
    pbc: int = 1
    Kb: np.ndarray | None = None
    adh: np.ndarray | None = None
    Kat: float = 0.0  # AllVertAttraction (off in the reference's own step loop)

    @property
    def ncells(self) -> int:
        return len(self.Kv)

    def copy(self) -> "Tissue3DState":
        return Tissue3DState(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                                for k, v in self.__dict__.items()})


class Port:
    """The oracle restatement (oracle/dpm_oracle.c)."""

    def __init__(self):
        self.lib = ctypes.CDLL(build_port())
        L = self.lib
        L.orc_area2d.restype = ctypes.c_float
        L.orc_box2d.restype = ctypes.c_float
        L.orc_box3d.restype = ctypes.c_float
        L.orc_l0_3d.restype = ctypes.c_float
        L.orc_l0_3d.argtypes = [ctypes.c_float]
        L.orc_volume3d.restype = ctypes.c_float
        L.orc_surface3d.restype = ctypes.c_float
        L.orc_bend_energy3d.restype = ctypes.c_double
        L.orc_cell2d.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_uint,
                                 ctypes.c_float, _f32p, _f32p, _f32p, _f32p]
        L.orc_box2d.argtypes = [_f32p, ctypes.c_int, ctypes.c_float]
        L.orc_box3d.argtypes = [_f32p, ctypes.c_int, ctypes.c_float]
        L.orc_cell3d.argtypes = [_f32p, ctypes.c_float, ctypes.c_float, ctypes.c_int, _f32p,
                                 _u32p, _f32p, _f32p, _f32p]
        L.orc_run2d.argtypes = [ctypes.POINTER(_Tissue2D), ctypes.c_float, ctypes.c_int, _f32p,
                                _f32p, _u8p, ctypes.c_int]
        L.orc_run3d.argtypes = [ctypes.POINTER(_Tissue3D), ctypes.c_float, ctypes.c_int, _f32p,
                                _f32p, _u8p, ctypes.c_int]
        L.orc_disperse2d.argtypes = [ctypes.c_int, _u32p, _u32p, _f32p, ctypes.c_float,
                                     ctypes.c_long, _f32p]
        L.orc_disperse3d.argtypes = [ctypes.c_int, ctypes.c_int, _f32p, ctypes.c_float,
                                     ctypes.c_long, _f32p]
        L.orc_diag2d.argtypes = [ctypes.POINTER(_Tissue2D), _f32p, _f64p, _f64p, _f64p]
        L.orc_diag3d.argtypes = [ctypes.POINTER(_Tissue3D), _f32p, _f64p, _f64p, _f64p]
        L.orc_bend_energy3d.argtypes = [ctypes.c_int, ctypes.c_int, _u32p, ctypes.c_double, _f64p]
        L.orc_attraction3d.argtypes = [ctypes.c_int, ctypes.c_int, _f32p, _f32p, ctypes.c_float,
                                       ctypes.c_int, ctypes.c_float, _f32p]

    # -- geometry --
    def cell2d(self, x0, y0, calA, nv, r0):
        xy = np.zeros((nv, 2), np.float32)
        a0, l0, c0 = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        self.lib.orc_cell2d(x0, y0, calA, nv, r0, _p(xy), ctypes.byref(a0), ctypes.byref(l0),
                            ctypes.byref(c0))
        return xy, a0.value, l0.value, c0.value

    def area2d(self, xy):
        xy = _f32(xy)
        return self.lib.orc_area2d(_p(xy), ctypes.c_uint(len(xy)))

    def box2d(self, areas, phi0):
        a = _f32(areas)
        return self.lib.orc_box2d(_p(a), len(a), phi0)

    def box3d(self, v0, phi0):
        a = _f32(v0)
        return self.lib.orc_box3d(_p(a), len(a), phi0)

    def l0_3d(self, a0):
        return self.lib.orc_l0_3d(a0)

    def icosphere_counts(self, level):
        nv, nf = ctypes.c_int(), ctypes.c_int()
        if self.lib.orc_icosphere_counts(level, ctypes.byref(nv), ctypes.byref(nf)):
            raise ValueError("bad subdivision level")
        return nv.value, nf.value

    def cell3d(self, start, calA, r0, level=2):
        nv, nf = self.icosphere_counts(level)
        xyz = np.zeros((nv, 3), np.float32)
        faces = np.zeros((nf, 3), np.uint32)
        s = _f32(start)
        v0, sa0, a0 = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        self.lib.orc_cell3d(_p(s), calA, r0, level, _p(xyz), _p(faces, _u32p), ctypes.byref(v0),
                            ctypes.byref(sa0), ctypes.byref(a0))
        return xyz, faces, v0.value, sa0.value, a0.value

    def volume3d(self, xyz, faces):
        xyz, faces = _f32(xyz), _u32(faces)
        return self.lib.orc_volume3d(_p(xyz), _p(faces, _u32p), len(faces))

    def surface3d(self, xyz, faces):
        xyz, faces = _f32(xyz), _u32(faces)
        return self.lib.orc_surface3d(_p(xyz), _p(faces, _u32p), len(faces))

    # -- stepping --
    def _t2(self, s: Tissue2DState, keep):
        arrs = dict(nv=_u32(s.nv), off=_u32(s.off), Ka=_f32(s.Ka), Kl=_f32(s.Kl), Kb=_f32(s.Kb),
                    a0=_f32(s.a0), l0=_f32(s.l0), r0=_f32(s.r0))
        keep.append(arrs)
        return _Tissue2D(len(s.nv), _p(arrs["nv"], _u32p), _p(arrs["off"], _u32p),
                         _p(arrs["Ka"]), _p(arrs["Kl"]), _p(arrs["Kb"]), _p(arrs["a0"]),
                         _p(arrs["l0"]), _p(arrs["r0"]), int(s.pbc), float(s.L), float(s.Kre),
                         float(s.Kat))

    def run2d(self, s: Tissue2DState, nsteps: int, dt: float, nthreads: int = 0):
        """Runs in place on s.xy; returns (forces of the last step, containment flags)."""
        keep = []
        t = self._t2(s, keep)
        s.xy = _f32(s.xy)
        F = np.zeros_like(s.xy)
        flags = np.zeros(len(s.xy), np.uint8)
        rc = self.lib.orc_run2d(ctypes.byref(t), dt, nsteps, _p(s.xy), _p(F), _p(flags, _u8p),
                                nthreads)
        if rc:
            raise RuntimeError(f"orc_run2d failed ({rc})")
        return F, flags

    def _t3(self, s: Tissue3DState, keep):
        arrs = dict(faces=_u32(s.faces), Kv=_f32(s.Kv), Ka=_f32(s.Ka), Ks=_f32(s.Ks),
                    v0=_f32(s.v0), a0=_f32(s.a0), l0=_f32(s.l0),
                    Kb=None if s.Kb is None else _f32(s.Kb),
                    adh=None if s.adh is None else _f32(s.adh))
        keep.append(arrs)
        return _Tissue3D(s.ncells, s.nv, len(s.faces), _p(arrs["faces"], _u32p), _p(arrs["Kv"]),
                         _p(arrs["Ka"]), _p(arrs["Ks"]), _p(arrs["v0"]), _p(arrs["a0"]),
                         _p(arrs["l0"]), _p(arrs["Kb"]), _p(arrs["adh"]), int(s.pbc),
                         float(s.L), float(s.Kre), float(s.Kat))

    def run3d(self, s: Tissue3DState, nsteps: int, dt: float, nthreads: int = 0):
        keep = []
        t = self._t3(s, keep)
        s.xyz = _f32(s.xyz)
        F = np.zeros_like(s.xyz)
        flags = np.zeros(len(s.xyz), np.uint8)
        rc = self.lib.orc_run3d(ctypes.byref(t), dt, nsteps, _p(s.xyz), _p(F), _p(flags, _u8p),
                                nthreads)
        if rc:
            raise RuntimeError(f"orc_run3d failed ({rc})")
        return F, flags

    def attraction3d(self, xyz, nv, l0, L, pbc, Kat):
        """AllVertAttraction alone: the forces it adds, [ncells*nv, 3]."""
        xyz = _f32(xyz)
        l0 = _f32(l0)
        F = np.zeros_like(xyz)
        self.lib.orc_attraction3d(len(l0), nv, _p(xyz), _p(l0), float(L), int(pbc), float(Kat),
                                  _p(F))
        return F

    def disperse2d(self, nv, r0, L, seed):
        nv = _u32(nv)
        off = np.zeros(len(nv), np.uint32)
        off[1:] = np.cumsum(nv[:-1])
        xy = np.zeros((int(nv.sum()), 2), np.float32)
        r = _f32(r0)
        self.lib.orc_disperse2d(len(nv), _p(nv, _u32p), _p(off, _u32p), _p(r), L, seed, _p(xy))
        return xy

    def disperse3d(self, xyz, nv, r0, L, seed):
        xyz = _f32(xyz).copy()
        r = _f32(r0)
        self.lib.orc_disperse3d(len(r), nv, _p(r), L, seed, _p(xyz))
        return xyz

    def diag2d(self, s: Tissue2DState, xy=None):
        keep = []
        t = self._t2(s, keep)
        xy = _f32(s.xy if xy is None else xy)
        n = len(s.nv)
        a, p, e = (np.zeros(n) for _ in range(3))
        self.lib.orc_diag2d(ctypes.byref(t), _p(xy), _p(a, _f64p), _p(p, _f64p), _p(e, _f64p))
        return a, p, e

    def diag3d(self, s: Tissue3DState, xyz=None):
        keep = []
        t = self._t3(s, keep)
        xyz = _f32(s.xyz if xyz is None else xyz)
        n = s.ncells
        v, a, e = (np.zeros(n) for _ in range(3))
        self.lib.orc_diag3d(ctypes.byref(t), _p(xyz), _p(v, _f64p), _p(a, _f64p), _p(e, _f64p))
        return v, a, e

    def bend_energy3d(self, xyz_f64, faces, kb):
        x = np.ascontiguousarray(xyz_f64, dtype=np.float64)
        f = _u32(faces)
        return self.lib.orc_bend_energy3d(len(x), len(f), _p(f, _u32p), kb, _p(x, _f64p))


def ref_available() -> bool:
    return os.path.exists(REF_SO) and os.path.exists(os.path.join(HERE, "_ref", "reference_dir.txt"))


class Ref:
    """The reference's own host code and kernel text, built for the CPU."""

    def __init__(self):
        if not ref_available():
            raise FileNotFoundError("oracle/_ref not built (needs the reference tree)")
        self.lib = ctypes.CDLL(REF_SO)
        self.refdir = open(os.path.join(HERE, "_ref", "reference_dir.txt")).read().strip().encode()
        self.lib.ref_last_error.restype = ctypes.c_char_p
        self.lib.ref2d_cell.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                        ctypes.c_uint, ctypes.c_float, _f32p, _f32p, _f32p, _f32p]
        self.lib.ref2d_run.argtypes = [ctypes.c_char_p, ctypes.c_int, _f32p, _f32p, _f32p, _u32p,
                                       _f32p, _f32p, _f32p, _f32p, _f32p, ctypes.c_float,
                                       ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                       ctypes.c_long, ctypes.c_int, ctypes.c_float, _f32p,
                                       _f32p, _f32p]
        self.lib.ref3d_cell.argtypes = [_f32p, ctypes.c_float, ctypes.c_float, _f32p, _u32p,
                                        _f32p, _f32p, _f32p, _f32p, _f32p]
        self.lib.ref3d_attraction.argtypes = [ctypes.c_char_p, ctypes.c_int, _f32p, _f32p,
                                              ctypes.c_float, ctypes.c_int, ctypes.c_float,
                                              _f32p]
        self.lib.ref3d_run.argtypes = [ctypes.c_char_p, ctypes.c_int, _f32p, _f32p, _f32p,
                                       _f32p, _f32p, _f32p, _f32p, ctypes.c_float,
                                       ctypes.c_float, ctypes.c_int, ctypes.c_long,
                                       ctypes.c_int, ctypes.c_float, _f32p, _f32p, _f32p,
                                       _f32p, _f32p]

    def cell2d(self, x0, y0, calA, nv, r0):
        xy = np.zeros((nv, 2), np.float32)
        a0, l0, c0 = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        self.lib.ref2d_cell(x0, y0, calA, nv, r0, _p(xy), ctypes.byref(a0), ctypes.byref(l0),
                            ctypes.byref(c0))
        return xy, a0.value, l0.value, c0.value

    def run2d(self, x0, y0, calA, nv, r0, Ka, Kl, Kb, xy=None, phi0=1.0, Kre=1.0, Kat=0.0,
              disperse=False, seed=0, nsteps=0, dt=0.005):
        """Constructs reference Cell2D/Tissue2D and runs CLEulerUpdate(nsteps, dt).

        Returns (xy, forces, L)."""
        x0, y0, calA, r0, Ka, Kl, Kb = map(_f32, (x0, y0, calA, r0, Ka, Kl, Kb))
        nv = _u32(nv)
        tot = int(nv.sum())
        xin = None if xy is None else _f32(xy)
        xo = np.zeros((tot, 2), np.float32)
        fo = np.zeros((tot, 2), np.float32)
        Lo = ctypes.c_float()
        rc = self.lib.ref2d_run(self.refdir, len(nv), _p(x0), _p(y0), _p(calA), _p(nv, _u32p),
                                _p(r0), _p(Ka), _p(Kl), _p(Kb), _p(xin), phi0, Kre, Kat,
                                int(disperse), seed, nsteps, dt, _p(xo), _p(fo), ctypes.byref(Lo))
        if rc:
            raise RuntimeError(f"ref2d_run: {self.lib.ref_last_error().decode()}")
        return xo, fo, Lo.value

    def cell3d(self, start, calA, r0):
        xyz = np.zeros((162, 3), np.float32)
        faces = np.zeros((320, 3), np.uint32)
        s = _f32(start)
        out = [ctypes.c_float() for _ in range(5)]
        self.lib.ref3d_cell(_p(s), calA, r0, _p(xyz), _p(faces, _u32p),
                            *[ctypes.byref(o) for o in out])
        return (xyz, faces) + tuple(o.value for o in out)

    def run3d(self, start, calA, r0, Kv, Ka, Ks, xyz=None, phi0=1.0, Kre=1.0, disperse=False,
              seed=0, nsteps=0, dt=0.005):
        """Constructs reference Cell3D/Tissue3D and runs CLEulerUpdate.

        Returns (xyz, forces, volume, surface_area, L)."""
        start, calA, r0, Kv, Ka, Ks = map(_f32, (start, calA, r0, Kv, Ka, Ks))
        n = len(Kv)
        xin = None if xyz is None else _f32(xyz)
        xo = np.zeros((n * 162, 3), np.float32)
        fo = np.zeros((n * 162, 3), np.float32)
        vo = np.zeros(n, np.float32)
        so = np.zeros(n, np.float32)
        Lo = ctypes.c_float()
        rc = self.lib.ref3d_run(self.refdir, n, _p(start), _p(calA), _p(r0), _p(Kv), _p(Ka),
                                _p(Ks), _p(xin), phi0, Kre, int(disperse), seed, nsteps, dt,
                                _p(xo), _p(fo), _p(vo), _p(so), ctypes.byref(Lo))
        if rc:
            raise RuntimeError(f"ref3d_run: {self.lib.ref_last_error().decode()}")
        return xo, fo, vo, so, Lo.value

    def attraction3d(self, xyz, l0, L, pbc, Kat):
        """The reference's AllVertAttraction kernel run once through its own
        OpenCL calls on the CPU shim (162 vertices per cell)."""
        xyz = _f32(xyz)
        l0 = _f32(l0)
        F = np.zeros_like(xyz)
        rc = self.lib.ref3d_attraction(self.refdir, len(l0), _p(xyz), _p(l0), float(L), int(pbc),
                                       float(Kat), _p(F))
        if rc:
            raise RuntimeError(f"ref3d_attraction: {self.lib.ref_last_error().decode()}")
        return F
