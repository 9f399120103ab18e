"""ctypes binding of the C ABI (include/dpm_gb300.h).

This is the same binding a Python caller of the library would write by hand;
the tests and the benchmark go through it so that what they exercise is the
C boundary itself.  Loading fails loudly when the native library is missing:
there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libdpm_gb300.so")

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_uint_p = ctypes.POINTER(ctypes.c_uint)
_c_float_p = ctypes.POINTER(ctypes.c_float)
_c_long_p = ctypes.POINTER(ctypes.c_long)
_c_ubyte_p = ctypes.POINTER(ctypes.c_ubyte)
_vp = ctypes.c_void_p

# name -> (restype, argtypes); the full exported surface of dpm_gb300.h
SIGNATURES = {
    "dpm_last_error": (ctypes.c_char_p, []),
    "dpm_version": (ctypes.c_char_p, []),
    "dpm_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp)]),
    "dpm_ctx_destroy": (ctypes.c_int, [_vp]),
    "dpm_ctx_synchronize": (ctypes.c_int, [_vp]),
    "dpm_ctx_sm_count": (ctypes.c_int, [_vp, _c_int_p]),
    "dpm_ctx_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "dpm2d_create": (ctypes.c_int, [_vp, ctypes.c_int, _c_int_p, _c_uint_p, ctypes.POINTER(_vp)]),
    "dpm2d_destroy": (ctypes.c_int, [_vp]),
    "dpm2d_set_cells": (ctypes.c_int, [_vp] + [_c_float_p] * 6),
    "dpm2d_set_tissues": (ctypes.c_int, [_vp, _c_float_p, _c_float_p, _c_float_p, _c_int_p]),
    "dpm2d_upload": (ctypes.c_int, [_vp, _vp]),
    "dpm2d_step": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_float]),
    "dpm2d_download": (ctypes.c_int, [_vp, _vp, _vp]),
    "dpm2d_sizes": (ctypes.c_int, [_vp, _c_int_p, _c_long_p]),
    "dpm2d_set_tuning": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_float, ctypes.c_int]),
    "dpm2d_set_kernel_variant": (ctypes.c_int, [_vp, ctypes.c_int]),
    "dpm2d_last_contained": (ctypes.c_int, [_vp, _c_ubyte_p]),
    "dpm2d_cell_areas": (ctypes.c_int, [_vp, _c_float_p]),
    "dpm2d_stats": (ctypes.c_int, [_vp, _c_long_p, _c_long_p]),
    "dpm2d_rebuild_now": (ctypes.c_int, [_vp]),
    "dpm2d_cell_list": (ctypes.c_int, [_vp, _c_uint_p, _c_uint_p, _c_int_p, _c_int_p, _c_int_p,
                                       _c_float_p]),
    "dpm2d_bins": (ctypes.c_int, [_vp, _c_int_p, _c_int_p, _c_float_p, _c_float_p]),
    "dpm2d_step_kernel": (ctypes.c_int, [_vp, ctypes.c_float]),
    "dpm2d_autotune": (ctypes.c_int, [_vp, ctypes.c_float, ctypes.c_int, ctypes.c_int, _c_int_p,
                                      _c_int_p, _c_int_p, _c_float_p, _c_float_p]),
    "dpm3d_create": (ctypes.c_int, [_vp, ctypes.c_int, _c_int_p, ctypes.c_int, ctypes.c_int,
                                    _c_uint_p, ctypes.POINTER(_vp)]),
    "dpm3d_destroy": (ctypes.c_int, [_vp]),
    "dpm3d_set_cells": (ctypes.c_int, [_vp] + [_c_float_p] * 8),
    "dpm3d_set_tissues": (ctypes.c_int, [_vp, _c_float_p, _c_float_p, _c_int_p]),
    "dpm3d_set_attraction": (ctypes.c_int, [_vp, _c_float_p]),
    "dpm3d_upload": (ctypes.c_int, [_vp, _vp]),
    "dpm3d_step": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_float]),
    "dpm3d_download": (ctypes.c_int, [_vp, _vp, _vp]),
    "dpm3d_sizes": (ctypes.c_int, [_vp, _c_int_p, _c_long_p]),
    "dpm3d_last_winding": (ctypes.c_int, [_vp, _c_ubyte_p]),
    "dpm3d_set_tuning": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_float]),
    "dpm3d_set_block_threads": (ctypes.c_int, [_vp, ctypes.c_int]),
    "dpm2d_step_noalloc": (ctypes.c_int, [ctypes.c_int, _c_uint_p] + [_c_float_p] * 6 +
                           [ctypes.c_float] * 3 + [ctypes.c_int, _vp, _vp, ctypes.c_int,
                                                   ctypes.c_float, _vp]),
    "dpm2d_diagnostics": (ctypes.c_int, [_vp] + [ctypes.POINTER(ctypes.c_double)] * 5),
    "dpm2d_set_packing_fraction": (ctypes.c_int, [_vp, _c_float_p]),
    "dpm2d_device_state": (ctypes.c_int, [_vp] + [ctypes.POINTER(_vp)] * 2),
    "dpm2d_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "dpm2d_open": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "dpm3d_device_state": (ctypes.c_int, [_vp] + [ctypes.POINTER(_vp)] * 6),
    "dpm3d_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "dpm3d_open": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "dpm3d_diagnostics": (ctypes.c_int, [_vp] + [ctypes.POINTER(ctypes.c_double)] * 3),
    "dpm_disperse": (ctypes.c_int, [_vp, ctypes.c_int, _c_int_p, _c_float_p, _c_float_p,
                                    _c_float_p, _c_float_p, _c_int_p]),
    "dpm_serve_create": (ctypes.c_int, [_vp, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(_vp)]),
    "dpm_serve_destroy": (ctypes.c_int, [_vp]),
    "dpm_serve_add_pool2d": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_float]),
    "dpm_serve_add_pool3d": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, _c_uint_p, ctypes.c_float]),
    "dpm_serve_pool_bytes": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_size_t)]),
    "dpm_serve_submit2d": (ctypes.c_int, [_vp, ctypes.c_int, _c_uint_p] + [_c_float_p] * 7 +
                           [ctypes.c_float] * 3 + [ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                   ctypes.POINTER(ctypes.c_uint64)]),
    "dpm_serve_submit3d": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int] + [_c_float_p] * 9 +
                           [ctypes.c_float] * 2 + [ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                   ctypes.POINTER(ctypes.c_uint64)]),
    "dpm_serve_step": (ctypes.c_int, [_vp, _c_int_p, _c_int_p, _c_int_p]),
    "dpm_serve_drain": (ctypes.c_int, [_vp]),
    "dpm_serve_result": (ctypes.c_int, [_vp, ctypes.c_uint64, _c_float_p, _c_float_p,
                                        ctypes.POINTER(ctypes.c_double), _c_int_p]),
    "dpm_serve_forget": (ctypes.c_int, [_vp, ctypes.c_uint64]),
    "dpm_serve_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_size_t)]),
}

_lib = None


class DPMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def load(path: str = LIB_PATH, strict: bool = False):
    """Loads the library and declares every entry point it exports.  With
    strict=True a missing symbol raises."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        try:
            fn = getattr(lib, name)
        except AttributeError:
            if strict:
                raise
            continue
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = lib
    return lib


def check(rc: int):
    if rc != 0:
        msg = _lib.dpm_last_error().decode() if _lib is not None else ""
        raise DPMError(rc, msg)


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_c_float_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class _DeviceArray:
    """A float32 device buffer described by __cuda_array_interface__ (v3),
    for zero-copy views (torch.as_tensor(obj, device=...)); keeps its owner
    alive."""

    def __init__(self, ptr: int, shape, owner):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4",
                                         "data": (int(ptr), False), "version": 3,
                                         "strides": None}
        self._owner = owner


def _torch_view(ptr: int, shape, owner, device: int):
    import torch
    return torch.as_tensor(_DeviceArray(ptr, shape, owner), device=f"cuda:{device}")


def _ckpt_shape(path: str, dim: int):
    """(ntissues, per-tissue cells, per-cell NV or mesh NV) from a checkpoint
    header (the layout written by dpm2d_save / dpm3d_save)."""
    with open(path, "rb") as f:
        head = f.read(16)
        if len(head) < 16 or head[:7] != b"DPMCKPT":
            raise DPMError(1, f"{path}: not a checkpoint")
        if dim == 2:
            T, N = np.frombuffer(f.read(8), np.int32)
            f.read(8)  # vertices (int64)
            nc = np.frombuffer(f.read(4 * T), np.int32).copy()
            nv = np.frombuffer(f.read(4 * N), np.uint32).copy()
            return int(T), nc, nv
        T, N, nv, nf = np.frombuffer(f.read(16), np.int32)
        f.read(4 * 3 * int(nf))
        nc = np.frombuffer(f.read(4 * T), np.int32).copy()
        return int(T), nc, int(nv)


class Context:
    """dpm_ctx: one CUDA device and stream."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.device = device
        h = _vp()
        check(self.lib.dpm_ctx_create(device, ctypes.byref(h)))
        self.h = h

    def sm_count(self) -> int:
        n = ctypes.c_int()
        check(self.lib.dpm_ctx_sm_count(self.h, ctypes.byref(n)))
        return n.value

    def synchronize(self):
        check(self.lib.dpm_ctx_synchronize(self.h))

    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        p = _vp()
        check(self.lib.dpm_ctx_stream(self.h, ctypes.byref(p)))
        return int(p.value or 0)

    def close(self):
        if self.h:
            self.lib.dpm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch2D:
    """dpm2d_batch: independent 2D tissues stepped together."""

    def __init__(self, ctx: Context, ncells, nv):
        self.ctx = ctx
        self.lib = ctx.lib
        nc = np.ascontiguousarray(ncells, dtype=np.int32)
        self.nv = np.ascontiguousarray(nv, dtype=np.uint32)
        h = _vp()
        check(self.lib.dpm2d_create(ctx.h, len(nc), nc.ctypes.data_as(_c_int_p),
                                    self.nv.ctypes.data_as(_c_uint_p), ctypes.byref(h)))
        self.h = h
        self.ntissues = len(nc)
        self.ncells = int(nc.sum())
        self.nverts = int(self.nv.sum())

    def set_cells(self, Ka, Kl, Kb, a0, l0, r0):
        arrs = [_f32(x) for x in (Ka, Kl, Kb, a0, l0, r0)]
        for x in arrs:
            if x.shape != (self.ncells,):
                raise ValueError("per-cell arrays must have one value per cell")
        check(self.lib.dpm2d_set_cells(self.h, *[fptr(x) for x in arrs]))

    def set_tissues(self, L, Kre, Kat, pbc):
        L, Kre, Kat = (_f32(np.broadcast_to(x, (self.ntissues,))) for x in (L, Kre, Kat))
        p = np.ascontiguousarray(np.broadcast_to(pbc, (self.ntissues,)), dtype=np.int32)
        check(self.lib.dpm2d_set_tissues(self.h, fptr(L), fptr(Kre), fptr(Kat),
                                         p.ctypes.data_as(_c_int_p)))

    def set_tuning(self, rebuild_period=0, skin_rel=0.0, warps=0):
        check(self.lib.dpm2d_set_tuning(self.h, rebuild_period, skin_rel, warps))

    def set_kernel_variant(self, variant: int):
        check(self.lib.dpm2d_set_kernel_variant(self.h, variant))

    def device_state(self):
        """Zero-copy torch views (nverts, 2) of the current positions and
        the last step's forces on the device; valid until the next step or
        upload."""
        p, f = _vp(), _vp()
        check(self.lib.dpm2d_device_state(self.h, ctypes.byref(p), ctypes.byref(f)))
        return (_torch_view(p.value, (self.nverts, 2), self, self.ctx.device),
                _torch_view(f.value, (self.nverts, 2), self, self.ctx.device))

    def save(self, path: str):
        check(self.lib.dpm2d_save(self.h, os.fsencode(path)))

    @classmethod
    def open(cls, ctx: Context, path: str) -> "Batch2D":
        """A batch restored from a checkpoint written by save()."""
        T, nc, nv = _ckpt_shape(path, 2)
        h = _vp()
        check(ctx.lib.dpm2d_open(ctx.h, os.fsencode(path), ctypes.byref(h)))
        b = cls.__new__(cls)
        b.ctx, b.lib, b.h = ctx, ctx.lib, h
        b.nv = nv
        b.ntissues, b.ncells, b.nverts = T, int(nc.sum()), int(nv.sum())
        return b

    def diagnostics(self) -> dict:
        """Per cell area, perimeter, energy; per tissue packing fraction and
        mean shape index (double, computed on the device)."""
        d = ctypes.POINTER(ctypes.c_double)
        a, p, e = (np.zeros(self.ncells) for _ in range(3))
        phi, si = np.zeros(self.ntissues), np.zeros(self.ntissues)
        check(self.lib.dpm2d_diagnostics(self.h, *[x.ctypes.data_as(d) for x in (a, p, e, phi, si)]))
        return {"area": a, "perimeter": p, "energy": e, "packing_fraction": phi,
                "shape_index": si}

    def set_packing_fraction(self, phi):
        """Rescales every tissue with phi > 0 to that true packing fraction
        on the device (box side and centroids; shapes kept); 0 leaves a
        tissue unchanged."""
        phi = _f32(np.broadcast_to(phi, (self.ntissues,)))
        check(self.lib.dpm2d_set_packing_fraction(self.h, fptr(phi)))

    def upload(self, xy):
        xy = _f32(xy)
        assert xy.size == 2 * self.nverts
        check(self.lib.dpm2d_upload(self.h, xy.ctypes.data))

    def upload_ptr(self, ptr: int):
        check(self.lib.dpm2d_upload(self.h, ctypes.c_void_p(ptr)))

    def step(self, nsteps: int, dt: float):
        check(self.lib.dpm2d_step(self.h, nsteps, dt))

    def download(self):
        xy = np.empty((self.nverts, 2), np.float32)
        F = np.empty((self.nverts, 2), np.float32)
        check(self.lib.dpm2d_download(self.h, xy.ctypes.data, F.ctypes.data))
        return xy, F

    def download_ptr(self, xy_ptr: int, f_ptr: int = 0):
        check(self.lib.dpm2d_download(self.h, ctypes.c_void_p(xy_ptr),
                                      ctypes.c_void_p(f_ptr) if f_ptr else None))

    def contained(self):
        f = np.empty(self.nverts, np.uint8)
        check(self.lib.dpm2d_last_contained(self.h, f.ctypes.data_as(_c_ubyte_p)))
        return f

    def areas(self):
        a = np.empty(self.ncells, np.float32)
        check(self.lib.dpm2d_cell_areas(self.h, fptr(a)))
        return a

    def stats(self):
        r, f = ctypes.c_long(), ctypes.c_long()
        check(self.lib.dpm2d_stats(self.h, ctypes.byref(r), ctypes.byref(f)))
        return r.value, f.value

    def step_kernel(self, dt: float):
        check(self.lib.dpm2d_step_kernel(self.h, dt))

    def autotune(self, dt: float, trial_blocks: int = 2, use_cache: bool = True) -> dict:
        w, o, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        sk, ms = ctypes.c_float(), ctypes.c_float()
        check(self.lib.dpm2d_autotune(self.h, dt, trial_blocks, int(use_cache), ctypes.byref(w),
                                      ctypes.byref(o), ctypes.byref(p), ctypes.byref(sk),
                                      ctypes.byref(ms)))
        return {"warps": w.value, "occupancy": o.value, "rebuild_period": p.value,
                "skin_rel": round(sk.value, 4), "ms_per_step": round(ms.value, 5)}

    def rebuild_now(self):
        check(self.lib.dpm2d_rebuild_now(self.h))

    def cell_list(self):
        n = self.ncells
        keys = np.empty(n, np.uint32)
        ids = np.empty(n, np.uint32)
        nn = np.empty(n, np.int32)
        maxnb = ctypes.c_int()
        # first query the capacity
        check(self.lib.dpm2d_cell_list(self.h, None, None, None, None, ctypes.byref(maxnb), None))
        nbr = np.empty(n * maxnb.value, np.int32)
        geom = np.empty((n, 8), np.float32)
        check(self.lib.dpm2d_cell_list(self.h, keys.ctypes.data_as(_c_uint_p),
                                       ids.ctypes.data_as(_c_uint_p),
                                       nn.ctypes.data_as(_c_int_p), nbr.ctypes.data_as(_c_int_p),
                                       ctypes.byref(maxnb), fptr(geom)))
        return keys, ids, nn, nbr.reshape(n, maxnb.value), geom

    def bins(self):
        lb = ctypes.c_int()
        nb = np.empty(self.ntissues, np.int32)
        bw = np.empty(self.ntissues, np.float32)
        sk = np.empty(self.ntissues, np.float32)
        check(self.lib.dpm2d_bins(self.h, ctypes.byref(lb), nb.ctypes.data_as(_c_int_p), fptr(bw),
                                  fptr(sk)))
        return lb.value, nb, bw, sk

    def close(self):
        if self.h:
            self.lib.dpm2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch3D:
    """dpm3d_batch: independent 3D tissues sharing one mesh topology."""

    def __init__(self, ctx: Context, ncells, faces, nv: int):
        self.ctx = ctx
        self.lib = ctx.lib
        nc = np.ascontiguousarray(ncells, dtype=np.int32)
        f = np.ascontiguousarray(faces, dtype=np.uint32)
        h = _vp()
        check(self.lib.dpm3d_create(ctx.h, len(nc), nc.ctypes.data_as(_c_int_p), nv, len(f),
                                    f.ctypes.data_as(_c_uint_p), ctypes.byref(h)))
        self.h = h
        self.ntissues = len(nc)
        self.ncells = int(nc.sum())
        self.nv = nv
        self.nverts = self.ncells * nv

    def set_cells(self, Kv, Ka, Ks, v0, a0, l0, Kb=None, adh=None):
        arrs = [_f32(x) for x in (Kv, Ka, Ks, v0, a0, l0)]
        kb = None if Kb is None else _f32(Kb)
        ad = None if adh is None else _f32(adh)
        check(self.lib.dpm3d_set_cells(self.h, *[fptr(x) for x in arrs],
                                       None if kb is None else fptr(kb),
                                       None if ad is None else fptr(ad)))

    def set_tissues(self, L, Kre, pbc):
        L, Kre = (_f32(np.broadcast_to(x, (self.ntissues,))) for x in (L, Kre))
        p = np.ascontiguousarray(np.broadcast_to(pbc, (self.ntissues,)), dtype=np.int32)
        check(self.lib.dpm3d_set_tissues(self.h, fptr(L), fptr(Kre), p.ctypes.data_as(_c_int_p)))

    def set_attraction(self, Kat):
        """Opt-in AllVertAttraction with strength Kat per tissue (0 = off)."""
        Kat = _f32(np.broadcast_to(Kat, (self.ntissues,)))
        check(self.lib.dpm3d_set_attraction(self.h, fptr(Kat)))

    def set_tuning(self, rebuild_period=0, skin_rel=0.0):
        check(self.lib.dpm3d_set_tuning(self.h, rebuild_period, skin_rel))

    def set_block_threads(self, threads: int = 0):
        """Threads per cell of the step kernel (128, 256, 512; 0: default)."""
        check(self.lib.dpm3d_set_block_threads(self.h, threads))

    def upload(self, xyz):
        xyz = _f32(xyz)
        assert xyz.size == 3 * self.nverts
        check(self.lib.dpm3d_upload(self.h, xyz.ctypes.data))

    def step(self, nsteps: int, dt: float):
        check(self.lib.dpm3d_step(self.h, nsteps, dt))

    def download(self):
        xyz = np.empty((self.nverts, 3), np.float32)
        F = np.empty((self.nverts, 3), np.float32)
        check(self.lib.dpm3d_download(self.h, xyz.ctypes.data, F.ctypes.data))
        return xyz, F

    def winding(self):
        f = np.empty(self.nverts, np.uint8)
        check(self.lib.dpm3d_last_winding(self.h, f.ctypes.data_as(_c_ubyte_p)))
        return f

    def device_state(self):
        """Zero-copy torch views (nverts,) of x, y, z and of the last step's
        force components on the device; valid until the next step or
        upload."""
        ptrs = [_vp() for _ in range(6)]
        check(self.lib.dpm3d_device_state(self.h, *[ctypes.byref(p) for p in ptrs]))
        return tuple(_torch_view(p.value, (self.nverts,), self, self.ctx.device) for p in ptrs)

    def save(self, path: str):
        check(self.lib.dpm3d_save(self.h, os.fsencode(path)))

    @classmethod
    def open(cls, ctx: Context, path: str) -> "Batch3D":
        """A batch restored from a checkpoint written by save()."""
        T, nc, nv = _ckpt_shape(path, 3)
        h = _vp()
        check(ctx.lib.dpm3d_open(ctx.h, os.fsencode(path), ctypes.byref(h)))
        b = cls.__new__(cls)
        b.ctx, b.lib, b.h = ctx, ctx.lib, h
        b.ntissues, b.ncells, b.nv = T, int(nc.sum()), nv
        b.nverts = b.ncells * nv
        return b

    def diagnostics(self) -> dict:
        """Per cell volume, surface area and energy (double, on the device)."""
        d = ctypes.POINTER(ctypes.c_double)
        v, a, e = (np.zeros(self.ncells) for _ in range(3))
        check(self.lib.dpm3d_diagnostics(self.h, *[x.ctypes.data_as(d) for x in (v, a, e)]))
        return {"volume": v, "surface_area": a, "energy": e}

    def close(self):
        if self.h:
            self.lib.dpm3d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def disperse(ctx: Context, ncells, radius, L, X, Y):
    """dpm_disperse: relaxed centres (X, Y) and iteration counts of
    len(ncells) systems, one thread block each."""
    nc = np.ascontiguousarray(ncells, dtype=np.int32)
    r = _f32(radius)
    Ls = _f32(np.broadcast_to(L, (len(nc),)))
    x = _f32(X).copy()
    y = _f32(Y).copy()
    it = np.zeros(len(nc), np.int32)
    check(ctx.lib.dpm_disperse(ctx.h, len(nc), nc.ctypes.data_as(_c_int_p), fptr(r), fptr(Ls),
                               fptr(x), fptr(y), it.ctypes.data_as(_c_int_p)))
    return x, y, it


class Server:
    """dpm_server: continuous batching of independent tissue simulations on
    resident slot pools (see dpm_serve_* in dpm_gb300.h)."""

    def __init__(self, ctx: Context, hbm_budget_bytes: int, chunk_steps: int = 256):
        self.ctx = ctx
        self.lib = ctx.lib
        h = _vp()
        check(self.lib.dpm_serve_create(ctx.h, int(hbm_budget_bytes), chunk_steps,
                                        ctypes.byref(h)))
        self.h = h
        self._shape = {}

    def add_pool2d(self, slots: int, cells_per_slot: int, nv_max: int, dt: float):
        check(self.lib.dpm_serve_add_pool2d(self.h, slots, cells_per_slot, nv_max, dt))

    def add_pool3d(self, slots: int, cells_per_slot: int, faces, nv: int, dt: float):
        f = np.ascontiguousarray(faces, dtype=np.uint32)
        check(self.lib.dpm_serve_add_pool3d(self.h, slots, cells_per_slot, nv, len(f),
                                            f.ctypes.data_as(_c_uint_p), dt))

    def pool_bytes(self) -> int:
        v = ctypes.c_size_t()
        check(self.lib.dpm_serve_pool_bytes(self.h, ctypes.byref(v)))
        return v.value

    def submit2d(self, nv, Ka, Kl, Kb, a0, l0, r0, xy, L, Kre, Kat, pbc, nsteps, dt) -> int:
        nvu = np.ascontiguousarray(nv, dtype=np.uint32)
        arrs = [_f32(x) for x in (Ka, Kl, Kb, a0, l0, r0, xy)]
        rid = ctypes.c_uint64()
        check(self.lib.dpm_serve_submit2d(self.h, len(nvu), nvu.ctypes.data_as(_c_uint_p),
                                          *[fptr(a) for a in arrs], L, Kre, Kat, int(pbc),
                                          nsteps, dt, ctypes.byref(rid)))
        self._shape[rid.value] = (int(nvu.sum()), 2)
        return rid.value

    def submit3d(self, nv, Kv, Ka, Ks, v0, a0, l0, xyz, L, Kre, pbc, nsteps, dt, Kb=None,
                 adh=None) -> int:
        arrs = [_f32(x) for x in (Kv, Ka, Ks, v0, a0, l0)]
        kb = None if Kb is None else _f32(Kb)
        ad = None if adh is None else _f32(adh)
        x = _f32(xyz)
        rid = ctypes.c_uint64()
        check(self.lib.dpm_serve_submit3d(self.h, len(arrs[0]), nv, *[fptr(a) for a in arrs],
                                          None if kb is None else fptr(kb),
                                          None if ad is None else fptr(ad), fptr(x), L, Kre,
                                          int(pbc), nsteps, dt, ctypes.byref(rid)))
        self._shape[rid.value] = (x.size // 3, 3)
        return rid.value

    def step(self):
        """Advances until some pool completes a chunk; returns (active,
        waiting, finished by this call)."""
        a, w, f = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self.lib.dpm_serve_step(self.h, ctypes.byref(a), ctypes.byref(w), ctypes.byref(f)))
        return a.value, w.value, f.value

    def drain(self):
        check(self.lib.dpm_serve_drain(self.h))

    def status(self, rid: int) -> int:
        st = ctypes.c_int()
        check(self.lib.dpm_serve_result(self.h, rid, None, None, None, ctypes.byref(st)))
        return st.value

    def result(self, rid: int):
        """(positions, forces, latency_s) of a finished request, else None."""
        n, d = self._shape[rid]
        x = np.empty((n, d), np.float32)
        F = np.empty((n, d), np.float32)
        lat = ctypes.c_double()
        st = ctypes.c_int()
        check(self.lib.dpm_serve_result(self.h, rid, fptr(x), fptr(F), ctypes.byref(lat),
                                        ctypes.byref(st)))
        if st.value != 2:
            return None
        return x, F, lat.value

    def forget(self, rid: int):
        check(self.lib.dpm_serve_forget(self.h, rid))
        self._shape.pop(rid, None)

    def stats(self):
        vs = ctypes.c_double()
        rb = ctypes.c_size_t()
        check(self.lib.dpm_serve_stats(self.h, ctypes.byref(vs), ctypes.byref(rb)))
        return vs.value, rb.value

    def close(self):
        if self.h:
            self.lib.dpm_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
