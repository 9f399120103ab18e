"""dpm2d_step_noalloc: the 2D step for callers that cannot allocate device
memory (their device memory belongs to another framework's pool, or they must
not synchronize the device the way cudaMalloc/cudaFree can).

The entry point works in a fixed array inside the library and the caller's
own device buffers.  Its results must equal those of the ordinary batch
entry points (dpm2d_create/upload/step/download) on the same inputs, within
the 2D parity tolerances, over two calls in a row on different tissues (the
second call must not see anything left in the shared array by the first).
"""
import ctypes

import numpy as np
import pytest

from cases import gpu_batch2d, make_tissue2d, rel_norm_err

DT = 0.005
F_TOL = 1e-5
X_TOL = 1e-4

_f = ctypes.POINTER(ctypes.c_float)
_u = ctypes.POINTER(ctypes.c_uint)


def noalloc_fn():
    from opencl_dpm_gb300.abi import load
    fn = load().dpm2d_step_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, _u] + [_f] * 6 + [ctypes.c_float] * 3 + [ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                   ctypes.c_void_p]
    return fn


def call_noalloc(fn, s, xy_dev, F_dev, nsteps, stream=None):
    arrs = [np.ascontiguousarray(getattr(s, k), np.float32)
            for k in ("Ka", "Kl", "Kb", "a0", "l0", "r0")]
    nv = np.ascontiguousarray(s.nv, np.uint32)
    return fn(len(nv), nv.ctypes.data_as(_u), *[a.ctypes.data_as(_f) for a in arrs], s.L, s.Kre,
              s.Kat, int(s.pbc), xy_dev, F_dev, nsteps, DT, stream)


def batch_run(ctx, s, nsteps):
    b = gpu_batch2d(ctx, [s])
    b.step(nsteps, DT)
    return b.download()


@pytest.mark.gpu
def test_noalloc_matches_batch_entry_two_calls():
    import torch
    from opencl_dpm_gb300.abi import Context
    ctx = Context(0)
    fn = noalloc_fn()
    cases = [(make_tissue2d(40, 32, phi=0.85, Kb=0.01, seed=31), 20),
             (make_tissue2d(25, 24, r0=1.2, calA=1.1, phi=0.8, Kat=0.3, seed=32), 13)]
    for s, nsteps in cases:
        rx, rF = batch_run(ctx, s, nsteps)
        xy = torch.from_numpy(s.xy.copy()).to("cuda:0")
        F = torch.zeros_like(xy)
        torch.cuda.synchronize()
        rc = call_noalloc(fn, s, xy.data_ptr(), F.data_ptr(), nsteps)
        assert rc == 0, ctx.lib.dpm_last_error().decode()
        x_out = xy.cpu().numpy()
        F_out = F.cpu().numpy()
        assert float(np.max(np.abs(x_out - rx) / np.maximum(np.abs(rx), 1.0))) <= X_TOL
        assert rel_norm_err(F_out, rF) <= F_TOL


def test_noalloc_rejects_oversize():
    from opencl_dpm_gb300.abi import load
    fn = noalloc_fn()
    n = 2049
    s = make_tissue2d(2, 16, seed=0)
    one = np.ones(n, np.float32)
    nv = np.full(n, 16, np.uint32)
    # sizes are checked on the host before any device work, so the position
    # buffer is never touched here
    dummy = np.zeros(2, np.float32)
    rc = fn(n, nv.ctypes.data_as(_u), *[one.ctypes.data_as(_f)] * 6, 10.0, 1.0, 0.0, 1,
            dummy.ctypes.data, None, 1, DT, None)
    assert rc == 3  # DPM_ECAPACITY
    assert b"2048" in load().dpm_last_error()


@pytest.mark.gpu
def test_noalloc_on_own_stream_against_oracle():
    """A caller that must not synchronize the whole device passes its own
    non-blocking stream (here a torch stream's handle); the result also
    matches the oracle directly.  nsteps == 0 leaves the buffers alone."""
    import torch
    from cases import port
    fn = noalloc_fn()
    s = make_tissue2d(30, 32, phi=0.85, Kb=0.02, seed=33)
    st = torch.cuda.Stream(device=0)
    xy = torch.from_numpy(s.xy.copy()).to("cuda:0")
    F = torch.full_like(xy, 7.0)
    torch.cuda.synchronize()
    assert call_noalloc(fn, s, xy.data_ptr(), F.data_ptr(), 0, st.cuda_stream) == 0
    assert np.array_equal(xy.cpu().numpy(), s.xy) and bool(torch.all(F == 7.0))
    assert call_noalloc(fn, s, xy.data_ptr(), F.data_ptr(), 25, st.cuda_stream) == 0
    r = s.copy()
    rF, _ = port().run2d(r, 25, DT)
    x_out = xy.cpu().numpy()
    assert float(np.max(np.abs(x_out - r.xy) / np.maximum(np.abs(r.xy), 1.0))) <= X_TOL
    # forces of one step from the device's positions, against the oracle
    s1 = s.copy()
    s1.xy = x_out.copy()
    assert call_noalloc(fn, s1, xy.data_ptr(), F.data_ptr(), 1, st.cuda_stream) == 0
    r1 = s1.copy()
    rF1, _ = port().run2d(r1, 1, DT)
    assert rel_norm_err(F.cpu().numpy(), rF1) <= F_TOL
