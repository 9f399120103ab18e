"""Edge cases of the 2D/3D paths: argument and state errors (the C ABI's
status codes), empty and single-cell tissues, the largest ring, tissues whose
vertices drifted several box lengths away (the reference never wraps
positions, so its floor/round offset shifts see large offsets), and cells
overlapping across a corner of the periodic box.  Physics cases are checked
against the oracle with the tolerances of test_gpu_2d.py."""
import numpy as np
import pytest

from cases import gpu_batch2d, make_tissue2d, make_tissue3d, gpu_batch3d, port, rel_norm_err

pytestmark = pytest.mark.gpu

DT = 0.005
X_TOL = 1e-4
F_TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    from opencl_dpm_gb300.abi import Context
    return Context(0)


def pos_err(x, ref):
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1.0)))


def oracle(state, nsteps):
    s = state.copy()
    F, flags = port().run2d(s, nsteps, DT)
    return s.xy, F, flags


def test_status_codes(ctx):
    from opencl_dpm_gb300.abi import Batch2D, DPMError
    with pytest.raises(DPMError) as e:
        Batch2D(ctx, [2], [16, 2])           # a ring needs 3 vertices
    assert e.value.code == 1
    with pytest.raises(DPMError) as e:
        Batch2D(ctx, [1], [257])             # more than 256 vertices
    assert e.value.code in (1, 3)
    with pytest.raises(DPMError) as e:
        Batch2D(ctx, [0], np.zeros(0, np.uint32))  # empty tissue
    assert e.value.code == 1
    b = Batch2D(ctx, [1], [16])
    with pytest.raises(DPMError) as e:
        b.step(1, DT)                        # nothing set or uploaded
    assert e.value.code == 5
    s = make_tissue2d(1, 16, seed=1)
    b.set_cells(s.Ka, s.Kl, s.Kb, s.a0, s.l0, s.r0)
    b.set_tissues([s.L], [s.Kre], [s.Kat], [1])
    b.upload(s.xy)
    with pytest.raises(DPMError) as e:
        b.step(-1, DT)
    assert e.value.code == 1
    with pytest.raises(DPMError) as e:
        b.step(1, float("nan"))
    assert e.value.code == 1
    b.step(0, DT)                            # zero steps: nothing changes
    x, _ = b.download()
    assert np.array_equal(x, s.xy.reshape(-1, 2))
    bad = s.xy.copy()
    bad[0, 0] = np.inf
    b.upload(bad)
    b.step(1, DT)
    with pytest.raises(DPMError) as e:
        b.download()
    assert e.value.code == 4


def test_single_cell_and_largest_ring(ctx):
    # 256-vertex rings have short stiff edges: the reference's explicit
    # Euler diverges at dt = 0.005 within 30 steps, so they step at 0.001
    for s, dt in ((make_tissue2d(1, 32, calA=1.2, Kb=0.05, seed=2), DT),
                  (make_tissue2d(3, 256, calA=1.1, Kb=0.01, phi=0.8, seed=3), 0.001)):
        b = gpu_batch2d(ctx, [s])
        b.step(30, dt)
        x, F = b.download()
        r = s.copy()
        port().run2d(r, 30, dt)
        assert pos_err(x, r.xy) <= X_TOL


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_drifted_tissue(ctx, seed):
    """Cells moved to other periodic images (whole multiples of L, up to two
    box lengths per axis) and the whole tissue translated: offsets between
    cells of up to a few L, the reference's per-edge floor (x) and round (y)
    shifts, the far-pair paths and large coordinates."""
    s = make_tissue2d(24, 24, calA=1.15, Kb=0.01, phi=0.85, seed=4)
    rng = np.random.default_rng(40 + seed)
    img = rng.integers(-2, 3, size=(24, 2)).astype(np.float32)
    img[0] = 0.0
    per_vertex = np.repeat(img, s.nv.astype(np.int64), axis=0) * np.float32(s.L)
    xy = s.xy.reshape(-1, 2) + per_vertex + np.float32(s.L) * np.float32(seed * 1.7)
    s.xy = xy.astype(np.float32).reshape(s.xy.shape)
    b = gpu_batch2d(ctx, [s])
    b.step(40, DT)
    x, F = b.download()
    rx, rF, rflags = oracle(s, 40)
    assert pos_err(x, rx) <= X_TOL
    # one step from the same positions: forces and flags
    s2 = s.copy()
    s2.xy = x.reshape(s.xy.shape).copy()
    b2 = gpu_batch2d(ctx, [s2])
    b2.step(1, DT)
    _, F1 = b2.download()
    _, rF1, rfl1 = oracle(s2, 1)
    assert rel_norm_err(F1, rF1) <= F_TOL
    assert np.array_equal(b2.contained(), rfl1)


def test_corner_overlaps(ctx):
    """Cells centred on the four corners of the box overlap through both
    periodic directions at once."""
    L = 6.0
    centres = np.array([[0.2, 0.1], [L - 0.3, 0.2], [0.1, L - 0.2], [L - 0.2, L - 0.1],
                        [L / 2, L / 2]], np.float32)
    s = make_tissue2d(5, 32, calA=1.2, Kb=0.01, phi=0.8, seed=5, centers=centres)
    scale = np.float32(L / s.L)
    s.xy = (s.xy * scale).astype(np.float32)
    s.L = float(L)
    b = gpu_batch2d(ctx, [s])
    b.step(1, DT)
    _, F = b.download()
    _, rF, rflags = oracle(s, 1)
    assert rel_norm_err(F, rF) <= F_TOL
    assert np.array_equal(b.contained(), rflags)
    b = gpu_batch2d(ctx, [s])
    b.step(50, DT)
    x, _ = b.download()
    rx, _, _ = oracle(s, 50)
    assert pos_err(x, rx) <= X_TOL


def test_3d_single_cell_and_far_neighbours(ctx):
    s = make_tissue3d(1, level=2, phi0=0.5, seed=6)
    b = gpu_batch3d(ctx, [s])
    b.step(5, DT)
    x, F = b.download()
    r = s.copy()
    rF, _ = port().run3d(r, 5, DT)
    assert pos_err(x.reshape(-1), r.xyz.reshape(-1)) <= X_TOL
    # two cells a box length apart: neighbours only through the periodic box
    s = make_tissue3d(2, level=2, phi0=0.5, seed=7,
                      centers=np.array([[0.3, 0.3, 1.0], [0.3, 0.3, 1.0]], np.float32))
    s.xyz = s.xyz.copy()
    s.xyz[s.nv:, 0] += np.float32(s.L - 0.5)
    b = gpu_batch3d(ctx, [s])
    b.step(5, DT)
    x, F = b.download()
    r = s.copy()
    port().run3d(r, 5, DT)
    assert pos_err(x.reshape(-1), r.xyz.reshape(-1)) <= X_TOL


@pytest.mark.parametrize("nv", [100, 200])
def test_large_rings_with_attraction(ctx, nv):
    """Rings of more than 64 vertices (4 and 8 slots per lane) with the
    attraction compiled in, against the oracle."""
    s = make_tissue2d(6, nv, calA=1.1, Kb=0.01, phi=0.85, Kat=0.4, seed=nv)
    for steps in (1, 20):
        b = gpu_batch2d(ctx, [s])
        b.step(steps, 0.001)
        x, F = b.download()
        r = s.copy()
        rF, _ = port().run2d(r, steps, 0.001)
        assert pos_err(x, r.xy) <= X_TOL
        if steps == 1:
            assert rel_norm_err(F, rF) <= F_TOL
