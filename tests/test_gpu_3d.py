"""3D parity of the CUDA path against the oracle, through the C ABI.

Tolerances (FP32):
  * forces of one step from the same positions: ||F - F_ref|| <= 1e-5 ||F_ref||
  * positions after N steps: max |x - x_ref| / max(|x_ref|, 1) <= 1e-4
  * winding-number hit counts: equal, except where the oracle's own sum sits
    at the reference's 1e-6 threshold by rounding noise: at most 0.2% of the
    vertices may differ, and at least one is always allowed (a 5-cell tissue
    of icosahedra has 60 vertices, where 0.2% is less than one); their force
    contribution is ~1e-6 * Kc.
"""
import numpy as np
import pytest

from cases import gpu_batch3d, make_tissue3d, port, rel_norm_err

pytestmark = pytest.mark.gpu

DT = 0.005
F_TOL = 1e-5
X_TOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    from opencl_dpm_gb300.abi import Context
    return Context(0)


def oracle_run(state, nsteps, dt=DT):
    s = state.copy()
    F, wn = port().run3d(s, nsteps, dt)
    return s.xyz, F, wn


def pos_err(x, ref):
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1.0)))


def run_case(ctx, state, nsteps, tuning=None):
    b = gpu_batch3d(ctx, [state], tuning)
    b.step(nsteps, DT)
    x, F = b.download()
    wn = b.winding()
    rx, rF, rwn = oracle_run(state, nsteps)
    return x, F, wn, rx, rF, rwn


def wn_ok(a, b):
    """Hit counts equal except on at most max(1, 0.2% of the vertices)."""
    bad = int(np.count_nonzero(a != b))
    return bad <= max(1, int(2e-3 * a.size)), bad


@pytest.mark.parametrize("seed", [0, 1])
def test_one_step_level2(ctx, seed):
    s = make_tissue3d(6, level=2, phi0=0.5, seed=seed)
    x, F, wn, rx, rF, rwn = run_case(ctx, s, 1)
    assert rwn.sum() > 0  # the cells overlap: repulsion is exercised
    assert wn_ok(wn, rwn)[0], wn_ok(wn, rwn)
    assert rel_norm_err(F, rF) <= F_TOL
    assert pos_err(x, rx) <= X_TOL


def test_50_steps_level2(ctx):
    s = make_tissue3d(6, level=2, phi0=0.45, seed=3)
    x, F, wn, rx, rF, rwn = run_case(ctx, s, 50)
    assert pos_err(x, rx) <= X_TOL
    # forces of one step from the GPU's positions
    s2 = s.copy()
    s2.xyz = x.copy()
    b = gpu_batch3d(ctx, [s2])
    b.step(1, DT)
    _, F1 = b.download()
    _, rF1, _ = oracle_run(s2, 1)
    assert rel_norm_err(F1, rF1) <= F_TOL


def test_level3(ctx):
    s = make_tissue3d(4, level=3, phi0=0.5, seed=4)
    x, F, wn, rx, rF, rwn = run_case(ctx, s, 1)
    assert rel_norm_err(F, rF) <= F_TOL
    assert wn_ok(wn, rwn)[0], wn_ok(wn, rwn)
    x, F, wn, rx, rF, rwn = run_case(ctx, s, 10)
    assert pos_err(x, rx) <= X_TOL


def test_bending_and_adhesion_range(ctx):
    s = make_tissue3d(4, level=2, phi0=0.5, seed=5, Kb=0.05, adh=0.1)
    # squash the meshes a little so that bending is active
    s.xyz[:, 2] *= np.float32(0.9)
    x, F, wn, rx, rF, rwn = run_case(ctx, s, 1)
    assert rel_norm_err(F, rF) <= F_TOL
    x, F, wn, rx, rF, rwn = run_case(ctx, s, 20)
    assert pos_err(x, rx) <= X_TOL


def test_no_repulsion_and_open_box(ctx):
    s = make_tissue3d(5, level=2, phi0=0.5, seed=6, Kre=0.0, pbc=0)
    x, F, wn, rx, rF, rwn = run_case(ctx, s, 5)
    assert rel_norm_err(F, rF) <= F_TOL
    assert wn.sum() == 0


def test_batched_equals_alone_3d(ctx):
    states = [make_tissue3d(int(n), level=2, phi0=0.5, seed=10 + n) for n in (3, 5, 4)]
    b = gpu_batch3d(ctx, states)
    b.step(12, DT)
    x, F = b.download()
    off = 0
    for s in states:
        n = s.ncells * s.nv
        a = gpu_batch3d(ctx, [s])
        a.step(12, DT)
        ax, aF = a.download()
        assert np.array_equal(ax, x[off:off + n])
        rx, rF, _ = oracle_run(s, 12)
        assert pos_err(x[off:off + n], rx) <= X_TOL
        off += n


def test_deterministic_3d(ctx):
    s = make_tissue3d(6, level=2, phi0=0.5, seed=7)
    out = []
    for _ in range(2):
        b = gpu_batch3d(ctx, [s])
        b.step(10, DT)
        out.append(b.download())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_monolayer_level3_contacts(ctx):
    """A contact-rich monolayer at subdivision 3 (642 vertices, jittered
    hexagonal lattice, overlapping neighbours): the candidates go through
    every winding certificate (centre-direction support, inner ball, face
    plane) and the deferred full sums."""
    import bench
    from opencl_dpm_gb300 import clDPM
    from oracle.oracle import Tissue3DState
    t = bench.build_monolayer(clDPM, np.random.default_rng(11), 16, 3)
    s = Tissue3DState(nv=t["nv"], faces=t["faces"], xyz=t["xyz"].copy(), Kv=t["Kv"], Ka=t["Ka"],
                      Ks=t["Ks"], v0=t["v0"], a0=t["a0"], l0=t["l0"], L=float(t["L"]), Kre=1.0,
                      pbc=1, Kb=t["Kb"], adh=t["adh"])
    for nsteps in (1, 10):
        x, F, wn, rx, rF, rwn = run_case(ctx, s, nsteps)
        assert rwn.sum() > 100  # many vertices inside a neighbour
        assert wn_ok(wn, rwn)[0], wn_ok(wn, rwn)
        assert pos_err(x, rx) <= X_TOL
        if nsteps == 1:
            assert rel_norm_err(F, rF) <= F_TOL


@pytest.mark.parametrize("level", [2, 3])
def test_dense_overlap_block_sizes_same_bits(ctx, level):
    """Strongly overlapping cells (packing fraction 0.8 in the reference's
    box rule, random centres): each cell has many neighbours within winding
    reach and many vertices lie inside a neighbour.  512-thread blocks run
    the neighbour pipeline (two staging buffers, candidates from a shared
    counter), 256 and 128 threads the two-barrier loop: the same bits, and
    the same as the oracle within the parity criteria."""
    s = make_tissue3d(20, level=level, phi0=0.8, seed=40 + level, Kb=0.05, adh=0.1)
    out = {}
    for threads in (512, 256, 128):
        b = gpu_batch3d(ctx, [s])
        b.set_block_threads(threads)
        b.step(5, DT)
        x, F = b.download()
        out[threads] = (x, F, b.winding())
    x0, F0, w0 = out[512]
    assert w0.sum() > 200  # many hits
    for threads in (256, 128):
        x, F, w = out[threads]
        assert np.array_equal(x, x0) and np.array_equal(F, F0), threads
        assert np.array_equal(w, w0), threads
    x, F, wn, rx, rF, rwn = run_case(ctx, s, 1)
    assert wn_ok(wn, rwn)[0], wn_ok(wn, rwn)
    assert rel_norm_err(F, rF) <= F_TOL
    assert pos_err(x, rx) <= X_TOL


@pytest.mark.parametrize("level", [2, 3])
def test_block_sizes_same_bits(ctx, level):
    """128, 256 and 512 threads per cell (and the default) give the same
    bits: every block-wide sum is formed in the 512-thread order.  A
    contact-rich monolayer with bending and adhesion, and the opt-in
    attraction."""
    import bench
    from opencl_dpm_gb300 import clDPM
    from oracle.oracle import Tissue3DState
    t = bench.build_monolayer(clDPM, np.random.default_rng(21), 12, level)
    s = Tissue3DState(nv=t["nv"], faces=t["faces"], xyz=t["xyz"].copy(), Kv=t["Kv"], Ka=t["Ka"],
                      Ks=t["Ks"], v0=t["v0"], a0=t["a0"], l0=t["l0"], L=float(t["L"]), Kre=1.0,
                      pbc=1, Kb=t["Kb"], adh=t["adh"])
    for kat in (0.0, 0.05):
        s.Kat = kat
        out = {}
        for threads in (512, 256, 128, 0):
            b = gpu_batch3d(ctx, [s])
            b.set_block_threads(threads)
            b.step(10, DT)
            x, F = b.download()
            out[threads] = (x, F, b.winding())
        x0, F0, w0 = out[512]
        assert w0.sum() > 0
        for threads in (256, 128, 0):
            x, F, w = out[threads]
            assert np.array_equal(x, x0) and np.array_equal(F, F0), (kat, threads)
            assert np.array_equal(w, w0), (kat, threads)
    with pytest.raises(Exception):
        b.set_block_threads(384)


def test_tuning_same_bits_3d(ctx):
    """The rebuild period and skin change only the neighbour lists, which
    only prune: the same bits (a stale list falls back to the tissue scan)."""
    s = make_tissue3d(6, level=2, phi0=0.5, seed=12)
    out = []
    for tuning in (dict(rebuild_period=1, skin_rel=1e-6), dict(rebuild_period=8, skin_rel=0.1),
                   dict(rebuild_period=16, skin_rel=1e-6)):
        b = gpu_batch3d(ctx, [s], tuning)
        b.step(16, DT)
        x, F = b.download()
        out.append((x, F, b.winding()))
    assert out[0][2].sum() > 0
    for x, F, w in out[1:]:
        assert np.array_equal(x, out[0][0]) and np.array_equal(F, out[0][1])
        assert np.array_equal(w, out[0][2])


def test_larger_mesh_after_smaller(ctx):
    """A batch of a larger mesh still steps after a batch of a smaller mesh
    was made (the step's shared-memory limit is shared by all batches)."""
    s3 = make_tissue3d(2, level=3, phi0=0.5, seed=5)
    b3 = gpu_batch3d(ctx, [s3])
    s2 = make_tissue3d(2, level=2, phi0=0.5, seed=5)
    b2 = gpu_batch3d(ctx, [s2])
    b3.step(2, DT)
    b2.step(2, DT)
    x3, _ = b3.download()
    r = s3.copy()
    port().run3d(r, 2, DT)
    assert pos_err(x3, r.xyz) <= X_TOL


@pytest.mark.parametrize("level", [0, 1])
def test_coarse_meshes(ctx, level):
    """Icosahedron (12 vertices) and subdivision 1 (42): a single vertex
    patch or two, few edges."""
    s = make_tissue3d(5, level=level, phi0=0.6, seed=20 + level)
    for nsteps in (1, 10):
        x, F, wn, rx, rF, rwn = run_case(ctx, s, nsteps)
        assert wn_ok(wn, rwn)[0], wn_ok(wn, rwn)
        assert pos_err(x, rx) <= X_TOL
        if nsteps == 1:
            assert rel_norm_err(F, rF) <= F_TOL
