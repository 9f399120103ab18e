"""AllVertAttraction, the reference's 3D vertex-pair attraction
(shaders/Cell3D_Kernel.cl:313-364), which its own step loop never enqueues:
opt-in here (dpm3d_set_attraction, Tissue3D.AllVertAttraction).  The CUDA
step against the oracle, through the C ABI; the oracle's attraction is
pinned to the reference kernel itself in test_oracle_golden.py.

Tolerances (FP32), as for the 3D step: forces of one step within 1e-5 of
the oracle's norm; positions after N steps within 1e-4.  The terms are the
reference's arithmetic pair by pair; only the order in which a vertex sums
its pairs differs.
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


def pos_err(x, ref):
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1.0)))


def run_both(ctx, s, nsteps):
    b = gpu_batch3d(ctx, [s])
    b.step(nsteps, DT)
    x, F = b.download()
    r = s.copy()
    rF, _ = port().run3d(r, nsteps, DT)
    return x, F, r.xyz, rF


def attraction_share(s):
    """Norm of the one-step force change that the attraction makes."""
    a, b = s.copy(), s.copy()
    b.Kat = 0.0
    Fa, _ = port().run3d(a, 1, DT)
    Fb, _ = port().run3d(b, 1, DT)
    return float(np.linalg.norm(Fa - Fb) / np.linalg.norm(Fa))


@pytest.mark.parametrize("seed", [0, 1])
def test_one_step_level2(ctx, seed):
    s = make_tissue3d(6, level=2, phi0=0.5, seed=seed)
    s.Kat = 0.5
    assert attraction_share(s) > 1e-2  # the attraction is exercised
    x, F, rx, rF = run_both(ctx, s, 1)
    assert rel_norm_err(F, rF) <= F_TOL
    assert pos_err(x, rx) <= X_TOL


def test_steps_level2(ctx):
    s = make_tissue3d(5, level=2, phi0=0.45, seed=4)
    s.Kat = 0.3
    x, F, rx, rF = run_both(ctx, s, 20)
    assert pos_err(x, rx) <= X_TOL


def test_monolayer_level3(ctx):
    import bench
    from opencl_dpm_gb300 import clDPM
    from oracle.oracle import Tissue3DState
    t = bench.build_monolayer(clDPM, np.random.default_rng(5), 16, 3)
    s = Tissue3DState(nv=t["nv"], faces=t["faces"], xyz=t["xyz"].copy(), Kv=t["Kv"], Ka=t["Ka"],
                      Ks=t["Ks"], v0=t["v0"], a0=t["a0"], l0=t["l0"], L=float(t["L"]), Kre=1.0,
                      pbc=1, Kb=t["Kb"], adh=t["adh"], Kat=0.2)
    assert attraction_share(s) > 1e-3
    x, F, rx, rF = run_both(ctx, s, 1)
    assert rel_norm_err(F, rF) <= F_TOL


def test_pairs_across_the_boundary(ctx):
    """Two cells touching through the periodic boundary in x and y."""
    s0 = make_tissue3d(2, level=2, phi0=0.3, seed=0)
    L = s0.L
    c = np.array([[0.6, 0.7, 1.0], [L - 0.9, L - 0.8, 1.0]], np.float32)
    s = make_tissue3d(2, level=2, phi0=0.3, centers=c)
    s.Kat = 0.6
    assert attraction_share(s) > 1e-2
    x, F, rx, rF = run_both(ctx, s, 1)
    assert rel_norm_err(F, rF) <= F_TOL


def test_small_box_every_pair(ctx):
    """A box too small for the image of the centres to serve every vertex
    pair: each pair takes its own nearest image, as in the reference."""
    s = make_tissue3d(2, level=2, phi0=0.55, seed=2)
    assert s.L < 4.5
    s.Kat = 0.4
    x, F, rx, rF = run_both(ctx, s, 1)
    assert rel_norm_err(F, rF) <= F_TOL


def test_off_by_default(ctx):
    """Kat alone has no effect, as in the reference; switching the
    attraction on through the host API changes the run and matches the
    oracle."""
    from opencl_dpm_gb300 import clDPM

    def run(kat, on):
        cells = []
        for k, (x0, y0) in enumerate([(0.0, 0.0), (1.9, 0.3), (0.8, 1.7)]):
            c = clDPM.Cell3D([x0, y0, 1.0], 1.05, 1.0)
            c.Kv, c.Ka, c.Ks = 1.0, 0.5, 0.1
            cells.append(c)
        T = clDPM.Tissue3D(cells, 0.5)
        T.Kre = 1.0
        T.Kat = kat
        T.AllVertAttraction = on
        T.CLEulerUpdate(3, DT)
        return np.concatenate([np.array(c.Verts, np.float32) for c in T.Cells])

    base = run(0.0, False)
    assert np.array_equal(run(0.7, False), base)
    on = run(0.7, True)
    assert not np.array_equal(on, base)


def test_checkpoint_keeps_attraction(ctx, tmp_path):
    from opencl_dpm_gb300.abi import Batch3D
    s = make_tissue3d(4, level=2, phi0=0.5, seed=7)
    s.Kat = 0.5
    b = gpu_batch3d(ctx, [s])
    b.step(2, DT)
    path = str(tmp_path / "att.ckpt")
    b.save(path)
    b.step(3, DT)
    x1, _ = b.download()
    b2 = Batch3D.open(ctx, path)
    b2.step(3, DT)
    x2, _ = b2.download()
    assert np.array_equal(x1, x2)


def test_checkpoint_without_attraction_section(ctx, tmp_path):
    """A 3D checkpoint that ends before the attraction section (as files
    written before it existed) opens with the attraction off."""
    from opencl_dpm_gb300.abi import Batch3D
    s = make_tissue3d(3, level=2, phi0=0.5, seed=9)
    b = gpu_batch3d(ctx, [s])
    b.step(2, DT)
    path = tmp_path / "old.ckpt"
    b.save(str(path))
    data = path.read_bytes()
    path.write_bytes(data[:-4 * 1])  # one tissue: drop its Kat
    b.step(3, DT)
    x1, _ = b.download()
    b2 = Batch3D.open(ctx, str(path))
    b2.step(3, DT)
    x2, _ = b2.download()
    assert np.array_equal(x1, x2)


def test_status_codes(ctx):
    """dpm3d_set_attraction needs the cells and tissues first and a finite
    strength."""
    from opencl_dpm_gb300.abi import Batch3D, DPMError
    s = make_tissue3d(2, level=2, phi0=0.5, seed=1)
    b = Batch3D(ctx, [s.ncells], s.faces, s.nv)
    with pytest.raises(DPMError) as e:
        b.set_attraction([0.5])             # cells and tissues not set
    assert e.value.code == 5
    b.set_cells(s.Kv, s.Ka, s.Ks, s.v0, s.a0, s.l0, None, None)
    b.set_tissues([s.L], [s.Kre], [s.pbc])
    with pytest.raises(DPMError) as e:
        b.set_attraction([float("nan")])
    assert e.value.code == 1
    b.set_attraction([0.5])
    b.upload(s.xyz)
    b.step(1, DT)
