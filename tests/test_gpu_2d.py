"""2D parity of the CUDA path against the oracle, through the C ABI.

Tolerances (FP32; the oracle reproduces the reference bit for bit):
  * forces of one step from the same positions:
    ||F - F_ref|| <= 1e-5 ||F_ref||
  * positions after 100 steps: max |x - x_ref| / max(|x_ref|, 1) <= 1e-4
  * containment flags (the reference's `overlaps`): identical.
Forces after many steps are compared by re-evaluating one step from the GPU's
positions on both sides: trajectories that differ by float rounding give
forces that differ by the spring stiffness times that drift, which is not
what the per-step criterion measures.
"""
import numpy as np
import pytest

from cases import gpu_batch2d, make_tissue2d, perturb, port, rel_norm_err

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
    F, flags = port().run2d(s, nsteps, dt)
    return s.xy, F, flags


def pos_err(xy, ref):
    return float(np.max(np.abs(xy - ref) / np.maximum(np.abs(ref), 1.0)))


def check_case(ctx, state, nsteps, tuning=None):
    b = gpu_batch2d(ctx, [state], tuning)
    b.step(nsteps, DT)
    xy, F = b.download()
    flags = b.contained()
    rx, rF, rflags = oracle_run(state, nsteps)
    return xy, F, flags, rx, rF, rflags


def step_force_err(ctx, state, xy):
    """One step from positions xy on both sides: force error and flag equality."""
    s = state.copy()
    s.xy = np.asarray(xy, np.float32).copy()
    b = gpu_batch2d(ctx, [s])
    b.step(1, DT)
    _, F = b.download()
    flags = b.contained()
    _, rF, rflags = oracle_run(s, 1)
    return rel_norm_err(F, rF), bool(np.array_equal(flags, rflags))


def test_one_step_c0(ctx):
    s = make_tissue2d(16, 32, phi=0.6, seed=0)
    xy, F, flags, rx, rF, rflags = check_case(ctx, s, 1)
    assert np.array_equal(flags, rflags)
    assert rel_norm_err(F, rF) <= F_TOL
    assert pos_err(xy, rx) <= X_TOL


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_100_steps_c0(ctx, seed):
    s = make_tissue2d(16, 32, phi=0.6, seed=seed)
    xy, F, flags, rx, rF, rflags = check_case(ctx, s, 100)
    assert np.array_equal(flags, rflags)
    assert pos_err(xy, rx) <= X_TOL
    ferr, same = step_force_err(ctx, s, xy)
    assert same and ferr <= F_TOL


def test_dense_overlaps(ctx):
    # crowded box: many vertices start inside neighbours
    s = make_tissue2d(40, 32, r0=1.0, calA=1.1, Kb=0.01, phi=0.9, seed=5)
    xy, F, flags, rx, rF, rflags = check_case(ctx, s, 1)
    assert rflags.sum() > 20
    assert np.array_equal(flags, rflags)
    assert rel_norm_err(F, rF) <= F_TOL
    xy, F, flags, rx, rF, rflags = check_case(ctx, s, 100)
    assert np.array_equal(flags, rflags)
    assert pos_err(xy, rx) <= X_TOL
    ferr, same = step_force_err(ctx, s, xy)
    assert same and ferr <= F_TOL


def test_ragged_attraction(ctx):
    rng = np.random.default_rng(3)
    n = 30
    nv = rng.choice([16, 24, 32, 48], size=n)
    r0 = rng.uniform(0.8, 1.4, size=n)
    s = make_tissue2d(n, nv, r0=r0, calA=rng.uniform(1.0, 1.2, n), Kb=0.02, phi=0.8,
                      Kat=0.5, seed=4)
    xy, F, flags, rx, rF, rflags = check_case(ctx, s, 1)
    assert np.array_equal(flags, rflags)
    assert rel_norm_err(F, rF) <= F_TOL
    xy, F, flags, rx, rF, rflags = check_case(ctx, s, 100)
    assert np.array_equal(flags, rflags)
    assert pos_err(xy, rx) <= X_TOL
    ferr, same = step_force_err(ctx, s, xy)
    assert same and ferr <= F_TOL


def test_large_nv(ctx):
    s = make_tissue2d(12, 100, r0=2.0, Kb=0.05, phi=0.7, seed=8)
    xy, F, flags, rx, rF, rflags = check_case(ctx, s, 1)
    assert np.array_equal(flags, rflags)
    assert rel_norm_err(F, rF) <= F_TOL
    xy, F, flags, rx, rF, rflags = check_case(ctx, s, 20)
    assert np.array_equal(flags, rflags)
    assert pos_err(xy, rx) <= X_TOL


def test_open_boundary(ctx):
    s = make_tissue2d(20, 32, phi=0.8, seed=9, pbc=0)
    xy, F, flags, rx, rF, rflags = check_case(ctx, s, 50)
    assert np.array_equal(flags, rflags)
    assert pos_err(xy, rx) <= X_TOL


def test_brute_force_path_matches(ctx):
    # rebuild every 2 steps with a tiny skin (lists go stale -> tissue scan)
    s = make_tissue2d(30, 32, phi=0.85, seed=11, Kb=0.01)
    xy1, F1, fl1, rx, rF, rflags = check_case(ctx, s, 40, tuning=dict(rebuild_period=2,
                                                                      skin_rel=1e-6))
    xy2, F2, fl2, *_ = check_case(ctx, s, 40, tuning=dict(rebuild_period=40, skin_rel=1e-6))
    assert np.array_equal(fl1, rflags) and np.array_equal(fl2, rflags)
    assert pos_err(xy1, rx) <= X_TOL and pos_err(xy2, rx) <= X_TOL
    # the lists only prune: the rebuild period and skin change no bit
    assert np.array_equal(xy1, xy2) and np.array_equal(F1, F2)


def test_batched_equals_alone(ctx):
    rng = np.random.default_rng(21)
    states = []
    for t in range(6):
        n = int(rng.integers(8, 40))
        nv = int(rng.choice([16, 24, 32, 48]))
        states.append(make_tissue2d(n, nv, calA=rng.uniform(1.0, 1.3, n),
                                    Kb=float(10 ** rng.uniform(-3, -1)),
                                    phi=float(rng.uniform(0.6, 0.9)), seed=100 + t))
    b = gpu_batch2d(ctx, states)
    b.step(60, DT)
    xy, F = b.download()
    off = 0
    for s in states:
        nvt = int(s.nv.sum())
        rx, rF, _ = oracle_run(s, 60)
        assert pos_err(xy[off:off + nvt], rx) <= X_TOL
        # same tissue alone on the GPU: identical bits (no cross-tissue effect)
        a = gpu_batch2d(ctx, [s])
        a.step(60, DT)
        ax, aF = a.download()
        assert np.array_equal(ax, xy[off:off + nvt])
        off += nvt


def test_mixed_slot_classes(ctx):
    """Tissues of different ring sizes in one batch run one kernel per
    vertex-slot class; a tissue with rings of 16 and 48 vertices belongs to
    the class of its largest ring (its cells hold neighbours of 48).  Every
    tissue equals itself alone, bit for bit, and the oracle (one step: flags
    identical, forces within tolerance)."""
    rng = np.random.default_rng(5)
    specs = [(24, rng.choice([16, 48], size=24), 0.5), (30, 16, 0.0), (20, 24, 0.3),
             (18, rng.choice([16, 24, 32], size=18), 0.0), (9, 100, 0.0)]
    states = [make_tissue2d(n, nv, r0=rng.uniform(0.9, 1.3, n), calA=rng.uniform(1.0, 1.2, n),
                            Kb=0.02, phi=0.82, Kat=kat, seed=60 + k)
              for k, (n, nv, kat) in enumerate(specs)]
    b = gpu_batch2d(ctx, states)
    b.step(1, DT)
    xy, F = b.download()
    flags = b.contained()
    b.step(29, DT)
    xy30, _ = b.download()
    off = 0
    for s in states:
        nvt = int(s.nv.sum())
        rx, rF, rflags = oracle_run(s, 1)
        assert np.array_equal(flags[off:off + nvt], rflags)
        assert rel_norm_err(F[off:off + nvt], rF) <= F_TOL
        a = gpu_batch2d(ctx, [s])
        a.step(30, DT)
        ax, _ = a.download()
        assert np.array_equal(ax, xy30[off:off + nvt])
        off += nvt


def test_deterministic(ctx):
    s = make_tissue2d(64, 32, phi=0.85, seed=13, Kb=0.01)
    out = []
    for _ in range(2):
        b = gpu_batch2d(ctx, [s])
        b.step(50, DT)
        out.append(b.download())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_cell_list_bit_exact(ctx):
    from host_celllist import host_rebuild
    rng = np.random.default_rng(17)
    states = [make_tissue2d(int(rng.integers(20, 200)), int(rng.choice([16, 32, 48])),
                            phi=float(rng.uniform(0.6, 0.9)), Kat=float(t % 2) * 0.3,
                            seed=200 + t) for t in range(5)]
    b = gpu_batch2d(ctx, states)
    b.step(37, DT)  # move the cells, then rebuild on the current positions
    b.rebuild_now()
    keys, ids, nn, nbr, geom = b.cell_list()
    local_bits, nbins, binw, skin = b.bins()
    tissues, tissue_of, l0 = [], [], []
    begin = 0
    for t, s in enumerate(states):
        n = len(s.nv)
        a0max = float(np.max(s.a0))
        cap = int(np.floor(np.float64(np.float32(s.L)) / max(np.sqrt(a0max / np.pi), 1e-6)))
        tissues.append(dict(L=np.float32(s.L), skin=np.float32(skin[t]), Kat=s.Kat, pbc=s.pbc,
                            l0max=np.float32(np.max(s.l0)), cap=max(1, min(cap, 1024)),
                            begin=begin, end=begin + n))
        tissue_of += [t] * n
        l0.append(s.l0)
        begin += n
    hk, hid, hnn, hnbr, hnb = host_rebuild(geom, tissue_of, tissues, np.concatenate(l0),
                                           local_bits)
    assert np.array_equal(hnb, nbins)
    assert np.array_equal(hk, keys)
    assert np.array_equal(hid, ids)
    assert np.array_equal(hnn, nn)
    for c in range(len(nn)):
        if nn[c] > 0:
            assert np.array_equal(hnbr[c, :nn[c]], nbr[c, :nn[c]])


def test_kernel_variants_identical(ctx):
    """Register cap and static/dynamic schedule change nothing in the results
    (the dynamic schedule's counters reset themselves between launches)."""
    rng = np.random.default_rng(31)
    states = [make_tissue2d(int(rng.integers(8, 60)), int(rng.choice([16, 32, 48])),
                            phi=float(rng.uniform(0.6, 0.9)), Kb=0.01, seed=200 + t)
              for t in range(5)]
    out = {}
    for variant in (0, 1, 2, 3, 8, 11, 40, 41):
        for warps in (4, 8, 16):
            b = gpu_batch2d(ctx, states, dict(warps=warps))
            b.set_kernel_variant(variant)
            b.step(40, DT)
            b.step(7, DT)
            out[(variant, warps)] = b.download()
    ref = out[(1, 8)]
    for k, (xy, F) in out.items():
        assert np.array_equal(xy, ref[0]) and np.array_equal(F, ref[1]), k


def test_team_cells_same_bits(ctx):
    """Four warps per cell (variant bit 5; no attraction): the warps split a
    cell's listed neighbours and OR their containment flags, which is the
    one-warp result bit for bit -- positions, forces and flags -- for rings
    of one and two slots in one batch, and the oracle's."""
    rng = np.random.default_rng(47)
    states = [make_tissue2d(150, 32, r0=rng.permutation(np.r_[np.ones(75), np.full(75, 1.4)]),
                            calA=rng.uniform(1.0, 1.2, 150), Kb=0.01, phi=0.85, seed=320),
              make_tissue2d(90, rng.choice([20, 48], size=90), calA=1.1, phi=0.8, seed=321),
              make_tissue2d(70, 16, phi=0.9, seed=322)]
    res = []
    for variant in (11, 40, 41):
        b = gpu_batch2d(ctx, states)
        b.set_kernel_variant(variant)
        b.step(40, DT)
        xy, F = b.download()
        res.append((xy, F, b.contained()))
    for r in res[1:]:
        assert all(np.array_equal(u, v) for u, v in zip(res[0], r))
    s = perturb(states[0], 0.05, 3)
    b = gpu_batch2d(ctx, [s])
    b.set_kernel_variant(41)
    b.step(1, DT)
    _, F = b.download()
    _, rF, rflags = oracle_run(s, 1)
    assert np.array_equal(b.contained(), rflags)
    assert rel_norm_err(F, rF) <= F_TOL


def test_resident_run_same_bits(ctx):
    """Batches of small tissues step with one block per tissue held in
    shared memory for the whole call; that run equals the graph path (variant
    bit 3 switches it off) bit for bit -- positions, last-step forces and
    containment flags -- with ragged rings, attraction, and a call longer
    than one resident launch (4,096 steps)."""
    rng = np.random.default_rng(41)
    states = [make_tissue2d(16, 32, phi=0.6, seed=300),
              make_tissue2d(40, rng.choice([16, 24, 32, 48], size=40), r0=rng.uniform(0.9, 1.3, 40),
                            calA=rng.uniform(1.0, 1.2, 40), Kb=0.02, phi=0.85, Kat=0.4, seed=301),
              make_tissue2d(9, 20, calA=1.1, phi=0.8, seed=302)]
    for nsteps in (1, 37, 4100):
        res = []
        for variant in (3, 11):
            b = gpu_batch2d(ctx, states)
            b.set_kernel_variant(variant)
            b.step(nsteps, DT)
            xy, F = b.download()
            res.append((xy, F, b.contained()))
        assert all(np.array_equal(u, v) for u, v in zip(res[0], res[1])), nsteps
    # and the oracle, one step from a perturbed state
    s = perturb(states[1], 0.05, 7)
    b = gpu_batch2d(ctx, [s])
    b.step(1, DT)
    _, F = b.download()
    _, rF, rflags = oracle_run(s, 1)
    assert np.array_equal(b.contained(), rflags)
    assert rel_norm_err(F, rF) <= F_TOL


def test_attraction_variant_same_bits(ctx):
    """A batch with one tissue using the attraction runs the step with the
    attraction compiled in; its other tissues (Kat = 0) must come out with
    the same bits as alone, where the smaller kernel without it runs."""
    states = [make_tissue2d(24, 24, phi=0.8, seed=40 + t, Kb=0.01) for t in range(3)]
    att = make_tissue2d(20, 32, phi=0.85, seed=50)
    att.Kat = 0.3
    b = gpu_batch2d(ctx, states + [att])
    b.step(40, DT)
    xy, _ = b.download()
    off = 0
    for s in states:
        nvt = int(s.nv.sum())
        a = gpu_batch2d(ctx, [s])
        a.step(40, DT)
        ax, _ = a.download()
        assert np.array_equal(ax, xy[off:off + nvt])
        off += nvt
    rx, _, _ = oracle_run(att, 40)
    assert pos_err(xy[off:], rx) <= X_TOL
