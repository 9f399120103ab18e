"""Serving (dpm_serve_*): continuous batching of independent requests.

The property under test is that a request's result does not depend on what
it shares the GPU with: every request is run through the server in a mix of
other requests (more requests than slots, so later ones join running pools
between chunks, and step budgets that end mid-chunk), and its final
positions and last-step forces must equal, bit for bit, those of the same
tissue run alone as a plain batch for the same number of steps.  One request
per dimension is also checked against the oracle (tolerances as in the
2D/3D parity tests).
"""
import numpy as np
import pytest

from cases import gpu_batch2d, gpu_batch3d, make_tissue2d, make_tissue3d, port

pytestmark = pytest.mark.gpu

DT = 0.005
X_TOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    from opencl_dpm_gb300.abi import Context
    return Context(0)


def pos_err(x, ref):
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1.0)))


def submit2d(srv, s, nsteps):
    return srv.submit2d(s.nv, s.Ka, s.Kl, s.Kb, s.a0, s.l0, s.r0, s.xy, s.L, s.Kre, s.Kat,
                        s.pbc, nsteps, DT)


def submit3d(srv, s, nsteps):
    return srv.submit3d(s.nv, s.Kv, s.Ka, s.Ks, s.v0, s.a0, s.l0, s.xyz, s.L, s.Kre, s.pbc,
                        nsteps, DT, Kb=s.Kb, adh=s.adh)


def drain(srv, ids, max_rounds=1000):
    trace = []
    for _ in range(max_rounds):
        a, w, f = srv.step()
        trace.append((a, w, f))
        if all(srv.status(i) == 2 for i in ids):
            return trace
    raise AssertionError("requests did not finish")


def alone2d(ctx, s, nsteps):
    b = gpu_batch2d(ctx, [s])
    b.step(nsteps, DT)
    return b.download()


def alone3d(ctx, s, nsteps):
    b = gpu_batch3d(ctx, [s])
    b.step(nsteps, DT)
    return b.download()


def requests2d(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for t in range(n):
        nc = int(rng.integers(6, 30))
        nv = int(rng.choice([16, 24, 32]))
        s = make_tissue2d(nc, nv, calA=rng.uniform(1.0, 1.2, nc),
                          Kb=float(10 ** rng.uniform(-3, -1)),
                          phi=float(rng.uniform(0.6, 0.9)), seed=seed + t)
        out.append((s, int(rng.integers(20, 140))))
    return out


def test_serve_2d_mix_equals_alone(ctx):
    from opencl_dpm_gb300.abi import Server
    reqs = requests2d(7, 300)
    srv = Server(ctx, hbm_budget_bytes=1 << 30, chunk_steps=32)
    srv.add_pool2d(slots=3, cells_per_slot=32, nv_max=32, dt=DT)
    srv.add_pool2d(slots=2, cells_per_slot=32, nv_max=48, dt=DT)
    ids = [submit2d(srv, s, n) for s, n in reqs]
    trace = drain(srv, ids)
    # five slots, seven requests: some waited and joined later
    assert sum(trace[0]) == 7 and trace[0][1] + trace[0][2] >= 2
    assert max(a for a, _, _ in trace) <= 5
    for rid, (s, n) in zip(ids, reqs):
        x, F, lat = srv.result(rid)
        ax, aF = alone2d(ctx, s, n)
        assert np.array_equal(x, ax) and np.array_equal(F, aF), (rid, n)
        assert lat > 0.0
    s, n = reqs[0]
    r = s.copy()
    port().run2d(r, n, DT)
    assert pos_err(srv.result(ids[0])[0], r.xy) <= X_TOL


def test_serve_3d_and_2d_pools_together(ctx):
    from opencl_dpm_gb300.abi import Server
    s3 = [make_tissue3d(int(n), level=2, phi0=0.5, seed=40 + int(n)) for n in (3, 5, 4)]
    steps3 = [10, 21, 16]
    reqs2 = requests2d(3, 500)
    srv = Server(ctx, hbm_budget_bytes=1 << 30, chunk_steps=16)
    srv.add_pool3d(slots=2, cells_per_slot=5, faces=s3[0].faces, nv=s3[0].nv, dt=DT)
    srv.add_pool2d(slots=2, cells_per_slot=32, nv_max=32, dt=DT)
    ids3 = [submit3d(srv, s, n) for s, n in zip(s3, steps3)]
    ids2 = [submit2d(srv, s, n) for s, n in reqs2]
    drain(srv, ids3 + ids2)
    for rid, s, n in zip(ids3, s3, steps3):
        x, F, _ = srv.result(rid)
        ax, aF = alone3d(ctx, s, n)
        assert np.array_equal(x.reshape(-1), ax.reshape(-1)), (rid, n)
        assert np.array_equal(F.reshape(-1), aF.reshape(-1)), (rid, n)
    for rid, (s, n) in zip(ids2, reqs2):
        x, F, _ = srv.result(rid)
        ax, aF = alone2d(ctx, s, n)
        assert np.array_equal(x, ax) and np.array_equal(F, aF)
    r = s3[1].copy()
    port().run3d(r, steps3[1], DT)
    assert pos_err(srv.result(ids3[1])[0].reshape(-1), r.xyz.reshape(-1)) <= X_TOL


def test_serve_admission_by_footprint(ctx):
    from opencl_dpm_gb300.abi import DPMError, Server
    reqs = [(make_tissue2d(12, 24, phi=0.8, seed=700 + t), 20 + 9 * t) for t in range(3)]
    # resident footprint of a 2D request: 25 bytes per vertex (positions
    # twice, forces, flags) and 548 per cell (constants, geometry, lists)
    fp = 25 * 12 * 24 + 548 * 12
    # a budget that holds one request but never two, with slots for three
    srv = Server(ctx, hbm_budget_bytes=fp + fp // 2, chunk_steps=16)
    srv.add_pool2d(slots=3, cells_per_slot=32, nv_max=32, dt=DT)
    ids = [submit2d(srv, s, n) for s, n in reqs]
    assert srv.step()[:2] == (1, 2)
    assert srv.stats()[1] == fp
    trace = drain(srv, ids)
    assert max(a for a, _, _ in trace) == 1
    for rid, (s, n) in zip(ids, reqs):
        x, F, _ = srv.result(rid)
        ax, aF = alone2d(ctx, s, n)
        assert np.array_equal(x, ax)
    # a request no pool can hold is refused at submit
    s = make_tissue2d(40, 32, seed=1)
    with pytest.raises(DPMError) as e:
        submit2d(srv, s, 10)
    assert e.value.code == 3
    srv.forget(ids[0])
    with pytest.raises(DPMError):
        srv.status(ids[0])
