"""Pin of the oracle's 3D triangle bending (an extension: the reference has
no 3D bending, so nothing of the reference can pin it).

The oracle's bending force (`bend3d` in oracle/dpm_oracle.c, float) must be
minus the gradient of its bending energy E = kb * sum over edges of
(1 - n1.n2) (`orc_bend_energy3d`, double), taken by FP64 central finite
differences, on deformed icospheres of subdivision 2 and 3.  Every other
force is switched off (kv = ka = ks = kc = 0, the mesh far above the
substrate), so the oracle's step forces are the bending forces alone.
The GPU's bending force is checked against this oracle in the 3D tests."""
import numpy as np
import pytest

from cases import make_tissue3d, port

KB = 0.05


def deformed_cell(level, seed):
    s = make_tissue3d(1, level=level, Kv=0.0, Ka=0.0, Ks=0.0, Kre=0.0, Kb=KB, seed=seed, pbc=0)
    rng = np.random.default_rng(seed)
    c = s.xyz.mean(axis=0)
    d = (s.xyz - c) * (1.0 + 0.05 * rng.standard_normal((len(s.xyz), 1)))
    d *= np.array([1.2, 0.9, 0.8])
    s.xyz = (c + d + np.array([0.0, 0.0, 5.0])).astype(np.float32)
    return s


@pytest.mark.parametrize("level,seed", [(2, 1), (2, 2), (3, 3)])
def test_bending_force_is_minus_energy_gradient(level, seed):
    P = port()
    s = deformed_cell(level, seed)
    F, _ = P.run3d(s.copy(), 1, 0.002)
    x = s.xyz.astype(np.float64)
    fd = np.zeros_like(x)
    for v in range(len(x)):
        for k in range(3):
            h = 1e-6 * max(1.0, abs(x[v, k]))
            xp, xm = x.copy(), x.copy()
            xp[v, k] += h
            xm[v, k] -= h
            fd[v, k] = -(P.bend_energy3d(xp, s.faces, KB) - P.bend_energy3d(xm, s.faces, KB)) / (2 * h)
    err = np.linalg.norm(F.astype(np.float64) - fd) / np.linalg.norm(fd)
    # float forces against a double derivative: measured ~2e-7
    assert err <= 1e-6, err
    assert np.linalg.norm(fd) > 1.0  # the deformation bends the mesh
