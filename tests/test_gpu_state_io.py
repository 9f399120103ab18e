"""State I/O: checkpoints resume bit for bit, and the zero-copy device views
hold the same values as the host read-back."""
import numpy as np
import pytest

from cases import gpu_batch2d, gpu_batch3d, make_tissue2d, make_tissue3d

pytestmark = pytest.mark.gpu

DT = 0.005


@pytest.fixture(scope="module")
def ctx():
    from opencl_dpm_gb300.abi import Context
    return Context(0)


def test_checkpoint_2d_resumes_bitwise(ctx, tmp_path):
    from opencl_dpm_gb300.abi import Batch2D
    states = [make_tissue2d(20, 24, Kb=0.01, phi=0.8, seed=61),
              make_tissue2d(9, 48, calA=1.2, phi=0.7, seed=62, Kat=0.3)]
    a = gpu_batch2d(ctx, states)
    a.step(70, DT)
    ref_x, ref_f = a.download()
    b = gpu_batch2d(ctx, states)
    b.step(33, DT)
    path = str(tmp_path / "t2.ckpt")
    b.save(path)
    x33, f33 = b.download()
    c = Batch2D.open(ctx, path)
    cx, cf = c.download()
    assert np.array_equal(cx, x33) and np.array_equal(cf, f33)
    c.step(37, DT)
    x, f = c.download()
    assert np.array_equal(x, ref_x) and np.array_equal(f, ref_f)


def test_checkpoint_3d_resumes_bitwise(ctx, tmp_path):
    from opencl_dpm_gb300.abi import Batch3D
    states = [make_tissue3d(4, level=2, phi0=0.5, seed=63, Kb=0.05, adh=0.1),
              make_tissue3d(3, level=2, phi0=0.5, seed=64)]
    a = gpu_batch3d(ctx, states)
    a.step(20, DT)
    ref_x, ref_f = a.download()
    b = gpu_batch3d(ctx, states)
    b.step(9, DT)
    path = str(tmp_path / "t3.ckpt")
    b.save(path)
    c = Batch3D.open(ctx, path)
    c.step(11, DT)
    x, f = c.download()
    assert np.array_equal(x, ref_x) and np.array_equal(f, ref_f)


def test_device_views(ctx):
    import torch
    s = make_tissue2d(12, 32, phi=0.8, seed=65)
    b = gpu_batch2d(ctx, [s])
    b.step(5, DT)
    p, f = b.device_state()
    x, F = b.download()
    assert p.is_cuda and p.shape == (b.nverts, 2)
    torch.cuda.synchronize()
    assert np.array_equal(p.cpu().numpy(), x) and np.array_equal(f.cpu().numpy(), F)
    s3 = make_tissue3d(3, level=2, phi0=0.5, seed=66)
    b3 = gpu_batch3d(ctx, [s3])
    b3.step(3, DT)
    views = b3.device_state()
    x3, F3 = b3.download()
    torch.cuda.synchronize()
    got = np.stack([v.cpu().numpy() for v in views[:3]], axis=1)
    gotf = np.stack([v.cpu().numpy() for v in views[3:]], axis=1)
    assert np.array_equal(got, x3) and np.array_equal(gotf, F3)


def test_checkpoint_rejects_garbage(ctx, tmp_path):
    from opencl_dpm_gb300.abi import Batch2D, DPMError
    p = tmp_path / "bad.ckpt"
    p.write_bytes(b"not a checkpoint at all")
    with pytest.raises(DPMError):
        Batch2D.open(ctx, str(p))
