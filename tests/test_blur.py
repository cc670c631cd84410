"""The reference's depth-aware blur (blurX/blurY over Shader/Lighting/bilateralBlur.inc:19-73).

CPU: exp2 of the weights, a flat image stays flat, no bleeding across a depth step, FP32 against FP64.  GPU: the
device image is bit-identical to the FP32 restatement.
"""
import numpy as np
import pytest


def test_weight_exp2(orc):
    t = np.concatenate([np.linspace(-125.9, 0, 20001), -np.logspace(-8, 2, 300)]).astype(np.float32)
    got = np.array([orc.exp2_poly(x) for x in t])
    ref = np.exp2(t.astype(np.float64))
    assert (np.abs(got - ref) / ref).max() < 2e-7
    assert orc.exp2_poly(-200.0) == 0.0


def test_flat_image_and_depth_step(orc):
    H, W = 40, 64
    img = np.zeros((H, W, 4), np.float32)
    img[..., :3] = 0.25
    depth = np.full((H, W), 0.5, np.float32)
    out = orc.blur(img, depth)
    assert np.allclose(out[..., :3], 0.25, rtol=1e-6) and np.all(out[..., 3] == 0)
    # left half near, right half far: 512 * 0.05 = 25.6, weight 2^-655 -> nothing crosses the step
    img[:, W // 2:, :3] = 1.0
    depth[:, W // 2:] = 0.55
    out = orc.blur(img, depth)
    assert np.allclose(out[:, : W // 2, :3], 0.25, rtol=1e-6)
    assert np.allclose(out[:, W // 2:, :3], 1.0, rtol=1e-6)


def test_fp32_against_fp64(orc):
    rng = np.random.default_rng(3)
    H, W = 48, 80
    img = rng.uniform(0, 2, (H, W, 4)).astype(np.float32)
    depth = (0.9 + 0.01 * rng.uniform(0, 1, (H, W))).astype(np.float32)
    a = orc.blur(img, depth)
    b = orc.blur(img.astype(np.float64), depth, f64=True)
    assert np.abs(a[..., :3] - b[..., :3]).max() / np.abs(b[..., :3]).max() < 1e-5


@pytest.mark.gpu
def test_gpu_blur_bit_identical(lib, orc):
    import torch

    import final184_gb300 as g

    rng = np.random.default_rng(4)
    H, W = 181, 323
    img = rng.uniform(0, 2, (H, W, 4)).astype(np.float32)
    depth = (0.95 + 0.002 * rng.uniform(0, 1, (H, W))).astype(np.float32)
    depth[:, 100:140] = 0.97
    dev = torch.device("cuda:0")
    ti, td = torch.from_numpy(img).to(dev), torch.from_numpy(depth).to(dev)
    to = torch.empty_like(ti)
    gi = g.VoxelGI(0)
    gi.blur(ti.data_ptr(), td.data_ptr(), W, H, to.data_ptr())
    gi.sync()
    got = to.cpu().numpy()
    gi.close()
    ref = orc.blur(img, depth)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
