"""Golden fixtures from the reference's own shaders (tests/golden/make_golden.py):
the CPU restatement and the CUDA path must reproduce them exactly."""
import os

import numpy as np
import pytest

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(G, name))


def test_oracle_rgb2lab(orc):
    f = load("rgb2lab_sample.npz")
    assert np.array_equal(orc.rgb2lab(f["rgb"])[:, :3].astype(np.float32), f["lab"])


def test_oracle_derivative(orc):
    f = load("derivative.npz")
    assert np.array_equal(orc.gradient_half(f["rgb"]), f["gradient"].astype(np.float16).view(np.uint16))


@pytest.mark.parametrize("step", [1, 3, 7])
def test_oracle_flood(orc, step):
    f = load(f"flood_step{step}.npz")
    lab4 = orc.rgb2lab(f["rgb"])
    got = orc.jfa_pass(f["labels"], lab4, f["seeds"], int(f["step"]), np.float32(f["ratio"]))
    assert np.array_equal(got, f["out"])


def test_oracle_aver_exception(orc):
    f = load("aver_exception.npz")
    rgb = f["rgb"]
    D, H, W, _ = rgb.shape
    kp = f["pos"].shape[0]
    pos, col = orc.finalize((D, H, W), f["sums"], orc.rgb2lab(rgb), np.zeros((kp, 3), np.float32),
                            np.zeros((kp, 3), np.float32))
    assert np.array_equal(pos, f["pos"][:, :3])
    assert np.array_equal(col, f["col"])


@pytest.mark.gpu
def test_cuda_rgb2lab(asv):
    f = load("rgb2lab_sample.npz")
    rgb = f["rgb"].reshape(2, 64, 128, 3)
    img = asv.Image(lloyd_iters=1)
    img.init_gpu(rgb, 100)
    img.RGB2LAB()
    assert np.array_equal(img.lab()[..., :3].reshape(-1, 3).astype(np.float32), f["lab"])


@pytest.mark.gpu
@pytest.mark.parametrize("step", [1, 3, 7])
def test_cuda_flood(asv, step):
    f = load(f"flood_step{step}.npz")
    rgb = f["rgb"]
    D, H, W, _ = rgb.shape
    img = asv.Image(lloyd_iters=1)
    img.init_gpu(rgb, 20)
    img.RGB2LAB()
    assert img.info().Kp == f["seeds"].shape[0]
    img.set_seeds(f["seeds"])
    got = img.jfa_pass(f["labels"], int(f["step"]), float(np.float32(f["ratio"])))
    assert np.array_equal(got, f["out"])
