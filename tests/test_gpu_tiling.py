"""The JFA tile depth (voxels of a column one block walks along a step's
chains) changes only the schedule: labels are identical at every depth, and
asv_autotune keeps one of its candidates and leaves the labels of a run."""
import numpy as np
import pytest

from conftest import small_clip

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,D,K", [(64, 48, 37, 150), (40, 30, 9, 40), (80, 33, 70, 400)])
def test_depth_does_not_change_labels(asv, orc, W, H, D, K):
    rgb, fwd, bwd = small_clip(asv, W=W, H=H, D=D, seed=D, jitter=0.3, drift=1.0)
    want, _, _, _ = orc.run_clip(rgb, fwd, bwd, K, iters=3, nthreads=8)
    for z in (1, 3, 4, 8, 16, 32, 64, 200):
        with asv.Image(lloyd_iters=3, jfa_zrun=z) as im:
            got = im.segment(rgb, fwd, bwd, K)
        assert np.array_equal(got, want), f"depth {z}"


def test_autotune_keeps_labels(asv):
    rgb, fwd, bwd = small_clip(asv, W=96, H=64, D=40, seed=5, jitter=0.2)
    with asv.Image(lloyd_iters=4) as im:
        want = im.segment(rgb, fwd, bwd, 300)
        z = im.autotune()
        assert z in (4, 8, 16, 32)
        assert np.array_equal(im.labels(), want)
        im.run_lloyd()
        assert np.array_equal(im.labels(), want)


@pytest.mark.parametrize("z", [0, 4, 32])
def test_tile_blocks_grid_keeps_labels(asv, orc, z):
    """One block per tile (the server's grid) instead of the persistent grid:
    the same labels."""
    W, H, D, K = 72, 40, 45, 220
    rgb, fwd, bwd = small_clip(asv, W=W, H=H, D=D, seed=11, jitter=0.3, drift=1.0)
    want, _, _, _ = orc.run_clip(rgb, fwd, bwd, K, iters=3, nthreads=8)
    with asv.Image(lloyd_iters=3, jfa_zrun=z, jfa_tile_blocks=1) as im:
        assert np.array_equal(im.segment(rgb, fwd, bwd, K), want)
