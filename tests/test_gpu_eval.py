"""Supervoxel quality measures on the GPU (asv_evaluate) against their NumPy
restatement (oracle/evaluate.py): equal counts and equal doubles."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(asv, labels, truth):
    from oracle import evaluate as ev
    with asv.Image(lloyd_iters=1) as img:
        got = img.evaluate(labels, truth)
    want = ev.evaluate(labels, truth)
    assert got == want, (got, want)
    return got


def test_random_volumes(asv):
    rng = np.random.default_rng(3)
    for shape, L, G in (((5, 17, 23), 40, 6), ((1, 30, 30), 300, 2), ((12, 9, 1), 5, 40)):
        _check(asv, rng.integers(-1, L, shape).astype(np.int32), rng.integers(0, G, shape).astype(np.int32))


def test_segmentation_against_synthetic_truth(asv):
    kw = dict(n_ellipses=8, noise_sigma=4.0, vmax=2.0, seed=21)
    rgb, fwd, bwd = asv.synth_clip(96, 72, 16, **kw)
    truth = asv.synth_truth(96, 72, 16, **kw)
    with asv.Image(lloyd_iters=5) as img:
        labels = img.segment(rgb, fwd, bwd, 200)
    r = _check(asv, labels, truth)
    assert r["truth_segments"] >= 2 and 0.0 < r["boundary_recall"] <= 1.0


def test_out_of_range_is_an_error(asv):
    lab = np.zeros((2, 4, 4), np.int32)
    truth = np.zeros((2, 4, 4), np.int32)
    truth[0, 0, 0] = 5000
    with asv.Image(lloyd_iters=1) as img:
        with pytest.raises(asv.AsvError):
            img.evaluate(lab, truth)
        lab[1, 1, 1] = -2
        truth[0, 0, 0] = 0
        with pytest.raises(asv.AsvError):
            img.evaluate(lab, truth)
