"""3D connectivity enforcement on the GPU (asv_enforce_connectivity*) against
the CPU restatement of Image::EnforceLabelConnectivity3D, which is pinned to
the reference's own C++ (tests/test_ref_pin.py, tests/golden/connectivity.npz)."""
import numpy as np
import pytest

from conftest import small_clip

pytestmark = pytest.mark.gpu


def test_after_lloyd_matches_oracle(asv, orc):
    for (W, H, D, K) in ((64, 48, 12, 120), (96, 64, 20, 300), (33, 17, 9, 40)):
        rgb, fwd, bwd = small_clip(asv, W=W, H=H, D=D, seed=W + D, jitter=0.3, drift=1.0)
        with asv.Image(lloyd_iters=3) as img:
            img.segment(rgb, fwd, bwd, K)
            raw = img.raw_labels()
            got, n = img.enforce_connectivity()
        want, m = orc.enforce_connectivity(raw, W * H * D // K)
        assert n == m and np.array_equal(got, want)


@pytest.mark.parametrize("shape,kind", [((85, 240, 320), "blocky"), ((30, 160, 240), "noisy"),
                                        ((16, 64, 64), "uniform"), ((12, 50, 70), "speckle"),
                                        ((1, 300, 200), "noisy"), ((40, 1, 500), "speckle")])
def test_volumes_match_oracle(asv, orc, shape, kind):
    rng = np.random.default_rng(sum(shape))
    D, H, W = shape
    if kind == "uniform":
        labels = np.full(shape, 7, np.int32)
    elif kind == "speckle":                    # very many tiny segments
        labels = rng.integers(-1, 12, shape).astype(np.int32)
    else:
        c = rng.integers(0, [W, H, D], (200, 3))
        zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij", sparse=True)
        best = np.full(shape, np.inf)
        labels = np.zeros(shape, np.int32)
        for i, (cx, cy, cz) in enumerate(c):
            d = (xx - cx) ** 2 + (yy - cy) ** 2 + 3 * (zz - cz) ** 2
            m = d < best
            best[m] = d[m]
            labels[m] = i
        if kind == "noisy":
            flip = rng.random(shape) < 0.03
            labels[flip] = rng.integers(-1, 200, int(flip.sum()))
    supsz = labels.size // 200
    with asv.Image(lloyd_iters=1) as img:
        got, n = img.enforce_connectivity_labels(labels, supsz)
    want, m = orc.enforce_connectivity(labels, supsz)
    assert n == m
    assert np.array_equal(got, want)


def test_repeated_runs_are_identical(asv, orc):
    """Many tiny segments, 40 runs: the union-find flattening must leave every
    voxel at its root in every run (a path-halving write landing after a
    voxel's own flatten once left an ancestor in about 1 run in 14)."""
    rng = np.random.default_rng(73)
    labels = rng.integers(-1, 12, (12, 50, 70)).astype(np.int32)
    supsz = labels.size // 200
    want, m = orc.enforce_connectivity(labels, supsz)
    with asv.Image(lloyd_iters=1) as img:
        for _ in range(40):
            got, n = img.enforce_connectivity_labels(labels, supsz)
            assert n == m and np.array_equal(got, want)
