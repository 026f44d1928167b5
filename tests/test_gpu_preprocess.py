"""Raw-frame preprocessing on the device (asv_init_gpu_bgr) against the host
restatement of Render::cvMat2TexureInput (asv_preprocess_frame): the same
RGB bytes, hence the same LAB volume and labels."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,D", [(64, 48, 6), (33, 17, 5), (1, 9, 3), (12, 1, 4), (2, 2, 2)])
def test_bgr_frames_equal_host_preprocess(asv, W, H, D):
    rng = np.random.default_rng(W * 131 + H)
    bgr = rng.integers(0, 256, (D, H, W, 3), dtype=np.uint8)
    rgb = np.stack([asv.preprocess_frame(bgr[z]) for z in range(D)])
    lib = asv.load()
    K = next(k for k in range(max(2, W * H * D // 40), W * H * D + 1) if lib.asv_clip_bytes(W, H, D, k))
    with asv.Image(lloyd_iters=1) as a, asv.Image(lloyd_iters=1) as b:
        a.init_gpu(rgb, K)
        a.RGB2LAB()
        b.init_gpu_bgr(bgr, K)
        b.RGB2LAB()
        assert np.array_equal(a.lab(), b.lab())


def test_bgr_clip_segments_like_host(asv):
    rgb0, fwd, bwd = asv.synth_clip(80, 60, 10, n_ellipses=5, seed=9)
    # raw frames as a video reader gives them: top row first, BGR
    bgr = np.ascontiguousarray(rgb0[:, ::-1, :, ::-1])
    rgb = np.stack([asv.preprocess_frame(bgr[z]) for z in range(bgr.shape[0])])
    with asv.Image(lloyd_iters=3) as a, asv.Image(lloyd_iters=3) as b:
        want = a.segment(rgb, fwd, bwd, 150)
        b.init_gpu_bgr(bgr, 150)
        b.upload_flow(fwd, bwd)
        b.initialization()
        b.seed_matrix()
        b.RGB2LAB()
        b.run_lloyd()
        assert np.array_equal(b.labels(), want)
