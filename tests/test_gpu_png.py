"""Render::run from a folder of PNG frames (Image.segment_folder): host PNG
decoding, device preprocessing and optical flow, the plain sequence.  The
labels equal the CPU restatement's run on the same frames (host
preprocessing, the NumPy flow restatement, the oracle's clip run)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_png_folder_matches_oracle(asv, orc, tmp_path):
    from oracle import flow as ofl
    rgb0, _, _ = asv.synth_clip(64, 48, 6, n_ellipses=5, noise_sigma=3.0, jitter=0.3, seed=12)
    bgr = np.ascontiguousarray(rgb0[:, ::-1, :, ::-1])          # frames as files hold them
    for t in range(bgr.shape[0]):
        asv.write_png(str(tmp_path / f"{t + 1:05d}.png"), bgr[t][..., ::-1])
    assert np.array_equal(asv.read_frames(asv.list_frames(str(tmp_path))), bgr)
    K, iters = 90, 3
    with asv.Image(lloyd_iters=iters) as img:
        got = img.segment_folder(str(tmp_path), K)
        got_raw = img.raw_labels()
    rgb = np.stack([asv.preprocess_frame(bgr[z]) for z in range(bgr.shape[0])])
    fwd, bwd = ofl.compute_flow(rgb)
    want, want_raw, _, _ = orc.run_clip(rgb, fwd, bwd, K, iters=iters)
    assert np.array_equal(got_raw, want_raw)
    assert np.array_equal(got, want)
