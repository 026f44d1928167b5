"""Streaming form on the GPU (asv_stream_*) against the CPU restatement of
streamGPU-AS's block scheduler: video-wide labels must be identical."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_stream(asv, rgb, fwd, bwd, seeds100, iters, bs=30, reuse_out=False):
    D_all, H, W, _ = rgb.shape
    st = asv.Stream(W, H, D_all, seeds_num_100=seeds100, block_size=bs, lloyd_iters=iters)
    out = np.full((D_all, H, W), -7, np.int32)
    buf = np.full((bs + bs // 3, H, W), -9, np.int32) if reuse_out else None   # the longest block
    info = st.info()
    nb = info.blocks
    for b in range(nb):
        inf = st.info()
        z0 = inf.block_end - inf.block_start - inf.frames_needed
        a, e = inf.block_start + z0, inf.block_end
        f0, lab = st.push(rgb[a:e], fwd[a:e], bwd[a:e], out=buf)
        out[f0:f0 + lab.shape[0]] = lab
    info = st.info()
    st.close()
    return out, nb, info.seeds_placed


@pytest.mark.parametrize("W,H,D,seeds100,iters", [(48, 40, 75, 200, 4), (64, 48, 95, 120, 6),
                                                  (40, 32, 36, 300, 3)])
def test_stream_matches_oracle(asv, orc, W, H, D, seeds100, iters):
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=6, noise_sigma=5.0, vmax=2.0, jitter=0.3,
                                   drift_amp=2.0, drift_period=40.0, seed=W + D)
    got, nb, placed = _run_stream(asv, rgb, fwd, bwd, seeds100, iters)
    want, info = orc.run_stream(rgb, fwd, bwd, seeds_num_100=seeds100, iters=iters, nthreads=8)
    assert nb == info["blocks"]
    assert placed == info["placed"]
    assert (got != -7).all()
    assert np.array_equal(got, want)


def test_stream_reused_output_buffer(asv, orc):
    """labels read into one caller buffer for every block equal the oracle's"""
    W, H, D = 40, 32, 56
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=6, noise_sigma=5.0, vmax=2.0, jitter=0.3,
                                   drift_amp=2.0, drift_period=40.0, seed=11)
    got, nb, _ = _run_stream(asv, rgb, fwd, bwd, 250, 3, reuse_out=True)
    want, info = orc.run_stream(rgb, fwd, bwd, seeds_num_100=250, iters=3, nthreads=8)
    assert nb == info["blocks"] and nb > 1
    assert np.array_equal(got, want)
    st = asv.Stream(W, H, D, seeds_num_100=250, block_size=30, lloyd_iters=3)
    with pytest.raises(ValueError):
        st.push(rgb[:30], fwd[:30], bwd[:30], out=np.zeros((29, H, W), np.int32))
    st.close()


def test_stream_720p_windows_match_oracle(asv, orc):
    """the 1280x720 streaming configuration (windows of 30 frames, 10 overlap,
    seeds_num_100 = 10000) over its first two windows, three Lloyd
    iterations each: video-wide labels identical"""
    rgb, fwd, bwd = asv.synth_clip(1280, 720, 50, n_ellipses=60, noise_sigma=5.0, vmax=3.0,
                                   drift_amp=6.0, drift_period=90.0, seed=20240604)
    got, nb, placed = _run_stream(asv, rgb, fwd, bwd, 10000, 3)
    want, info = orc.run_stream(rgb, fwd, bwd, seeds_num_100=10000, iters=3, nthreads=16)
    assert nb == info["blocks"] == 2
    assert placed == info["placed"]
    assert (got != -7).all()
    assert np.array_equal(got, want)
