"""Optical flow on the device (asv_compute_flow) against its NumPy restatement
(oracle/flow.py, the same float32 operations in the same order): bit-exact;
and its accuracy on a textured clip moved by known sub-pixel shifts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_flow(asv, rgb, K=40):
    with asv.Image(lloyd_iters=1) as img:
        img.init_gpu(rgb, K)
        img.compute_flow()
        return img.flow()


@pytest.mark.parametrize("W,H,D", [(96, 64, 4), (40, 33, 3), (20, 12, 2)])
def test_flow_matches_restatement(asv, W, H, D):
    from oracle import flow as ofl
    rgb, _, _ = asv.synth_clip(W, H, D, n_ellipses=5, noise_sigma=3.0, vmax=2.0, seed=W + D)
    got_f, got_b = _device_flow(asv, rgb)
    want_f, want_b = ofl.compute_flow(rgb)
    assert np.array_equal(got_f, want_f)
    assert np.array_equal(got_b, want_b)


def test_flow_accuracy_on_textured_shifts(asv):
    scipy_nd = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(5)
    H, W, D = 96, 128, 4
    base = scipy_nd.gaussian_filter(rng.random((H + 40, W + 40)) * 255.0, 3.0)
    shifts = [(0.0, 0.0), (1.25, -0.5), (2.0, 0.75), (3.5, 1.0)]     # cumulative (x, y) per frame
    frames = [scipy_nd.shift(base, (sy, sx), order=3, mode="nearest")[20:20 + H, 20:20 + W] for sx, sy in shifts]
    g = np.clip(np.round(np.stack(frames)), 0, 255).astype(np.uint8)
    rgb = np.repeat(g[..., None], 3, -1)
    fwd, bwd = _device_flow(asv, rgb)
    m = (slice(16, -16), slice(16, -16))
    for z in range(D - 1):
        want = np.array(shifts[z + 1]) - np.array(shifts[z])
        e = np.sqrt(((fwd[z][m] - want) ** 2).sum(-1))
        assert e.mean() < 0.08, (z, float(e.mean()))
        e = np.sqrt(((bwd[z + 1][m] + want) ** 2).sum(-1))
        assert e.mean() < 0.08, (z, float(e.mean()))
    assert not fwd[D - 1].any() and not bwd[0].any()


def test_segmentation_with_device_flow_is_deterministic(asv):
    rgb, _, _ = asv.synth_clip(80, 60, 8, n_ellipses=6, noise_sigma=3.0, vmax=2.0, seed=12)
    out = []
    for _ in range(2):
        with asv.Image(lloyd_iters=3) as img:
            img.init_gpu(rgb, 120)
            img.compute_flow()
            img.initialization()
            img.seed_matrix()
            img.RGB2LAB()
            img.run_lloyd()
            out.append(img.labels())
    assert np.array_equal(out[0], out[1])
    assert (out[0] >= 0).all()


def test_stream_with_device_flow_matches_oracle(asv, orc):
    """Streaming with the block's flow computed on the device equals the
    CPU restatement of the streaming form fed with the restated flow (each
    frame pair's flow depends only on its two frames)."""
    from oracle import flow as ofl
    W, H, D, s100, iters = 48, 40, 75, 200, 4
    rgb, _, _ = asv.synth_clip(W, H, D, n_ellipses=6, noise_sigma=3.0, vmax=2.0, jitter=0.3, drift_amp=2.0,
                               drift_period=40.0, seed=7)
    fwd, bwd = ofl.compute_flow(rgb)
    st = asv.Stream(W, H, D, seeds_num_100=s100, lloyd_iters=iters)
    got = np.full((D, H, W), -7, np.int32)
    for _ in range(st.info().blocks):
        inf = st.info()
        a = inf.block_end - inf.frames_needed
        f0, lab = st.push(rgb[a:inf.block_end])
        got[f0:f0 + lab.shape[0]] = lab
    st.close()
    want, _ = orc.run_stream(rgb, fwd, bwd, seeds_num_100=s100, iters=iters, nthreads=8)
    assert np.array_equal(got, want)


def test_clip_without_flow_uses_device_flow(asv):
    rgb, _, _ = asv.synth_clip(64, 48, 6, n_ellipses=5, noise_sigma=3.0, seed=4)
    with asv.Image(lloyd_iters=3) as a:
        a.init_gpu(rgb, 100)
        a.compute_flow()
        a.initialization()
        a.seed_matrix()
        a.RGB2LAB()
        a.run_lloyd()
        want = a.labels()
    with asv.Server(max_slots=1, lloyd_iters=3) as srv:
        got, _, _ = srv.wait(srv.submit_clip(rgb, None, None, 100))
    assert np.array_equal(got, want)
