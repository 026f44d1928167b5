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


def _fed_frames(st, b, rgb, fwd, bwd, flow=True):
    a, e, n = st.block(b)
    z0 = e - a - n
    return (rgb[a + z0:e], fwd[a + z0:e], bwd[a + z0:e]) if flow else (rgb[a + z0:e],)


def test_stream_fed_ahead_matches_oracle(asv, orc):
    """frames uploaded a block ahead (asv_stream_feed / asv_stream_push_fed) give
    the oracle's labels; the call-order rules are enforced"""
    W, H, D, s100, iters = 48, 40, 75, 200, 4
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=6, noise_sigma=5.0, vmax=2.0, jitter=0.3,
                                   drift_amp=2.0, drift_period=40.0, seed=W + D)
    st = asv.Stream(W, H, D, seeds_num_100=s100, block_size=30, lloyd_iters=iters)
    nb = st.info().blocks
    assert nb == 3
    out = np.full((D, H, W), -7, np.int32)
    with pytest.raises(asv.AsvError):
        st.push_fed()                                    # nothing fed
    assert st.feed(*_fed_frames(st, 0, rgb, fwd, bwd)) == 0
    with pytest.raises(asv.AsvError):
        st.push(*_fed_frames(st, 0, rgb, fwd, bwd))      # a fed block goes through push_fed
    assert st.feed(*_fed_frames(st, 1, rgb, fwd, bwd)) == 1
    with pytest.raises(asv.AsvError):
        st.feed(*_fed_frames(st, 2, rgb, fwd, bwd))      # at most two blocks ahead
    buf = np.full((40, H, W), -9, np.int32)
    for b in range(nb):
        if 1 <= b and b + 1 < nb:
            assert st.feed(*_fed_frames(st, b + 1, rgb, fwd, bwd)) == b + 1
        f0, lab = st.push_fed(out=buf)
        out[f0:f0 + lab.shape[0]] = lab
    with pytest.raises(asv.AsvError):
        st.push_fed()                                    # the video is done
    st.close()
    want, info = orc.run_stream(rgb, fwd, bwd, seeds_num_100=s100, iters=iters, nthreads=8)
    assert np.array_equal(out, want)


def test_stream_pipelined_matches_oracle(asv, orc):
    """two blocks in flight (asv_stream_push_fed_async / asv_stream_wait) give
    the oracle's labels; the in-flight rules are enforced"""
    W, H, D, s100, iters = 48, 40, 75, 200, 4
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=6, noise_sigma=5.0, vmax=2.0, jitter=0.3,
                                   drift_amp=2.0, drift_period=40.0, seed=W + D)
    st = asv.Stream(W, H, D, seeds_num_100=s100, block_size=30, lloyd_iters=iters)
    assert st.info().blocks == 3
    bufs = [np.full((40, H, W), -9, np.int32) for _ in range(2)]
    out = np.full((D, H, W), -7, np.int32)
    st.feed(*_fed_frames(st, 0, rgb, fwd, bwd))
    assert st.push_fed_async(bufs[0]) == 0
    st.feed(*_fed_frames(st, 1, rgb, fwd, bwd))
    assert st.push_fed_async(bufs[1]) == 1                   # two blocks in flight
    st.feed(*_fed_frames(st, 2, rgb, fwd, bwd))
    with pytest.raises(asv.AsvError):
        st.push_fed_async(np.zeros((40, H, W), np.int32))    # a third: wait first
    with pytest.raises(asv.AsvError):
        st.push_fed()                                        # synchronous push with blocks in flight
    for b in range(3):
        f0, lab = st.wait()
        out[f0:f0 + lab.shape[0]] = lab
        if b == 0:
            assert st.push_fed_async(bufs[0]) == 2           # block 0's buffer is free again
    with pytest.raises(asv.AsvError):
        st.wait()                                            # nothing in flight
    st.close()
    want, info = orc.run_stream(rgb, fwd, bwd, seeds_num_100=s100, iters=iters, nthreads=8)
    assert np.array_equal(out, want)


def test_stream_close_with_blocks_in_flight(asv):
    """closing a stream with two blocks enqueued and not waited for is clean,
    and a new stream on the device works after it"""
    W, H, D = 40, 32, 56
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=6, noise_sigma=5.0, vmax=2.0, jitter=0.3,
                                   drift_amp=2.0, drift_period=40.0, seed=21)
    bufs = [np.full((40, H, W), -9, np.int32) for _ in range(2)]
    st = asv.Stream(W, H, D, seeds_num_100=250, block_size=30, lloyd_iters=3)
    for b in range(2):
        st.feed(*_fed_frames(st, b, rgb, fwd, bwd))
        st.push_fed_async(bufs[b])
    st.close()                                               # waits for the device, drops the blocks
    assert (bufs[0] != -9).any()                             # the first block's labels did arrive
    got, nb, _ = _run_stream(asv, rgb, fwd, bwd, 250, 3)
    want, _, _ = _run_stream(asv, rgb, fwd, bwd, 250, 3, reuse_out=True)
    assert nb == 2 and np.array_equal(got, want)


def test_stream_fed_ahead_device_flow_equals_push(asv):
    """fed without flow: the device computes each block's flow, as push does"""
    W, H, D = 40, 32, 56
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=6, noise_sigma=5.0, vmax=2.0, jitter=0.3,
                                   drift_amp=2.0, drift_period=40.0, seed=5)
    res = []
    for mode in ("push", "fed"):
        st = asv.Stream(W, H, D, seeds_num_100=250, block_size=30, lloyd_iters=3)
        nb = st.info().blocks
        out = np.full((D, H, W), -7, np.int32)
        if mode == "fed":
            st.feed(*_fed_frames(st, 0, rgb, fwd, bwd, flow=False))
        for b in range(nb):
            if mode == "fed":
                if b + 1 < nb:
                    st.feed(*_fed_frames(st, b + 1, rgb, fwd, bwd, flow=False))
                f0, lab = st.push_fed()
            else:
                f0, lab = st.push(*_fed_frames(st, b, rgb, fwd, bwd, flow=False))
            out[f0:f0 + lab.shape[0]] = lab
        st.close()
        res.append(out)
    assert (res[0] != -7).all()
    assert np.array_equal(res[0], res[1])


def test_stream_fed_bgr_equals_host_preprocessing(asv):
    """frames fed as decoded BGR (asv_stream_feed_bgr, preprocessed on the
    device) give the labels of the host-preprocessed frames pushed as RGB"""
    W, H, D = 40, 32, 56
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=6, noise_sigma=5.0, vmax=2.0, jitter=0.3,
                                   drift_amp=2.0, drift_period=40.0, seed=9)
    bgr = np.ascontiguousarray(rgb[:, ::-1, :, ::-1])     # as imread would give the frames
    pre = np.stack([asv.preprocess_frame(f) for f in bgr])
    res = []
    for mode in ("push", "fed_bgr"):
        st = asv.Stream(W, H, D, seeds_num_100=250, block_size=30, lloyd_iters=3)
        nb = st.info().blocks
        out = np.full((D, H, W), -7, np.int32)
        if mode == "fed_bgr":
            st.feed(*_fed_frames(st, 0, bgr, fwd, bwd), bgr=True)
        for b in range(nb):
            if mode == "fed_bgr":
                if b + 1 < nb:
                    st.feed(*_fed_frames(st, b + 1, bgr, fwd, bwd), bgr=True)
                f0, lab = st.push_fed()
            else:
                f0, lab = st.push(*_fed_frames(st, b, pre, fwd, bwd))
            out[f0:f0 + lab.shape[0]] = lab
        st.close()
        res.append(out)
    assert (res[0] != -7).all()
    assert np.array_equal(res[0], res[1])


def test_stream_feed_over_budget_leaves_push_usable(asv):
    """a feed whose staging does not fit the context's HBM budget fails, again
    on a retry, and the stream still runs through push"""
    W, H, D = 40, 32, 56
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=6, noise_sigma=5.0, vmax=2.0, jitter=0.3,
                                   drift_amp=2.0, drift_period=40.0, seed=13)
    lo, hi = 0, 1 << 30                       # the least budget the stream's layout fits in
    while hi - lo > 4096:
        mid = (lo + hi) // 2
        try:
            asv.Stream(W, H, D, seeds_num_100=250, block_size=30, lloyd_iters=3, hbm_budget=mid).close()
            hi = mid
        except asv.AsvError:
            lo = mid
    st = asv.Stream(W, H, D, seeds_num_100=250, block_size=30, lloyd_iters=3, hbm_budget=hi)
    for _ in range(2):
        with pytest.raises(asv.AsvError):
            st.feed(*_fed_frames(st, 0, rgb, fwd, bwd))
    got = np.full((D, H, W), -7, np.int32)
    for b in range(st.info().blocks):
        f0, lab = st.push(*_fed_frames(st, b, rgb, fwd, bwd))
        got[f0:f0 + lab.shape[0]] = lab
    st.close()
    want, _, _ = _run_stream(asv, rgb, fwd, bwd, 250, 3)
    assert np.array_equal(got, want)


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
