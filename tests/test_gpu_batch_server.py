"""Batched form (asv_batch_*) and the request pool (asv_server_*) on the GPU.

Both are new launch shapes around the same per-clip algorithm, so the bar is
identity: every clip of a batch, and every request of a mixed server load,
gives the labels of the same clip segmented alone (and those of the CPU
restatement)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIMS = [(64, 48, 12, 120), (40, 32, 9, 60), (96, 64, 16, 300), (48, 48, 7, 80), (33, 17, 5, 20)]


def _clip(asv, W, H, D, seed):
    return asv.synth_clip(W, H, D, n_ellipses=5, noise_sigma=5.0, vmax=2.5, jitter=0.2,
                          drift_amp=1.0, drift_period=20.0, seed=seed)


def _alone(asv, rgb, fwd, bwd, K, iters):
    with asv.Image(lloyd_iters=iters) as im:
        return im.segment(rgb, fwd, bwd, K), im.info()


def test_batch_equals_single_clips(asv, orc):
    iters = 5
    clips = [_clip(asv, W, H, D, 11 + i) for i, (W, H, D, K) in enumerate(DIMS)]
    b = asv.Batch(DIMS, lloyd_iters=iters)
    for i, (rgb, fwd, bwd) in enumerate(clips):
        b.upload(i, rgb, fwd, bwd)
    b.prepare()
    b.run_lloyd()
    for i, ((W, H, D, K), (rgb, fwd, bwd)) in enumerate(zip(DIMS, clips)):
        got = b.clip_labels(i)
        want, inf = _alone(asv, rgb, fwd, bwd, K, iters)
        assert np.array_equal(got, want), f"clip {i}"
        bi = b.clip_info(i)
        assert (bi.Kp, bi.dead, bi.neg_count, bi.final_label_num) == \
            (inf.Kp, inf.dead, inf.neg_count, inf.final_label_num)
        labels, _, _, _ = orc.run_clip(rgb, fwd, bwd, K, iters=iters, nthreads=8)
        assert np.array_equal(got, labels), f"clip {i} vs oracle"
    b.close()


def test_batch_uneven_large_clips_equal_alone(asv):
    """Two clips of the 16-clip workload whose border tiles end early: lanes
    that leave a tile run ahead into the next clip's tiles, and the fused
    centroid sums must still go to each lane's own clip."""
    from anisotropic_supervoxel_gb300 import workloads
    ws = workloads.batch_clips()
    pick = [ws[9], ws[8], ws[5]]
    dims = [(w["W"], w["H"], w["D"], w["K"]) for w in pick]
    clips = [workloads.make_clip(w) for w in pick]
    iters = 3
    b = asv.Batch(dims, lloyd_iters=iters)
    for i, c in enumerate(clips):
        b.upload(i, *c)
    b.prepare()
    b.run_lloyd()
    for i, ((W, H, D, K), c) in enumerate(zip(dims, clips)):
        want, _ = _alone(asv, *c, K, iters)
        assert np.array_equal(b.clip_labels(i), want), f"clip {i}"
    b.close()


def test_batch_rerun_same_context(asv):
    """A second upload + run in the same batch context replays the graph."""
    iters = 3
    dims = DIMS[:3]
    b = asv.Batch(dims, lloyd_iters=iters)
    res = []
    for rnd in range(2):
        clips = [_clip(asv, W, H, D, 100 * rnd + i) for i, (W, H, D, K) in enumerate(dims)]
        for i, c in enumerate(clips):
            b.upload(i, *c)
        b.prepare()
        b.run_lloyd()
        for i, ((W, H, D, K), c) in enumerate(zip(dims, clips)):
            want, _ = _alone(asv, *c, K, iters)
            assert np.array_equal(b.clip_labels(i), want), (rnd, i)
            res.append(b.clip_labels(i))
    b.close()


def test_server_alone_vs_mix(asv):
    """Every clip request of a mixed load returns its alone labels."""
    iters = 4
    rng = np.random.default_rng(3)
    shapes = [DIMS[int(rng.integers(len(DIMS)))] for _ in range(14)]
    clips = [_clip(asv, W, H, D, 500 + i) for i, (W, H, D, K) in enumerate(shapes)]
    alone = [_alone(asv, *c, K, iters)[0] for c, (W, H, D, K) in zip(clips, shapes)]
    with asv.Server(max_slots=3, lloyd_iters=iters) as srv:
        ids = [srv.submit_clip(*c, K) for c, (W, H, D, K) in zip(clips, shapes)]
        for i, rid in enumerate(ids):
            got, lat, qms = srv.wait(rid)
            assert np.array_equal(got, alone[i]), f"request {i}"
            assert lat >= qms >= 0.0
        st = srv.stats()
        assert st.completed == len(ids) and st.failed == 0 and st.queued == 0


def test_server_budget_admission(asv):
    """A budget that holds one large clip or several small ones: every request
    still completes with its alone labels, and memory in use never passes it."""
    iters = 3
    big = (96, 64, 16, 300)
    small = (40, 32, 9, 60)
    lib = asv.load()
    b_big = lib.asv_clip_bytes(*big)
    b_small = lib.asv_clip_bytes(*small)
    budget = b_big + b_small // 2
    shapes = [big, small, small, big, small, big, small]
    clips = [_clip(asv, W, H, D, 900 + i) for i, (W, H, D, K) in enumerate(shapes)]
    alone = [_alone(asv, *c, K, iters)[0] for c, (W, H, D, K) in zip(clips, shapes)]
    with asv.Server(max_slots=4, hbm_budget=budget, lloyd_iters=iters) as srv:
        ids = [srv.submit_clip(*c, K) for c, (W, H, D, K) in zip(clips, shapes)]
        peak = 0
        for i, rid in enumerate(ids):
            while not srv.poll(rid):
                peak = max(peak, srv.stats().bytes_in_use)
            got, _, _ = srv.wait(rid)
            assert np.array_equal(got, alone[i]), f"request {i}"
        assert peak <= budget
        assert srv.stats().failed == 0


def test_server_rejects_over_budget(asv):
    lib = asv.load()
    need = lib.asv_clip_bytes(64, 48, 12, 120)
    rgb, fwd, bwd = _clip(asv, 64, 48, 12, 1)
    with asv.Server(max_slots=1, hbm_budget=need // 2) as srv:
        with pytest.raises(asv.AsvError):
            srv.submit_clip(rgb, fwd, bwd, 120)


def test_server_session_windows_match_stream(asv):
    """Windows of a session interleaved with clip requests give the labels of
    a Stream run alone."""
    W, H, D_all, s100, iters = 48, 40, 75, 200, 4
    rgb, fwd, bwd = asv.synth_clip(W, H, D_all, n_ellipses=6, noise_sigma=5.0, vmax=2.0,
                                   jitter=0.3, drift_amp=2.0, drift_period=40.0, seed=W + D_all)
    st = asv.Stream(W, H, D_all, seeds_num_100=s100, lloyd_iters=iters)
    want = np.full((D_all, H, W), -7, np.int32)
    ranges = []
    for _ in range(st.info().blocks):
        inf = st.info()
        a = inf.block_end - inf.frames_needed
        ranges.append((a, inf.block_end))
        f0, lab = st.push(rgb[a:inf.block_end], fwd[a:inf.block_end], bwd[a:inf.block_end])
        want[f0:f0 + lab.shape[0]] = lab
    st.close()
    clips = [_clip(asv, W2, H2, D2, 70 + i) for i, (W2, H2, D2, K2) in enumerate(DIMS[:3])]
    alone = [_alone(asv, *c, d[3], iters)[0] for c, d in zip(clips, DIMS[:3])]
    with asv.Server(max_slots=2, lloyd_iters=iters) as srv:
        sid = srv.open_session(W, H, D_all, seeds_num_100=s100)
        wids = [srv.submit_window(sid, rgb[a:e], fwd[a:e], bwd[a:e]) for a, e in ranges]
        cids = [srv.submit_clip(*c, d[3]) for c, d in zip(clips, DIMS[:3])]
        got = np.full((D_all, H, W), -7, np.int32)
        f0 = 0
        for rid in wids:
            lab, _, _ = srv.wait(rid)
            got[f0:f0 + lab.shape[0]] = lab
            f0 += lab.shape[0]
        for i, rid in enumerate(cids):
            assert np.array_equal(srv.wait(rid)[0], alone[i])
    assert f0 == D_all
    assert np.array_equal(got, want)
