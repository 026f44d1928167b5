"""Full-size parity of every benchmarked workload against the oracle.

Each test runs a benchmarked configuration at its own size and iteration
count on the GPU and compares the labels, raw (the last JFA pass) and
post-processed, bit for bit with the oracle on the same seeded inputs:

- the 320x240x85 clip, K=1000, 15 Lloyd iterations (GPU-AS/Render.cpp:277-293);
- the 1280x720 stream (windows of 30 frames, 10 overlap, 2000 new seeds per
  window) at its 20 Lloyd iterations over its first two windows
  (streamGPU-AS/Render.cpp:470-504);
- four of the 16 uneven clips of the batched workload, run inside the batch,
  including its two largest;
- one request of each class of the serving mix, taken from one mixed run of
  the request pool.

The oracle runs on all host threads; this file is collected after the other
GPU tests so that a run stopping at its first failure has reported the rest.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 8


def test_clip_320x240x85_full_bit_exact(asv, orc):
    from anisotropic_supervoxel_gb300 import workloads
    w = workloads.CLIP_320x240x85
    rgb, fwd, bwd = workloads.make_clip(w)
    with asv.Image(lloyd_iters=w["iters"]) as img:
        labels = img.segment(rgb, fwd, bwd, w["K"])
        raw = img.raw_labels()
        kp = img.info().Kp
    want, want_raw, seeds, info = orc.run_clip(rgb, fwd, bwd, w["K"], iters=w["iters"], nthreads=NT)
    assert kp == info["Kp"] == 936
    assert np.array_equal(raw, want_raw)
    assert np.array_equal(labels, want)


def test_stream_720p_two_windows_20_iterations(asv, orc):
    from anisotropic_supervoxel_gb300 import workloads
    w = workloads.STREAM_720P
    W, H, D = w["W"], w["H"], 50                       # windows [0, 30) and [20, 50)
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=w["n_ellipses"], noise_sigma=w["noise_sigma"],
                                   vmax=w["vmax"], drift_amp=w["drift_amp"],
                                   drift_period=w["drift_period"], seed=w["seed"])
    st = asv.Stream(W, H, D, seeds_num_100=w["seeds_num_100"], block_size=w["block_size"],
                    lloyd_iters=w["iters"])
    got = np.full((D, H, W), -7, np.int32)
    nb = st.info().blocks
    for _ in range(nb):
        inf = st.info()
        a, e = inf.block_end - inf.frames_needed, inf.block_end
        f0, lab = st.push(rgb[a:e], fwd[a:e], bwd[a:e])
        got[f0:f0 + lab.shape[0]] = lab
    placed = st.info().seeds_placed
    st.close()
    want, info = orc.run_stream(rgb, fwd, bwd, seeds_num_100=w["seeds_num_100"], iters=w["iters"],
                                block_size=w["block_size"], nthreads=NT)
    assert nb == info["blocks"] == 2
    assert placed == info["placed"]
    assert (got != -7).all()
    assert np.array_equal(got, want)


def test_batch16_clips_inside_batch_match_oracle(asv, orc):
    from anisotropic_supervoxel_gb300 import workloads
    ws = workloads.batch_clips()
    dims = [(w["W"], w["H"], w["D"], w["K"]) for w in ws]
    size = [W * H * D for W, H, D, _ in dims]
    order = np.argsort(size)
    pick = [int(order[-1]), int(order[-2]), int(order[0]), int(order[len(order) // 2])]
    clips = [workloads.make_clip(w) for w in ws]
    iters = ws[0]["iters"]
    b = asv.Batch(dims, lloyd_iters=iters)
    for i, c in enumerate(clips):
        b.upload(i, *c)
    b.prepare()
    b.run_lloyd()
    got = {i: b.clip_labels(i) for i in pick}
    b.close()
    for i in pick:
        rgb, fwd, bwd = clips[i]
        want, _, _, _ = orc.run_clip(rgb, fwd, bwd, dims[i][3], iters=iters, nthreads=NT)
        assert np.array_equal(got[i], want), f"clip {i} {dims[i]}"


def test_serve_mix_one_request_per_class_matches_oracle(asv, orc):
    from anisotropic_supervoxel_gb300 import workloads
    mix = workloads.serving_mix()
    small, mid, win = (dict(m[1]) for m in mix)
    iters = small["iters"]
    small["seed"], mid["seed"] = 881, 882
    c_small = workloads.make_clip(small)
    c_small2 = workloads.make_clip(dict(small, seed=883))
    c_mid = workloads.make_clip(mid)
    w_rgb, w_fwd, w_bwd = asv.synth_clip(win["W"], win["H"], 30, n_ellipses=win["n_ellipses"],
                                         noise_sigma=win["noise_sigma"], vmax=win["vmax"], seed=884)
    with asv.Server(max_slots=4, hbm_budget=120 << 30, lloyd_iters=iters) as srv:
        sid = srv.open_session(win["W"], win["H"], 30, seeds_num_100=win["K"] * 100 // 20)
        r1 = srv.submit_clip(*c_small, small["K"])
        r2 = srv.submit_clip(*c_mid, mid["K"])
        r3 = srv.submit_window(sid, w_rgb, w_fwd, w_bwd)
        r4 = srv.submit_clip(*c_small2, small["K"])
        g_small, g_mid, g_win, g_small2 = (srv.wait(r)[0] for r in (r1, r2, r3, r4))
        assert srv.stats().failed == 0
    for got, (rgb, fwd, bwd), K in ((g_small, c_small, small["K"]), (g_small2, c_small2, small["K"]),
                                    (g_mid, c_mid, mid["K"])):
        want, _, _, _ = orc.run_clip(rgb, fwd, bwd, K, iters=iters, nthreads=NT)
        assert np.array_equal(got, want), rgb.shape
    want, info = orc.run_stream(w_rgb, w_fwd, w_bwd, seeds_num_100=win["K"] * 100 // 20, iters=iters,
                                nthreads=NT)
    assert info["blocks"] == 1
    assert g_win.shape == want.shape
    assert np.array_equal(g_win, want)
