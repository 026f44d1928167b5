"""The five seeded synthetic workloads the benchmark and tests use.

They stand in for the LIBSVX datasets (SegTrackv2, BuffaloXiph) the reference
is evaluated on: seeded synthetic clips with the configured shapes, motion
and noise (generator: asv_synth_clip).
"""
import numpy as np

# plain single clip: 240x160x30, 12 ellipses, sigma 5, K=200, 10 iterations, the
# full JFA ladder (powers of two from log2 of the largest dimension, then 2, 1)
CLIP_240x160x30 = dict(W=240, H=160, D=30, n_ellipses=12, noise_sigma=5.0, vmax=3.0,
                       jitter=0.0, K=200, iters=10, full_ladder=1, seed=20240601)
# single clip: 320x240x85, 30 ellipses with +-0.5 px/frame jitter, sigma 8, K=1000, 15 iterations
CLIP_320x240x85 = dict(W=320, H=240, D=85, n_ellipses=30, noise_sigma=8.0, vmax=3.0,
                       jitter=0.5, K=1000, iters=15, seed=20240602)
# streaming 1280x720 video, 60 ellipses, sinusoidal background drift, windows 30/10;
# K = 2000 new seeds per window of 20 new frames: seeds_num_100 = 2000 * 100 / 20
# (the window also carries the seeds of its 10 overlap frames from the previous one)
STREAM_720P = dict(W=1280, H=720, D_all=900, n_ellipses=60, noise_sigma=5.0, vmax=3.0,
                   jitter=0.0, drift_amp=6.0, drift_period=90.0, K_window=2000,
                   seeds_num_100=10000, iters=20, block_size=30, seed=20240604)


def batch_clips(n=16, seed=20240603):
    """16 clips of uneven size: W x H uniform in [240x160, 640x480], D in [20, 120],
    K in [200, 2000], 10 iterations."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        t = rng.uniform()
        W = int(round(240 + t * 400)) // 8 * 8
        H = int(round(160 + t * 320)) // 8 * 8
        out.append(dict(W=W, H=H, D=int(rng.integers(20, 121)), n_ellipses=int(rng.integers(8, 31)),
                        noise_sigma=5.0, vmax=3.0, jitter=0.0, K=int(rng.integers(200, 2001)),
                        iters=10, seed=seed * 100 + i))
    return out


def serving_mix():
    """request classes of the Poisson serving mix (mean 40 req/s)."""
    return [
        (0.50, dict(W=240, H=160, D=30, n_ellipses=12, noise_sigma=5.0, vmax=3.0, jitter=0.0,
                    K=200, iters=10)),
        (0.35, dict(W=640, H=480, D=60, n_ellipses=30, noise_sigma=5.0, vmax=3.0, jitter=0.0,
                    K=1000, iters=10)),
        (0.15, dict(W=1280, H=720, D=30, n_ellipses=60, noise_sigma=5.0, vmax=3.0, jitter=0.0,
                    K=2000, iters=10)),
    ]


def make_clip(w, scale=None, gen=None):
    """rgb, fwd, bwd of a workload dict (optionally spatially scaled for
    tests).  `gen` is the generator (a function with synth_clip's
    arguments); default this package's."""
    if gen is None:
        from .image import synth_clip as gen
    W, H, D = w["W"], w["H"], w["D"]
    if scale:
        W, H, D = max(8, int(W * scale)), max(8, int(H * scale)), max(4, int(D * scale))
    return gen(W, H, D, n_ellipses=w["n_ellipses"], noise_sigma=w["noise_sigma"],
               vmax=w["vmax"], jitter=w.get("jitter", 0.0),
               drift_amp=w.get("drift_amp", 0.0), drift_period=w.get("drift_period", 60.0),
               seed=w["seed"])


def stream_frames(w, frame0, n, gen=None, crop=None):
    """Frames [frame0, frame0 + n) of the streaming video `w` (rgb, fwd,
    bwd); crop = (x0, y0, cw, ch) cuts that region out of every frame (the
    rows counted in the frames' texture orientation, y up)."""
    if gen is None:
        from .image import synth_clip as gen
    rgb, fwd, bwd = gen(w["W"], w["H"], n, n_ellipses=w["n_ellipses"], noise_sigma=w["noise_sigma"],
                        vmax=w["vmax"], jitter=w.get("jitter", 0.0), drift_amp=w.get("drift_amp", 0.0),
                        drift_period=w.get("drift_period", 60.0), seed=w["seed"], frame0=frame0)
    if crop is not None:
        x0, y0, cw, ch = crop
        rgb, fwd, bwd = (np.ascontiguousarray(a[:, y0:y0 + ch, x0:x0 + cw]) for a in (rgb, fwd, bwd))
    return rgb, fwd, bwd
