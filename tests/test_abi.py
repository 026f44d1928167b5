"""C ABI and host pipeline checks that need no GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return set(re.findall(r"\b(asv_[a-z0-9_]+)\s*\(", src))


def test_every_declared_symbol_is_exported(asv):
    lib = asv.load()
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            names |= _declared(h)
    assert len(names) > 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    from anisotropic_supervoxel_gb300 import _lib
    assert names == set(_lib.SIGNATURES), names ^ set(_lib.SIGNATURES)


def test_status_strings_and_defaults(asv):
    lib = asv.load()
    for st in range(8):
        assert lib.asv_status_string(st)
    from anisotropic_supervoxel_gb300._lib import Config
    c = Config()
    lib.asv_config_default(ctypes.byref(c))
    assert (c.variant, c.lloyd_iters, c.density_adjust, c.use_graph) == (0, 20, 1, 1)
    assert lib.asv_version() >= 100


def test_clip_bytes(asv):
    lib = asv.load()
    n = lib.asv_clip_bytes(320, 240, 85, 1000)
    assert 320 * 240 * 85 * 27 < n < 320 * 240 * 85 * 60
    assert lib.asv_clip_bytes(0, 240, 85, 1000) == 0
    assert lib.asv_clip_bytes(320, 240, 1, 1000) == 0


def test_create_reports_missing_device(asv):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(asv.AsvError) as e:
        asv.Image()
    assert e.value.status == 7
    with pytest.raises(asv.AsvError) as e:
        asv.Server(max_slots=2)
    assert e.value.status == 7


def test_batch_bytes_is_sum_of_clips(asv):
    import ctypes
    import numpy as np
    lib = asv.load()
    dims = [(64, 48, 12, 120), (40, 32, 9, 60), (96, 64, 16, 300)]
    arr = [np.ascontiguousarray([d[i] for d in dims], np.int32) for i in range(4)]
    ptr = [a.ctypes.data_as(ctypes.c_void_p) for a in arr]
    total = lib.asv_batch_bytes(len(dims), *ptr)
    parts = [lib.asv_clip_bytes(*d) for d in dims]
    assert 0 < total <= sum(parts)
    assert total >= sum(parts) - 2 * 32 * 256 * len(dims)


def test_synth_deterministic_and_windowed(asv):
    a = asv.synth_clip(64, 48, 10, n_ellipses=5, seed=11, jitter=0.5, drift_amp=3.0)
    b = asv.synth_clip(64, 48, 10, n_ellipses=5, seed=11, jitter=0.5, drift_amp=3.0)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    w = asv.synth_clip(64, 48, 4, n_ellipses=5, seed=11, jitter=0.5, drift_amp=3.0, frame0=6)
    for x, y in zip(a, w):
        assert np.array_equal(x[6:10], y)


def test_synth_flow_is_the_motion(asv):
    """Noise-free clip: each foreground pixel shows the same colour one frame later at
    p + round(flow) (up to occlusion by other ellipses and the ellipse border)."""
    rgb, fwd, bwd = asv.synth_clip(96, 72, 6, n_ellipses=3, noise_sigma=0.0, vmax=3.0, seed=5)
    D, H, W, _ = rgb.shape
    ok = tot = 0
    for f in range(D - 1):
        ys, xs = np.nonzero(np.abs(fwd[f]).sum(-1) > 0.5)
        nx = np.clip(np.round(xs + fwd[f, ys, xs, 0]).astype(int), 0, W - 1)
        ny = np.clip(np.round(ys + fwd[f, ys, xs, 1]).astype(int), 0, H - 1)
        ok += (np.abs(rgb[f + 1, ny, nx].astype(int) - rgb[f, ys, xs].astype(int)).max(-1) == 0).sum()
        tot += ys.size
    assert tot > 0 and ok / tot > 0.9
    assert np.allclose(bwd[1:][np.abs(fwd[:-1]).sum(-1) > 0.5].sum(), -fwd[:-1][np.abs(fwd[:-1]).sum(-1) > 0.5].sum(),
                       rtol=0.2, atol=1e3)


def test_preprocess_frame_blur_flip(asv):
    rng = np.random.default_rng(0)
    bgr = rng.integers(0, 256, (9, 13, 3), dtype=np.uint8)
    got = asv.preprocess_frame(bgr)
    p = np.pad(bgr.astype(np.int64), ((1, 1), (1, 1), (0, 0)), mode="reflect")
    k = np.array([1, 2, 1])
    acc = sum(k[j] * k[i] * p[j:j + 9, i:i + 13] for j in range(3) for i in range(3))
    want = ((acc + 8) >> 4).astype(np.uint8)[::-1, :, ::-1]
    assert np.array_equal(got, want)


def test_labels_txt_format(asv, tmp_path):
    lab = np.array([[[0, 12], [345, -1]], [[6789, 5], [1, 2]]], np.int32)   # D=2, H=2, W=2
    p = str(tmp_path / "k.txt")
    asv.write_labels_txt(p, lab)
    txt = open(p).read()
    want = ""
    for t in range(2):
        for i in (1, 0):
            want += "".join(f"{v:<4d} " for v in lab[t, i]) + "\n"
        want += "\n\n"
    assert txt == want


def test_render_ppm(asv, tmp_path):
    lab = np.array([[[0, 1], [-1, 1]]], np.int32)
    prefix = str(tmp_path / "f_")
    asv.write_render_ppm(prefix, lab, 2)
    data = open(prefix + "00000.ppm", "rb").read()
    assert data.startswith(b"P6\n2 2\n255\n")
    px = np.frombuffer(data[len(b"P6\n2 2\n255\n"):], np.uint8).reshape(2, 2, 3)
    assert (px[0, 0] == 0).all()          # label -1 (row y=1 shown first) is black
    assert (px[0, 1] == px[1, 1]).all()   # both label 1


def test_shape_limits_agree_with_oracle(asv):
    """The library and the CPU restatement accept and refuse the same clip
    shapes: one frame, one-pixel-wide or -high frames are refused by both."""
    from oracle import oracle
    lib = asv.load()
    for (W, H, D, K) in [(40, 30, 1, 20), (1, 40, 10, 8), (40, 1, 10, 8), (1, 1, 50, 5),
                         (40, 30, 2, 30), (2, 2, 2, 1), (64, 64, 64, 32767)]:
        accepted = lib.asv_clip_bytes(W, H, D, K) > 0
        rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=3, noise_sigma=3.0, seed=W + H + D)
        try:
            oracle.run_clip(rgb, fwd, bwd, K, iters=1, nthreads=4)
            ran = True
        except ValueError:
            ran = False
        assert accepted == ran, (W, H, D, K)
