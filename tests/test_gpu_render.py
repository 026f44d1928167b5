"""The C++ drop-in of the reference's Render::run (asv_render_run and
asv_render_stream_run, include/asv_host.h): a small C++ host program built
with g++ against libasv.so reads a folder of PNG frames, segments it on the
GPU and writes the txt label file and the pseudo-colour frames.  The txt must
equal, byte for byte, the file of the oracle chain on the same frames (host
preprocessing, the NumPy flow restatement, the oracle's clip or streaming
run), written in print_sv_txt's format (pinned to the reference's compiled
print_sv_txt by tests/golden/labels_txt.npz)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _txt(labels):
    D, H, W = labels.shape
    out = []
    for t in range(D):
        for i in range(H - 1, -1, -1):
            out.append("".join(f"{v:<4d} " for v in labels[t, i]) + "\n")
        out.append("\n\n")
    return "".join(out).encode()


@pytest.fixture(scope="module")
def render_main(asv, tmp_path_factory):
    from anisotropic_supervoxel_gb300 import _build
    asv.load()
    exe = str(tmp_path_factory.mktemp("bin") / "render_main")
    lib_dir = os.path.dirname(_build.LIB)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "render_main.cpp"), "-o", exe, "-L", lib_dir, "-l:libasv.so",
                    f"-Wl,-rpath,{lib_dir}"], check=True, capture_output=True)
    return exe


def _video(asv, tmp, W, H, D, seed):
    rgb0, _, _ = asv.synth_clip(W, H, D, n_ellipses=5, noise_sigma=3.0, jitter=0.3, drift_amp=1.0,
                                drift_period=30.0, seed=seed)
    bgr = np.ascontiguousarray(rgb0[:, ::-1, :, ::-1])          # frames as files hold them
    folder = tmp / "PNGImages" / "clipA"
    folder.mkdir(parents=True)
    for t in range(D):
        asv.write_png(str(folder / f"{t + 1:05d}.png"), bgr[t][..., ::-1])
    rgb = np.stack([asv.preprocess_frame(bgr[z]) for z in range(D)])
    return rgb


def _run(exe, mode, tmp, K, iters):
    p = subprocess.run([exe, mode, str(tmp / "PNGImages"), str(tmp / "results") + "/", "synth", "clipA", str(K),
                        str(iters)], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    return tmp / "results" / "synth" / "AS" / "clipA"


def test_render_run_plain_matches_oracle(asv, orc, render_main, tmp_path):
    from oracle import flow as ofl
    W, H, D, K, iters = 64, 48, 8, 90, 3
    rgb = _video(asv, tmp_path, W, H, D, 31)
    out = _run(render_main, "plain", tmp_path, K, iters)
    fwd, bwd = ofl.compute_flow(rgb)
    want, _, _, info = orc.run_clip(rgb, fwd, bwd, K, iters=iters, nthreads=8)
    assert (out / f"{K}.txt").read_bytes() == _txt(want)
    pngs = sorted(p for p in os.listdir(out) if p.endswith(".png"))
    assert pngs == [f"{K}_{t + 1:05d}.png" for t in range(D)]
    colours = asv.render_rgb(want, info["final_label_num"])
    assert np.array_equal(asv.read_png(str(out / pngs[2]))[..., ::-1], colours[2])


def test_render_run_stream_matches_oracle(asv, orc, render_main, tmp_path):
    from oracle import flow as ofl
    W, H, D, K, iters = 48, 40, 50, 250, 3                    # two blocks; seeds_num_100 = 500
    rgb = _video(asv, tmp_path, W, H, D, 32)
    out = _run(render_main, "stream", tmp_path, K, iters)
    fwd, bwd = ofl.compute_flow(rgb)
    want, info = orc.run_stream(rgb, fwd, bwd, K_video=K, iters=iters, nthreads=8)
    assert info["blocks"] == 2
    assert (out / f"{K}.txt").read_bytes() == _txt(want)
    assert len([p for p in os.listdir(out) if p.endswith(".png")]) == D


def test_render_run_errors(render_main, tmp_path):
    (tmp_path / "PNGImages" / "empty").mkdir(parents=True)
    p = subprocess.run([render_main, "plain", str(tmp_path / "PNGImages"), str(tmp_path) + "/", "db", "empty", "10",
                        "2"], capture_output=True, text=True)
    assert p.returncode == 1 and "render failed: -2" in p.stderr
