"""Generates the golden fixtures of tests/golden/ from the reference's own
shaders compiled as C++ (oracle/build_ref.py; needs the reference tree).

    python tests/golden/make_golden.py

Fixtures (npz): inputs plus the compiled reference shaders' outputs for
RGB2LAB.fs (a seeded sample of RGB values), derivative_t.gs, flood.gs (one
pass at several steps) and aver_exception.vs, and of the reference's
Image::EnforceLabelConnectivity3D (connectivity.npz), Image::init_seeds
(seed_grid.npz), Image::sequence_label (sequence_label.npz) and the host
parts of Image::initialization (density_placement.npz) compiled from its C++,
and check_dead_seeds' 1-3 dead-seed branch (label_replace.gs with its host
loop, then sequence_label: few_dead.npz) and the JFA pass ladder with its ratio
uniforms (Image::init_variables and Image::flood: flood_ladder.npz).
tests/test_golden.py checks the CPU restatement and the CUDA path against
them.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))


def main():
    from oracle import build_ref, oracle
    import test_ref_pin as pin
    import anisotropic_supervoxel_gb300 as asv

    path = build_ref.build()
    if path is None:
        raise SystemExit("reference tree not present")
    lib = ctypes.CDLL(path)
    V = ctypes.c_void_p
    lib.ref_rgb2lab.argtypes = [V, ctypes.c_long, V]
    lib.ref_derivative.argtypes = [V, ctypes.c_int, ctypes.c_int, ctypes.c_int, V]
    lib.ref_flood.argtypes = [V, V, V, V, V, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.c_float, ctypes.c_float, V]
    lib.ref_aver_exception.argtypes = [V, V, V, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, V, V]
    P = pin.P
    rng = np.random.default_rng(20240610)

    rgb = rng.integers(0, 256, (16384, 3), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "rgb2lab_sample.npz"), rgb=rgb, lab=pin.ref_lab(lib, rgb))

    clip = asv.synth_clip(24, 18, 6, n_ellipses=4, noise_sigma=6.0, seed=77)[0]
    D, H, W, _ = clip.shape
    rgbf = np.ascontiguousarray(clip.astype(np.float32) / np.float32(255.0))
    g = np.zeros((D, H, W), np.float32)
    lib.ref_derivative(P(rgbf), W, H, D, P(g))
    np.savez_compressed(os.path.join(HERE, "derivative.npz"), rgb=clip, gradient=g)

    lab4 = oracle.rgb2lab(clip)
    assert np.array_equal(lab4[..., :3].astype(np.float32), pin.ref_lab(lib, clip))
    k = 20
    for step, psd in ((1, True), (3, False), (7, True)):
        seeds = pin._flood_case(rng, W, H, D, k, psd)
        labels = rng.integers(-1, k, (D, H, W)).astype(np.int32)
        ratio = np.float32(0.125)
        lt, sc, f3, l3, img = pin._textures(seeds, labels, lab4)
        out = np.zeros((D, H, W, 4), np.float32)
        lib.ref_flood(P(lt), P(sc), P(f3), P(l3), P(img), W, H, D, float(step), float(ratio), P(out))
        np.savez_compressed(os.path.join(HERE, f"flood_step{step}.npz"), rgb=clip, seeds=seeds,
                            labels=labels, step=step, ratio=ratio, out=out[..., 3].astype(np.int32))

    kp = 20
    sums = np.zeros((kp + 1, 7), np.int64)
    cnt = rng.integers(1, 60, kp + 1)
    cnt[[0, 3, kp - 1]] = 0
    for i in range(kp + 1):
        c = int(cnt[i])
        if c:
            xs, ys, zs = rng.integers(0, W, c), rng.integers(0, H, c), rng.integers(0, D, c)
            sums[i, :4] = [(2 * xs + 1).sum(), (2 * ys + 1).sum(), (2 * zs + 1).sum(), c]
            sums[i, 4:] = rng.integers(0, 256, (c, 3)).sum(0)
    sp = np.zeros((D, H, W, 4), np.float32)
    scol = np.zeros((D, H, W, 4), np.float32)
    for i in range(kp + 1):
        y, x = divmod(i, W)
        sp[0, y, x] = [np.float32(sums[i, 0]) * np.float32(0.5), np.float32(sums[i, 1]) * np.float32(0.5),
                       np.float32(sums[i, 2]) * np.float32(0.5), np.float32(sums[i, 3])]
        scol[0, y, x] = [np.float32(sums[i, 4]), np.float32(sums[i, 5]), np.float32(sums[i, 6]),
                         np.float32(sums[i, 3])]
    img = np.ascontiguousarray(lab4[..., :3].astype(np.float32))
    pos = np.zeros((kp, 4), np.float32)
    col = np.zeros((kp, 3), np.float32)
    for i in range(kp):
        lib.ref_aver_exception(P(sp), P(scol), P(img), W, H, D, i, P(pos[i]), P(col[i]))
    np.savez_compressed(os.path.join(HERE, "aver_exception.npz"), rgb=clip, sums=sums, pos=pos, col=col)

    # Image::EnforceLabelConnectivity3D, compiled from the reference's C++
    host = ctypes.CDLL(build_ref.build_host())
    host.ref_enforce_connectivity.argtypes = [V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, V]
    host.ref_enforce_connectivity.restype = ctypes.c_int
    arrays = {}
    for i, (labels, supsz) in enumerate(pin.connectivity_cases(np.random.default_rng(31))):
        D, H, W = labels.shape
        out = np.empty_like(labels)
        n = host.ref_enforce_connectivity(P(labels), W, H, D, supsz, P(out))
        arrays.update({f"labels_{i}": labels, f"out_{i}": out, f"supsz_{i}": supsz, f"n_{i}": n})
    np.savez_compressed(os.path.join(HERE, "connectivity.npz"), **arrays)

    # Image::init_seeds and Image::sequence_label, compiled from the reference's C++
    host.ref_init_seeds.argtypes = [ctypes.c_int] * 5 + [V, ctypes.c_int, V]
    host.ref_init_seeds.restype = ctypes.c_int
    host.ref_sequence_label.argtypes = [V, ctypes.c_long, V, ctypes.c_int, ctypes.c_int]
    arrays = {}
    for i, (W, H, D, K) in enumerate(pin.GRID_SHAPES):
        if K > 3000:
            continue                                   # fixtures stay small; the pin test covers these
        for mb in (0, 1):
            g5 = np.zeros(5, np.int32)
            n = host.ref_init_seeds(W, H, D, K, mb, None, 0, P(g5))
            seeds = np.zeros((n, 4), np.float32)
            host.ref_init_seeds(W, H, D, K, mb, P(seeds), n, P(g5))
            arrays.update({f"shape_{i}_{mb}": np.array([W, H, D, K, mb]), f"seeds_{i}_{mb}": seeds,
                           f"grid_{i}_{mb}": g5})
    np.savez_compressed(os.path.join(HERE, "seed_grid.npz"), **arrays)
    arrays = {}
    for i, (labels, counts, kp) in enumerate(pin.sequence_label_cases(np.random.default_rng(41))):
        dead = int((counts[:kp] < 1).sum())
        if dead in (1, 2, 3):
            continue
        out = labels.copy()
        host.ref_sequence_label(P(out), out.size, P(counts), kp, 1 if dead > 3 else 0)
        arrays.update({f"labels_{i}": labels, f"counts_{i}": counts, f"kp_{i}": kp, f"out_{i}": out})
    np.savez_compressed(os.path.join(HERE, "sequence_label.npz"), **arrays)

    # the host parts of Image::initialization (cell-id grid, redistribution)
    host.ref_initialization.argtypes = [ctypes.c_int] * 5 + [V, V, V, ctypes.c_int]
    host.ref_initialization.restype = ctypes.c_int
    arrays = {}
    for i, (W, H, D, K, mb) in enumerate(DENSITY_CASES):
        rgb, _, _ = asv.synth_clip(W, H, D, n_ellipses=5, noise_sigma=4.0, seed=W * D + K)
        s4, g = oracle.grid_seeds(W, H, D, K, middlebury=mb)
        _, dens = oracle.density_adjust(rgb, s4, g)
        dens = np.ascontiguousarray(dens, np.float32)
        grid = np.empty((D, H, W), np.float32)
        seeds = np.zeros((g.Kp, 4), np.float32)
        n = host.ref_initialization(W, H, D, K, mb, P(dens), P(grid), P(seeds), g.Kp)
        arrays.update({f"case_{i}": np.array([W, H, D, K, mb]), f"seeds_{i}": seeds[:n], f"grid_{i}": grid})
    np.savez_compressed(os.path.join(HERE, "density_placement.npz"), **arrays)

    # check_dead_seeds with 1-3 dead seeds: label_replace.gs and sequence_label
    lib.ref_label_replace.argtypes = [V] + [ctypes.c_int] * 5 + [V]
    arrays = {}
    for i, (labels, counts, kp, dead) in enumerate(pin.few_dead_cases(np.random.default_rng(47))):
        out = pin.reference_few_dead(lib, host, labels, counts, kp, dead)
        arrays.update({f"labels_{i}": labels, f"counts_{i}": counts, f"kp_{i}": kp, f"out_{i}": out})
    np.savez_compressed(os.path.join(HERE, "few_dead.npz"), **arrays)

    # Image::init_variables + Image::flood: the pass ladder and ratio uniforms
    n = len(pin.LADDER_S)
    steps, ratios = np.zeros((n, 64), np.float32), np.zeros((n, 64), np.float32)
    count, ratio = np.zeros(n, np.int32), np.zeros(n, np.float32)
    for i, s in enumerate(pin.LADDER_S):
        st, ra, ratio[i] = pin.reference_ladder(host, s)
        count[i] = st.size
        steps[i, :st.size], ratios[i, :st.size] = st, ra
    np.savez_compressed(os.path.join(HERE, "flood_ladder.npz"), s=np.int32(pin.LADDER_S), count=count,
                        ratio=ratio, steps=steps, ratios=ratios)
    labels_txt(host)
    stream_scheduler(host)
    print("fixtures written to", HERE)


def stream_scheduler(host):
    """the streaming program's block partition and kept seeds
    (streamGPU-AS/Render.cpp:199-241, :519-540): stream_scheduler.npz"""
    V = ctypes.c_void_p
    host.ref_stream_blocks.argtypes = [ctypes.c_int, V, ctypes.c_int]
    host.ref_stream_keep.argtypes = [V, ctypes.c_int, ctypes.c_int, V]
    Ds = np.array(list(range(2, 200)) + [899, 900, 901], np.int32)
    iv = np.zeros((Ds.size, 512), np.int32)
    nb = np.zeros(Ds.size, np.int32)
    for i, D in enumerate(Ds):
        nb[i] = host.ref_stream_blocks(int(D), iv[i].ctypes.data_as(V), 512)
    rng = np.random.default_rng(20240612)
    info = np.zeros((2000, 4), np.float32)
    info[:, 0] = rng.integers(0, 1280, 2000) + 0.5
    info[:, 1] = rng.integers(0, 720, 2000) + 0.5
    info[:, 2] = rng.integers(0, 30, 2000) + 0.5
    info[::5, 2] = 20.0
    info[:, 3] = np.arange(2000)
    kept = np.zeros((2000, 4), np.float32)
    nk = host.ref_stream_keep(info.ctypes.data_as(V), 2000, 30, kept.ctypes.data_as(V))
    np.savez_compressed(os.path.join(HERE, "stream_scheduler.npz"), D=Ds, blocks=nb, intervals=iv, info=info,
                        kept=kept[:nk])


def labels_txt(host):
    """Image::print_sv_txt: label volumes and the bytes of the txt file the
    reference writes for them (labels_txt.npz)."""
    import tempfile
    host.ref_print_sv_txt.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_char_p]
    rng = np.random.default_rng(20240611)
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        for i, (D, H, W, hi) in enumerate([(3, 5, 7, 20), (2, 4, 6, 99999), (1, 1, 1, 5), (2, 1, 13, 1500)]):
            lab = rng.integers(-1, hi, (D, H, W)).astype(np.int32)
            stem = os.path.join(tmp, f"k{i}")
            host.ref_print_sv_txt(lab.ctypes.data_as(ctypes.c_void_p), W, H, D, stem.encode())
            arrays[f"labels_{i}"] = lab
            arrays[f"txt_{i}"] = np.frombuffer(open(stem + ".txt", "rb").read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "labels_txt.npz"), **arrays)


# clips of the density-placement fixture (W, H, D, K, middlebury); the clip is
# asv_synth_clip(W, H, D, n_ellipses=5, noise_sigma=4.0, seed=W * D + K)
DENSITY_CASES = [(64, 48, 12, 60, 0), (37, 23, 9, 25, 0), (120, 80, 15, 300, 0), (50, 50, 5, 3000, 0),
                 (64, 48, 12, 60, 1)]


if __name__ == "__main__":
    main()
