"""Known-answer tests of the CPU restatement (no GPU).

The reference ships no tests or fixtures; these answers come from the
maths and constants of its code (cited per test), and the golden fixtures
under tests/golden/ pin whole runs.
"""
import struct

import numpy as np
import pytest


def test_grid_seed_counts(orc):
    """Seed grid sizes of the workloads (GPU-AS/Image.cpp:20-92)."""
    cases = {(240, 160, 30, 200): (187, 17), (320, 240, 85, 1000): (936, 18),
             (640, 480, 120, 2000): (2000, 26), (1280, 720, 30, 2000): (1947, 23)}
    for (W, H, D, K), (kp, s) in cases.items():
        _, g = orc.grid_seeds(W, H, D, K)
        assert (g.Kp, g.s) == (kp, s)


def test_grid_positions_are_voxel_centres(orc):
    s4, g = orc.grid_seeds(240, 160, 30, 200)
    assert np.all(s4[:, :3] - np.floor(s4[:, :3]) == 0.5)
    assert np.array_equal(s4[:, 3], np.arange(g.Kp))
    assert s4[:, 0].max() < 240 and s4[:, 1].max() < 160 and s4[:, 2].max() < 30


@pytest.mark.parametrize("s,steps", [(17, [1, 8, 4, 2, 1, 2, 1]), (18, [1, 9, 5, 3, 2, 1, 2, 1]),
                                     (23, [1, 11, 6, 3, 2, 1, 2, 1]), (26, [1, 13, 7, 4, 2, 1, 2, 1]),
                                     (1, [1, 2, 1]), (3, [1, 1, 2, 1])])
def test_ladder(orc, s, steps):
    """JFA step ladder (GPU-AS/Image.cpp:1055-1190); last two passes at 2x ratio."""
    st, rm = orc.ladder(s)
    assert st == steps
    assert rm == [1.0] * (len(steps) - 2) + [2.0, 2.0]


def test_full_ladder(orc):
    st, rm = orc.ladder(17, full=1, maxdim=240)
    assert st == [1, 128, 64, 32, 16, 8, 4, 2, 1, 2, 1]


def test_ratio(orc):
    """ratio = (compactness/s)^2 in float (Image.cpp:1050-1051)."""
    c = np.float32(8.0) / np.float32(17)
    assert orc.ratio(17, 8.0) == np.float32(c * c)


def _lab_ref(rgb):
    """RGB2LAB.fs:11-79 in numpy float32 (correctly rounded pow via float64)."""
    c = np.asarray(rgb, np.float32) / np.float32(255.0)
    lin = np.where(c <= np.float32(0.04045), c / np.float32(12.92),
                   np.power(((c + np.float32(0.055)) / np.float32(1.055)).astype(np.float64),
                            np.float64(np.float32(2.4))).astype(np.float32))
    px = np.array([0.412453, 0.357580, 0.180423], np.float32)
    py = np.array([0.212671, 0.715160, 0.072169], np.float32)
    pz = np.array([0.019334, 0.119193, 0.950227], np.float32)

    def dot(p):
        return (lin[..., 0] * p[0] + lin[..., 1] * p[1]) + lin[..., 2] * p[2]

    r = np.stack([dot(px) / np.float32(0.950456), dot(py) / np.float32(1.0),
                  dot(pz) / np.float32(1.088754)], -1)
    e = np.float64(np.float32(1.0) / np.float32(3.0))
    f = np.where(r > np.float32(0.008856), np.power(r.astype(np.float64), e).astype(np.float32),
                 (np.float32(903.3) * r + np.float32(16.0)) / np.float32(116.0))
    L = (np.float32(116.0) * f[..., 1] - np.float32(16.0)) * np.float32(2.55)
    A = np.float32(500.0) * (f[..., 0] - f[..., 1]) + np.float32(128.0)
    B = np.float32(200.0) * (f[..., 1] - f[..., 2]) + np.float32(128.0)
    return np.clip(np.floor(np.stack([L, A, B], -1) + np.float32(0.5)), 0, 255).astype(np.uint8)


def test_rgb2lab_known_colours(orc):
    cols = np.array([[255, 255, 255], [0, 0, 0], [255, 0, 0], [0, 255, 0], [0, 0, 255],
                     [128, 128, 128]], np.uint8)
    got = orc.rgb2lab(cols)[:, :3].astype(int)
    # CIELAB D65 of the sRGB primaries (L*2.55, a+128, b+128, rounded)
    assert list(got[0]) == [255, 128, 128]
    assert list(got[1]) == [0, 128, 128]
    assert abs(got[2] - [136, 208, 195]).max() <= 1
    assert abs(got[3] - [224, 42, 211]).max() <= 1
    assert abs(got[4] - [82, 207, 20]).max() <= 1
    assert got[5][1] == 128 and got[5][2] == 128


def test_rgb2lab_matches_numpy_restatement(orc):
    rng = np.random.default_rng(3)
    rgb = rng.integers(0, 256, (200000, 3), dtype=np.uint8)
    assert np.array_equal(orc.rgb2lab(rgb)[:, :3], _lab_ref(rgb))


def test_float_to_half_matches_numpy(orc):
    vals = np.concatenate([np.arange(0, 40000, 1, dtype=np.float32),
                           np.random.default_rng(0).uniform(0, 800, 20000).astype(np.float32)])
    got = np.array([orc.load().orc_float_to_half(float(v)) for v in vals[::7]], np.uint16)
    want = vals[::7].astype(np.float16).view(np.uint16)
    assert np.array_equal(got, want)


def test_gradient_matches_numpy(orc):
    """derivative_t.gs:24-49: 0.33 * sum |dRGB| over left, y-1 and previous frame."""
    rng = np.random.default_rng(4)
    rgb = rng.integers(0, 256, (5, 7, 9, 3), dtype=np.uint8)
    c = rgb.astype(np.int32)
    nb = [np.concatenate([c[:, :, :1], c[:, :, :-1]], 2), np.concatenate([c[:, :1], c[:, :-1]], 1),
          np.concatenate([c[:1], c[:-1]], 0)]
    g = np.zeros(rgb.shape[:3], np.float32)
    for n in nb:
        d = np.abs(n - c).astype(np.float32)
        s = (d[..., 0] + d[..., 1]) + d[..., 2]
        g = g + np.float32(0.33) * s
    assert np.array_equal(orc.gradient_half(rgb), g.astype(np.float16).view(np.uint16))


def test_flow_angle_threshold():
    """T = smallest float c with float(double(acos_cr(c)) * (180/3.141592653)) < 90."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 120
    T = 1.5893254712295857e-08

    def theta(c):
        a = np.float32(float(mpmath.acos(mpmath.mpf(float(c)))))
        return np.float32(np.float64(a) * (180.0 / 3.141592653))

    below = struct.unpack("<f", struct.pack("<I", 0x328885A3 - 1))[0]
    assert struct.pack("<f", T) == struct.pack("<I", 0x328885A3)
    assert theta(T) < 90 and not theta(below) < 90


def test_slot_mapping_is_exact():
    """centroids.vs:38-43 / density_grid.vs:28-30 map id -> texel (id mod W, id div W)
    through float math; under IEEE float it is the integer mapping for these widths."""
    for W in (146, 240, 320, 352, 640, 1280):
        r = np.float32(1.0) / np.float32(W)
        ids = np.arange(0, 40000, dtype=np.float32)
        y = np.floor(ids * r)
        x = np.floor(ids - y / r)
        assert np.array_equal(y.astype(np.int64), np.arange(40000) // W)
        assert np.array_equal(x.astype(np.int64), np.arange(40000) % W)


def test_metric_zero_flow_is_identity(orc):
    W, H, D = 12, 10, 4
    z = np.zeros((D, H, W, 2), np.float32)
    M, neg = orc.metric_solve(z, z, 5.0, 5.0, 2)
    assert neg == 0
    assert np.allclose(M, [1, 0, 0, 1, 0, 1], atol=1e-5)


@pytest.mark.parametrize("fx,fy", [(1.0, 0.0), (2.0, -1.0), (-1.0, 3.0)])
def test_metric_pure_translation(orc, fx, fy):
    """With the true flow the system is consistent: M = S^T S,
    S = [[1,0,-fx],[0,1,-fy],[0,0,1]] (Image.cpp:884-930)."""
    W, H, D = 12, 10, 4
    fwd = np.zeros((D, H, W, 2), np.float32)
    fwd[..., 0], fwd[..., 1] = fx, fy
    bwd = -fwd
    S = np.array([[1, 0, -fx], [0, 1, -fy], [0, 0, 1]], np.float64)
    want = S.T @ S
    M, neg = orc.metric_solve(fwd, bwd, 5.0, 5.0, 2)
    assert neg == 0
    got = np.array([[M[0], M[1], M[2]], [M[1], M[3], M[4]], [M[2], M[4], M[5]]])
    assert np.allclose(got, want, atol=2e-4 * max(1.0, np.abs(want).max()))


def test_single_seed_labels_everything(orc):
    W, H, D = 20, 16, 6
    rng = np.random.default_rng(1)
    rgb = rng.integers(0, 256, (D, H, W, 3), dtype=np.uint8)
    lab4 = orc.rgb2lab(rgb)
    seeds = np.zeros((1, 12), np.float32)
    seeds[0, :3] = [10.5, 8.5, 3.5]
    seeds[0, 3:6] = lab4[3, 8, 10, :3]
    seeds[0, 6:12] = [1, 0, 0, 1, 0, 1]
    labels = orc.draw_seeds((D, H, W), seeds[:, :3])
    for st in orc.ladder(3)[0] + [8, 4, 2, 1]:
        labels = orc.jfa_pass(labels, lab4, seeds, st, 0.1)
    assert (labels == 0).all()


def test_jfa_euclidean_close_to_brute_force(orc):
    """M = I, uniform colour: JFA labels ~ Euclidean nearest seed."""
    W, H, D = 40, 32, 12
    rgb = np.full((D, H, W, 3), 120, np.uint8)
    lab4 = orc.rgb2lab(rgb)
    rng = np.random.default_rng(2)
    k = 25
    seeds = np.zeros((k, 12), np.float32)
    seeds[:, 0] = rng.integers(0, W, k) + 0.5
    seeds[:, 1] = rng.integers(0, H, k) + 0.5
    seeds[:, 2] = rng.integers(0, D, k) + 0.5
    seeds[:, 3:6] = lab4[0, 0, 0, :3]
    seeds[:, 6:12] = [1, 0, 0, 1, 0, 1]
    labels = orc.draw_seeds((D, H, W), seeds[:, :3])
    for st in [1, 16, 8, 4, 2, 1, 2, 1]:
        labels = orc.jfa_pass(labels, lab4, seeds, st, 1.0)
    zz, yy, xx = np.meshgrid(np.arange(D) + 0.5, np.arange(H) + 0.5, np.arange(W) + 0.5, indexing="ij")
    d2 = ((xx[..., None] - seeds[:, 0]) ** 2 + (yy[..., None] - seeds[:, 1]) ** 2
          + (zz[..., None] - seeds[:, 2]) ** 2)
    best = d2.min(-1)
    got = np.take_along_axis(d2, labels[..., None].astype(np.int64), -1)[..., 0]
    assert (labels >= 0).all()
    assert np.mean(got == best) > 0.99


def _sequence_label(labels, rank, dead_seed):
    """GPU-AS/Image.cpp:1727-1778 as written (raster loops, std::map [] -> 0)."""
    lab = labels.ravel().copy()

    def mp(v):
        return rank.get(int(v), 0)

    if dead_seed:
        last_label = int(lab[0])
        last_map = mp(last_label)
        lab[0] = last_map
        for i in range(1, lab.size):
            if lab[i] != last_label and lab[i] != -1:
                last_map = mp(lab[i])
            lab[i] = last_map
    else:
        last = 0
        if lab[0] >= 0:
            last = int(lab[0])
        for i in range(1, lab.size):
            if lab[i] != last:
                if lab[i] == -1:
                    lab[i] = last
                last = int(lab[i])
    return lab.reshape(labels.shape)


def _check_dead_seeds(raw, kp):
    """GPU-AS/Image.cpp:1579-1720 on a raw label volume."""
    cnt = np.bincount(np.where(raw < 0, kp, raw).ravel(), minlength=kp + 1)
    invalid = cnt[kp] > 0
    dead = [i for i in range(kp) if cnt[i] < 1]
    rank, v = {}, 0
    for i in range(kp):
        if cnt[i] >= 1:
            rank[i] = v
            v += 1
    lab = raw.copy()
    if len(dead) == 0:
        if invalid:
            lab = _sequence_label(lab, rank, False)
    elif len(dead) <= 3:
        last = kp
        for d in dead:
            last -= 1
            lab[lab == last] = d
        if invalid:
            lab = _sequence_label(lab, rank, False)
    else:
        lab = _sequence_label(lab, rank, True)
    return lab


@pytest.mark.parametrize("case", range(6))
def test_postprocess_matches_reference_loops(orc, case):
    rng = np.random.default_rng(10 + case)
    D, H, W, kp = 3, 9, 11, 20
    raw = rng.integers(0, kp, (D, H, W)).astype(np.int32)
    if case in (1, 3, 5):
        raw[rng.random(raw.shape) < 0.1] = -1
    if case == 2:
        raw[np.isin(raw, [4, kp - 1])] = 0
    if case in (3, 4):
        raw[np.isin(raw, [0, 1, 5, 6, 9])] = 3
    if case == 5:
        raw[0, 0, 0] = -1
        raw[np.isin(raw, [kp - 1, kp - 2, kp - 3])] = 2
    lab4 = np.zeros((D, H, W, 4), np.uint8)
    sums = orc.centroid_sums(raw, lab4, kp)
    got, stats = orc.postprocess(raw, sums, kp)
    assert np.array_equal(got, _check_dead_seeds(raw, kp))


def test_centroid_sums_exact(orc):
    rng = np.random.default_rng(5)
    D, H, W, kp = 4, 6, 8, 5
    raw = rng.integers(-1, kp, (D, H, W)).astype(np.int32)
    lab4 = rng.integers(0, 256, (D, H, W, 4), dtype=np.uint8)
    s = orc.centroid_sums(raw, lab4, kp)
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    for l in range(-1, kp):
        m = raw == l
        row = s[kp if l < 0 else l]
        assert row[0] == (2 * xx[m] + 1).sum() and row[1] == (2 * yy[m] + 1).sum()
        assert row[2] == (2 * zz[m] + 1).sum() and row[3] == m.sum()
        assert row[4] == lab4[m][:, 0].astype(int).sum()


def test_lloyd_uniform_colour_fixed_point(orc, asv):
    """Uniform colour, zero flow, grid seeds: after the Lloyd loop the seeds
    sit at the centroids of their regions (a fixed point of the reseed)."""
    W, H, D, K = 48, 36, 10, 40
    rgb = np.full((D, H, W, 3), 90, np.uint8)
    z = np.zeros((D, H, W, 2), np.float32)
    labels, raw, seeds, info = orc.run_clip(rgb, z, z, K, iters=8, density_adjust=0)
    assert info["dead"] == 0 and info["neg"] == 0
    lab4 = orc.rgb2lab(rgb)
    sums = orc.centroid_sums(raw, lab4, info["Kp"])
    cen = np.floor((sums[:-1, :3] / 2.0) / sums[:-1, 3:4]) + 0.5
    assert np.abs(cen - seeds[:, :3]).max() <= 1.0


def _negative_exact(M):
    """some eigenvalue < 0, in exact rational arithmetic (principal minors)"""
    from fractions import Fraction as F
    a, b, c, d, e, f = (F(float(v)) for v in M)
    minors = [a, d, f, a * d - b * b, a * f - c * c, d * f - e * e,
              a * (d * f - e * e) - b * (b * f - c * e) + c * (b * e - d * c)]
    return int(any(m < 0 for m in minors))


def test_psd_test_is_exact(orc):
    """The metric's PSD test (Image.cpp:997-1006, decided exactly) against
    rational arithmetic: random, rank-deficient, exactly singular and
    near-singular symmetric matrices."""
    rng = np.random.default_rng(17)
    cases = []
    for _ in range(3000):
        cases.append(rng.normal(size=6).astype(np.float32))
    for _ in range(1500):                      # S^T S of 1 or 2 rows: PSD, rank 1/2
        S = rng.normal(size=(int(rng.integers(1, 3)), 3)).astype(np.float32)
        A = (S.T.astype(np.float64) @ S.astype(np.float64)).astype(np.float32)
        cases.append(np.array([A[0, 0], A[0, 1], A[0, 2], A[1, 1], A[1, 2], A[2, 2]], np.float32))
    for _ in range(1500):                      # integer matrices: many exactly singular
        v = rng.integers(-3, 4, size=3).astype(np.float32)
        w = rng.integers(-3, 4, size=3).astype(np.float32)
        A = np.outer(v, v) + (rng.integers(0, 2) * np.outer(w, w))
        cases.append(np.array([A[0, 0], A[0, 1], A[0, 2], A[1, 1], A[1, 2], A[2, 2]], np.float32))
    cases += [np.zeros(6, np.float32), np.array([1, 1, 0, 1, 0, 0], np.float32),
              np.array([1, 0, 0, 1, 0, -1e-30], np.float32), np.array([1e-20, 1e-10, 0, 1, 0, 1], np.float32),
              np.array([3e38, 1e38, 0, 3e38, 0, 1e-38], np.float32)]
    for M in cases:
        assert orc.m6_negative(M) == _negative_exact(M), M.tolist()


def test_round_half_up_fp32_form():
    """The GPU's FP32 form of floor(f + 0.5) (no FP64) equals the FP64 form on
    random bit patterns, values next to every k + 0.5 and small values."""
    rng = np.random.default_rng(0)
    f = rng.integers(0, 2 ** 32, 4_000_000, dtype=np.uint64).astype(np.uint32).view(np.float32)
    near = (rng.integers(-2 ** 24, 2 ** 24, 1_000_000).astype(np.float64) + 0.5).astype(np.float32)
    near = np.concatenate([near, np.nextafter(near, np.float32(np.inf)), np.nextafter(near, np.float32(-np.inf))])
    f = np.concatenate([f, near, rng.uniform(-3, 3, 1_000_000).astype(np.float32),
                        np.array([0.0, -0.0, 0.5, -0.5, 0.49999997, -0.49999997, np.inf, -np.inf], np.float32)])
    with np.errstate(all="ignore"):
        want = np.floor(f.astype(np.float64) + 0.5).astype(np.float32)
        r = np.floor(f)
        got = (np.where(f - r >= np.float32(0.5), r + np.float32(1), r) + np.float32(0)).astype(np.float32)
    same = (want.view(np.uint32) == got.view(np.uint32)) | (np.isnan(want) & np.isnan(got))
    assert same.all()


def test_evaluate_known_answers():
    """The quality measures on a hand-checked case: truth = left/right halves
    of a 4x4x2 volume, supervoxels = top/bottom halves."""
    from oracle import evaluate as ev
    truth = np.zeros((2, 4, 4), np.int32)
    truth[:, :, 2:] = 1
    labels = np.zeros((2, 4, 4), np.int32)
    labels[:, 2:, :] = 1
    r = ev.evaluate(labels, truth)
    # each truth half (16 voxels) meets both supervoxels (16 each): (32 - 16) / 16 = 1
    assert r["undersegmentation"] == 1.0
    # each supervoxel is split 8/8: argmax ties go to truth 0, which gets 16 of 16
    assert r["segmentation_accuracy"] == (16 / 16 + 0 / 16) / 2
    assert r["mean_duration"] == 2.0 and r["supervoxels"] == 2 and r["truth_segments"] == 2
    # truth boundary: columns 1 and 2 (16 voxels); supervoxel boundary rows 1 and 2 cross them
    assert r["truth_boundary"] == 16 and r["recalled"] == 16
    same = ev.evaluate(truth, truth)
    assert same["undersegmentation"] == 0.0 and same["segmentation_accuracy"] == 1.0
    assert same["boundary_recall"] == 1.0


def test_middlebury_step_known_answers(orc):
    """GPU-AS/Image.cpp:25-29: s = int(floor(pow(1.0 * W * H / K, 0.5))) for the
    MiddleburyFlow dataset, s = int(floor(pow(N / K, 1/3))) (N / K integer) otherwise."""
    import math
    for (W, H, D, K) in [(64, 48, 12, 60), (90, 50, 8, 120), (640, 480, 2, 1000), (37, 23, 9, 25)]:
        _, g = orc.grid_seeds(W, H, D, K, middlebury=1)
        assert g.s == int(math.floor(math.pow(1.0 * W * H / K, 0.5))), (W, H, D, K)
        _, g0 = orc.grid_seeds(W, H, D, K, middlebury=0)
        assert g0.s == int(math.floor(math.pow((W * H * D) // K, 1.0 / 3))), (W, H, D, K)


def test_oracle_generator_equals_library(asv, orc):
    """The generator library of the CPU-only runs (oracle.synth_clip)
    produces the very clips of asv.synth_clip, so both timed arms segment
    the same inputs."""
    for args in [dict(W=64, H=48, D=5, n_ellipses=6, noise_sigma=5.0, seed=3),
                 dict(W=160, H=90, D=4, n_ellipses=60, noise_sigma=5.0, vmax=3.0, drift_amp=6.0,
                      drift_period=90.0, seed=20240604, frame0=37),
                 dict(W=33, H=17, D=3, n_ellipses=2, noise_sigma=8.0, jitter=0.5, seed=9)]:
        a = asv.synth_clip(**{k: v for k, v in args.items() if k not in ("W", "H", "D")},
                           W=args["W"], H=args["H"], D=args["D"])
        b = orc.synth_clip(**{k: v for k, v in args.items() if k not in ("W", "H", "D")},
                           W=args["W"], H=args["H"], D=args["D"])
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
