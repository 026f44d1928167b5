"""CUDA path (libasv through its C ABI) against the CPU restatement.

The bar is bit-exact: the kernels evaluate every float operation in the
restatement's order and the blend-order sums are exact integers on both
sides, so labels, seeds, metrics and sums must be identical.
"""
import numpy as np
import pytest

from conftest import mismatch, small_clip

pytestmark = pytest.mark.gpu


def _gpu_clip(asv, rgb, fwd, bwd, K, iters, **cfg):
    img = asv.Image(lloyd_iters=iters, **cfg)
    img.init_gpu(rgb, K)
    img.upload_flow(fwd, bwd)
    img.initialization()
    img.seed_matrix()
    img.RGB2LAB()
    return img


def test_lab_exhaustive(asv, orc):
    """RGB -> LAB on all 2^24 RGB8 values."""
    v = np.arange(1 << 24, dtype=np.uint32)
    rgb = np.stack([(v >> 16) & 255, (v >> 8) & 255, v & 255], -1).astype(np.uint8)
    rgb = rgb.reshape(2, 2048, 4096, 3)
    img = asv.Image(lloyd_iters=1)
    img.init_gpu(rgb, 1000)
    img.RGB2LAB()
    got = img.lab()
    want = orc.rgb2lab(rgb)
    bad = np.nonzero((got[..., :3] != want[..., :3]).any(-1).ravel())[0]
    assert bad.size == 0, f"{bad.size} RGB values differ, first {bad[:10]}"


@pytest.mark.parametrize("W,H,D,K", [(64, 48, 12, 60), (37, 23, 9, 25), (240, 160, 30, 200),
                                     (96, 64, 20, 400), (50, 50, 5, 3000)])
def test_density_seeds(asv, orc, W, H, D, K):
    rgb, fwd, bwd = small_clip(asv, W, H, D, seed=W * H + K)
    grid, g = orc.grid_seeds(W, H, D, K)
    want, _ = orc.density_adjust(rgb, grid, g)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, 2)
    assert img.info().Kp == g.Kp
    got = img.seeds()
    assert mismatch(got[:, :3], want[:, :3]) == 0


@pytest.mark.parametrize("W,H,D,K,jit", [(64, 48, 12, 60, 0.0), (80, 60, 16, 150, 0.5),
                                         (33, 41, 7, 40, 0.5)])
def test_seed_matrix(asv, orc, W, H, D, K, jit):
    rgb, fwd, bwd = small_clip(asv, W, H, D, seed=3 * W + K, jitter=jit)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, 2)
    s = img.seeds()
    want, kind = orc.seed_metrics(fwd, bwd, s[:, :3], 0, 1)
    assert mismatch(s[:, 6:12].view(np.uint32), want.view(np.uint32)) == 0


def test_seed_matrix_fallbacks(asv, orc):
    """Random flow makes non-PSD solves: exercise the 1-ring, 2-ring and nearest-PSD paths."""
    W, H, D, K = 48, 40, 10, 120
    rng = np.random.default_rng(5)
    rgb = rng.integers(0, 256, (D, H, W, 3), dtype=np.uint8)
    fwd = rng.normal(0, 2.0, (D, H, W, 2)).astype(np.float32)
    bwd = rng.normal(0, 2.0, (D, H, W, 2)).astype(np.float32)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, 2)
    s = img.seeds()
    want, kind = orc.seed_metrics(fwd, bwd, s[:, :3], 0, 1)
    assert set(np.unique(kind)) >= {0, 1}
    assert mismatch(s[:, 6:12].view(np.uint32), want.view(np.uint32)) == 0


@pytest.mark.parametrize("step", [1, 2, 3, 8, 11])
def test_jfa_single_pass(asv, orc, step):
    W, H, D, K = 70, 45, 14, 80
    rgb, fwd, bwd = small_clip(asv, W, H, D, seed=11)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, 2)
    lab4 = img.lab()
    rng = np.random.default_rng(step)
    kp = img.info().Kp
    seeds = np.zeros((kp, 12), np.float32)
    seeds[:, 0] = rng.integers(0, W, kp) + 0.5
    seeds[:, 1] = rng.integers(0, H, kp) + 0.5
    seeds[:, 2] = rng.integers(0, D, kp) + 0.5
    seeds[:, 3:6] = rng.uniform(0, 255, (kp, 3)).astype(np.float32)
    A = rng.normal(0, 1, (kp, 3, 3)).astype(np.float32)
    M = np.einsum("kij,kil->kjl", A, A)
    seeds[:, 6:12] = M[:, [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]]
    seeds[: kp // 8, 6:12] *= -1.0          # some non-PSD tables (clamped distance)
    img.set_seeds(seeds)
    labels = rng.integers(-1, kp, (D, H, W)).astype(np.int32)
    ratio = 0.1234567
    got = img.jfa_pass(labels, step, ratio)
    want = orc.jfa_pass(labels, lab4, seeds, step, ratio)
    assert mismatch(got, want) == 0


def _blocky_labels(rng, shape, kp, block, minus=0.02):
    """labels constant on block^3 cubes (few labels per JFA tile footprint), some -1"""
    D, H, W = shape
    nb = [(n + block - 1) // block for n in shape]
    ids = rng.integers(0, kp, nb).astype(np.int32)
    lab = ids[np.arange(D)[:, None, None] // block, np.arange(H)[None, :, None] // block,
              np.arange(W)[None, None, :] // block]
    lab[rng.random(shape) < minus] = -1
    return np.ascontiguousarray(lab)


@pytest.mark.parametrize("zrun", [4, 16, 64])
@pytest.mark.parametrize("step", [1, 2, 3, 4, 5, 6, 8])
def test_jfa_single_pass_bitset_and_ties(asv, orc, step, zrun):
    """Labels constant on small cubes keep a sub-tile's footprint under 32
    labels, so the pass takes the bit-set form (steps <= 6; with tiles of 4
    positions only steps 1-2, the list form above); seeds come in
    identical pairs (same position, colour and metric), so pairs of labels
    tie at the least distance (thousands of voxels per case) and the
    shader's candidate order decides.  A third of the volume holds random
    labels (footprints over 32 labels: the list form)."""
    W, H, D, K = 90, 70, 40, 300
    rgb, fwd, bwd = small_clip(asv, W, H, D, seed=13)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, 2, jfa_zrun=zrun)
    lab4 = img.lab()
    rng = np.random.default_rng(100 + step)
    kp = img.info().Kp
    seeds = np.zeros((kp, 12), np.float32)
    seeds[:, 0] = rng.integers(0, W, kp) + 0.5
    seeds[:, 1] = rng.integers(0, H, kp) + 0.5
    seeds[:, 2] = rng.integers(0, D, kp) + 0.5
    seeds[:, 3:6] = rng.integers(0, 256, (kp, 3)).astype(np.float32)
    A = rng.normal(0, 0.3, (kp, 3, 3)).astype(np.float32)
    M = np.einsum("kij,kil->kjl", A, A)
    seeds[:, 6:12] = M[:, [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]]
    seeds[: kp // 8, 6:12] *= -1.0
    seeds[1::2] = seeds[0::2][: kp // 2]                  # identical pairs: exact ties
    img.set_seeds(seeds)
    labels = _blocky_labels(rng, (D, H, W), 24, 6)           # 12 tying pairs, often neighbours
    labels[: D // 2, H // 2:] = _blocky_labels(rng, (D // 2, H - H // 2, W), kp, 5)
    labels[:, :, : W // 3] = rng.integers(-1, kp, (D, H, W // 3))
    ratio = 0.0123
    got = img.jfa_pass(labels, step, ratio)
    want = orc.jfa_pass(labels, lab4, seeds, step, ratio)
    assert mismatch(got, want) == 0
    img.close()


CASES = [
    # W, H, D, K, iters, variant, full_ladder, density
    (64, 48, 12, 60, 4, 0, 0, 1),
    (64, 48, 12, 60, 4, 1, 0, 1),
    (64, 48, 12, 60, 3, 0, 1, 1),
    (64, 48, 12, 60, 3, 0, 0, 0),
    (37, 23, 9, 25, 5, 0, 0, 1),
    (120, 80, 15, 300, 3, 0, 0, 1),
    (40, 30, 6, 400, 3, 0, 0, 1),       # many seeds for the volume: dead seeds, -1 fill
    (17, 9, 3, 2, 3, 0, 0, 1),          # two seeds
]


@pytest.mark.parametrize("W,H,D,K,iters,variant,full,dens", CASES)
def test_clip_bit_exact(asv, orc, W, H, D, K, iters, variant, full, dens):
    rgb, fwd, bwd = small_clip(asv, W, H, D, seed=W + 7 * K, jitter=0.5, drift=2.0)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, iters, variant=variant, full_ladder=full,
                    density_adjust=dens)
    img.run_lloyd()
    labels, raw, seeds, info = orc.run_clip(rgb, fwd, bwd, K, iters=iters, variant=variant,
                                            full_ladder=full, density_adjust=dens)
    assert mismatch(img.raw_labels(), raw) == 0
    assert mismatch(img.labels(), labels) == 0
    assert mismatch(img.seeds().view(np.uint32), seeds.view(np.uint32)) == 0
    gi = img.info()
    assert (gi.dead, gi.neg_count, gi.final_label_num) == (info["dead"], info["neg"],
                                                           info["final_label_num"])


@pytest.mark.parametrize("full", [1, 0])
def test_clip_240x160x30(asv, orc, full):
    """The 240x160x30 K=200 10-iteration workload (its full JFA ladder, and the
    reference ladder), bit-exact end to end."""
    from anisotropic_supervoxel_gb300 import workloads
    w = workloads.CLIP_240x160x30
    assert w["full_ladder"] == 1
    rgb, fwd, bwd = workloads.make_clip(w)
    img = _gpu_clip(asv, rgb, fwd, bwd, w["K"], w["iters"], full_ladder=full)
    img.run_lloyd()
    labels, raw, seeds, info = orc.run_clip(rgb, fwd, bwd, w["K"], iters=w["iters"], nthreads=8,
                                            full_ladder=full)
    assert img.info().Kp == 187
    assert img.info().passes == (11 if full else 7)          # [1, 128, 64, ..., 1, 2, 1] or [1, 8, 4, 2, 1, 2, 1]
    assert mismatch(img.raw_labels(), raw) == 0
    assert mismatch(img.labels(), labels) == 0


def test_post_processing_cases(asv, orc):
    """Dead-seed relabel (<= 3 and > 3 dead) and the -1 forward fills on crafted volumes."""
    W, H, D, K = 40, 30, 8, 60
    rgb, fwd, bwd = small_clip(asv, W, H, D, seed=99)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, 2)
    kp = img.info().Kp
    lab4 = img.lab()
    rng = np.random.default_rng(1)
    base = rng.integers(0, kp, (D, H, W)).astype(np.int32)
    cases = []
    a = base.copy(); a[rng.random(a.shape) < 0.05] = -1; cases.append(a)          # -1 only
    b = a.copy(); b[0, 0, 0] = -1; cases.append(b)                                 # -1 at voxel 0
    c = base.copy(); c[np.isin(c, [3, kp - 1])] = 5; c[rng.random(c.shape) < 0.02] = -1
    cases.append(c)                                                                # 2 dead (incl. last)
    d = base.copy(); d[np.isin(d, [0, 1, 2, 7, 9, 11])] = 4; d[0, 0, :3] = -1
    cases.append(d)                                                                # 6 dead, -1 first
    e = base.copy(); e[np.isin(e, [kp - 3, kp - 2, kp - 1])] = 0; cases.append(e)  # 3 dead at the end
    for raw in cases:
        got = img.check_dead_seeds_host(raw)
        sums = orc.centroid_sums(raw, lab4, kp)
        want, _ = orc.postprocess(raw, sums, kp)
        assert mismatch(got, want) == 0
        assert mismatch(img.sums(), sums) == 0


def test_graph_eager_and_stage_calls_agree(asv):
    rgb, fwd, bwd = small_clip(asv, 64, 48, 12, seed=5, jitter=0.5)
    outs = []
    for use_graph in (1, 0):
        img = _gpu_clip(asv, rgb, fwd, bwd, 60, 4, use_graph=use_graph)
        img.run_lloyd()
        img.run_lloyd()          # replay: same initial seeds, same result
        outs.append(img.labels())
    img = _gpu_clip(asv, rgb, fwd, bwd, 60, 4)
    img.Ld_first_init()
    for it in range(1, 5):
        if it > 1:
            img.Ld_next_seeds_matrix(it)
        img.flood(it)
        img.centroids_next_seeds(it)
    outs.append(img.check_dead_seeds())
    assert mismatch(outs[0], outs[1]) == 0
    assert mismatch(outs[0], outs[2]) == 0


def test_clip_320x240x85_properties(asv, orc):
    """Full-size 320x240x85 K=1000 15-iteration workload: size-independent properties
    (exact sums, every voxel counted once, determinism), plus bit-exact parity on the
    half-scale clip."""
    from anisotropic_supervoxel_gb300 import workloads
    w = workloads.CLIP_320x240x85
    rgb, fwd, bwd = workloads.make_clip(w)
    img = _gpu_clip(asv, rgb, fwd, bwd, w["K"], w["iters"])
    img.run_lloyd()
    raw1, lab1 = img.raw_labels(), img.labels()
    img.run_lloyd()
    assert mismatch(img.raw_labels(), raw1) == 0
    kp = img.info().Kp
    assert kp == 936
    sums = img.sums()
    assert sums[:, 3].sum() == raw1.size
    want = orc.centroid_sums(raw1, img.lab(), kp, nthreads=8)
    assert mismatch(sums, want) == 0
    assert lab1.min() >= -1 and lab1.max() < kp
    assert (lab1.ravel()[1:] >= 0).all()
    # half scale, bit-exact
    rgb, fwd, bwd = workloads.make_clip(w, scale=0.5)
    D, H, W, _ = rgb.shape
    img = _gpu_clip(asv, rgb, fwd, bwd, w["K"] // 4, w["iters"])
    img.run_lloyd()
    labels, raw, seeds, info = orc.run_clip(rgb, fwd, bwd, w["K"] // 4, iters=w["iters"], nthreads=8)
    assert mismatch(img.raw_labels(), raw) == 0
    assert mismatch(img.labels(), labels) == 0


EXTREMES = [
    (40, 30, 2, 30),          # two frames: one forward and one backward flow field
    (2, 2, 2, 1),             # one seed in a 2x2x2 clip
    (160, 128, 8, 30000),     # K' = 29952: more seeds than a label per 6 voxels
    (64, 64, 64, 32767),      # K' = 32736, next to the 32767-seed limit; -1 voxels remain
]


@pytest.mark.parametrize("W,H,D,K", EXTREMES)
def test_clip_extremes_bit_exact(asv, orc, W, H, D, K):
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=3, noise_sigma=3.0, seed=W + H + D)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, 2)
    img.run_lloyd()
    labels, raw, seeds, info = orc.run_clip(rgb, fwd, bwd, K, iters=2, nthreads=8)
    assert img.info().Kp == seeds.shape[0]
    assert np.array_equal(img.raw_labels(), raw)
    assert np.array_equal(img.labels(), labels)
    img.close()


def test_clip_full_size_bit_exact(asv, orc):
    """a 1280x720x36 clip (33.2 M voxels, next to the 2^25-voxel limit of the
    fixed-memory path) with K=2000, two Lloyd iterations: labels identical
    before and after post-processing"""
    W, H, D, K = 1280, 720, 36, 2000
    rgb, fwd, bwd = asv.synth_clip(W, H, D, n_ellipses=60, noise_sigma=5.0, vmax=3.0, seed=20240605)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, 2)
    img.run_lloyd()
    labels, raw, seeds, info = orc.run_clip(rgb, fwd, bwd, K, iters=2, nthreads=16)
    assert img.info().Kp == seeds.shape[0] == info["Kp"]
    assert np.array_equal(img.raw_labels(), raw)
    assert np.array_equal(img.labels(), labels)
    img.close()


@pytest.mark.parametrize("W,H,D,K", [(64, 48, 12, 60), (90, 50, 8, 120)])
def test_clip_middlebury_bit_exact(asv, orc, W, H, D, K):
    """middlebury = 1: base step s = floor(sqrt(W*H/K)) (GPU-AS/Image.cpp:25-29)."""
    rgb, fwd, bwd = small_clip(asv, W, H, D, seed=W + 3 * K, jitter=0.4, drift=1.0)
    img = _gpu_clip(asv, rgb, fwd, bwd, K, 3, middlebury=1)
    img.run_lloyd()
    labels, raw, seeds, info = orc.run_clip(rgb, fwd, bwd, K, iters=3, middlebury=1, nthreads=8)
    _, g = orc.grid_seeds(W, H, D, K, middlebury=1)
    assert img.info().s == g.s and img.info().Kp == seeds.shape[0]
    assert np.array_equal(img.raw_labels(), raw)
    assert np.array_equal(img.labels(), labels)
    img.close()
