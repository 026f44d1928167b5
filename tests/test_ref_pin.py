"""Pins the CPU restatement to the reference's own shader code.

oracle/build_ref.py compiles the reference's GLSL files (read where they lie
in the reference tree) as C++ with a harness that supplies GL's sampling and
builtins; these tests compare the restatement with those compiled shaders.
They need the reference tree, so they skip where it is absent; the golden
fixtures under tests/golden/ carry the same answers everywhere.
"""
import ctypes

import numpy as np
import pytest

from conftest import small_clip


@pytest.fixture(scope="module")
def ref():
    from oracle import build_ref
    path = build_ref.build()
    if path is None:
        pytest.skip("reference tree not present")
    lib = ctypes.CDLL(path)
    V = ctypes.c_void_p
    lib.ref_rgb2lab.argtypes = [V, ctypes.c_long, V]
    lib.ref_derivative.argtypes = [V, ctypes.c_int, ctypes.c_int, ctypes.c_int, V]
    lib.ref_flood.argtypes = [V, V, V, V, V, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.c_float, ctypes.c_float, V]
    lib.ref_centroid_target.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                        V, V]
    lib.ref_aver_exception.argtypes = [V, V, V, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, V, V]
    return lib


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def ref_lab(ref, rgb):
    rgb = np.ascontiguousarray(rgb, np.uint8)
    out = np.zeros(rgb.shape[:-1] + (3,), np.float32)
    ref.ref_rgb2lab(P(rgb), rgb.size // 3, P(out))
    return out


def test_rgb2lab_all_2e24(ref, orc):
    v = np.arange(1 << 24, dtype=np.uint32)
    rgb = np.stack([(v >> 16) & 255, (v >> 8) & 255, v & 255], -1).astype(np.uint8)
    want = ref_lab(ref, rgb)
    assert np.array_equal(want, np.floor(want))          # the shader writes integers
    got = orc.rgb2lab(rgb)[:, :3].astype(np.float32)
    bad = np.nonzero((got != want).any(-1))[0]
    assert bad.size == 0, f"{bad.size} RGB values differ, first {bad[:8]}"


def test_derivative(ref, orc, asv):
    for rgb in (small_clip(asv, 23, 17, 6, seed=2)[0],
                np.random.default_rng(3).integers(0, 256, (5, 11, 13, 3), dtype=np.uint8)):
        D, H, W, _ = rgb.shape
        rgbf = np.ascontiguousarray(rgb.astype(np.float32) / np.float32(255.0))
        g = np.zeros((D, H, W), np.float32)
        ref.ref_derivative(P(rgbf), W, H, D, P(g))
        assert np.array_equal(orc.gradient_half(rgb), g.astype(np.float16).view(np.uint16))


def _flood_case(rng, W, H, D, k, psd=True):
    seeds = np.zeros((k, 12), np.float32)
    vox = rng.choice(W * H * D, k, replace=False)          # distinct seed voxels
    seeds[:, 0] = vox % W + 0.5
    seeds[:, 1] = (vox // W) % H + 0.5
    seeds[:, 2] = vox // (W * H) + 0.5
    seeds[:, 3:6] = rng.uniform(0, 255, (k, 3)).astype(np.float32)
    A = rng.normal(0, 0.7, (k, 3, 3)).astype(np.float32)
    M = np.einsum("kij,kil->kjl", A, A) + (np.eye(3, dtype=np.float32) * 0.2)
    seeds[:, 6:12] = M[:, [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]]
    if not psd:
        seeds[: k // 4, 6:12] *= -1.0
    return seeds


def _textures(seeds, labels, lab4):
    D, H, W = labels.shape
    k = seeds.shape[0]
    ids = np.arange(k, dtype=np.float32)
    rec = np.concatenate([seeds[:, :3], ids[:, None]], 1)
    lt = np.where(labels[..., None] >= 0, rec[np.clip(labels, 0, None)], np.float32(-1)).astype(np.float32)
    sc = np.full((D, H, W, 4), -1, np.float32)
    f3 = np.full((D, H, W, 4), -1, np.float32)
    l3 = np.full((D, H, W, 4), -1, np.float32)
    x, y, z = seeds[:, 0].astype(int), seeds[:, 1].astype(int), seeds[:, 2].astype(int)
    sc[z, y, x] = np.concatenate([seeds[:, 3:6], ids[:, None]], 1)
    f3[z, y, x] = np.concatenate([seeds[:, 6:9], ids[:, None]], 1)
    l3[z, y, x] = np.concatenate([seeds[:, 9:12], ids[:, None]], 1)
    img = np.ascontiguousarray(lab4[..., :3].astype(np.float32))
    return [np.ascontiguousarray(a) for a in (lt, sc, f3, l3)] + [img]


@pytest.mark.parametrize("step,psd", [(1, True), (2, True), (3, False), (6, True), (11, False)])
def test_flood(ref, orc, asv, step, psd):
    W, H, D, k = 29, 21, 9, 40
    rgb = small_clip(asv, W, H, D, seed=step)[0]
    lab4 = orc.rgb2lab(rgb)
    rng = np.random.default_rng(step)
    seeds = _flood_case(rng, W, H, D, k, psd)
    labels = rng.integers(-1, k, (D, H, W)).astype(np.int32)
    ratio = np.float32(0.0873)
    lt, sc, f3, l3, img = _textures(seeds, labels, lab4)
    out = np.zeros((D, H, W, 4), np.float32)
    ref.ref_flood(P(lt), P(sc), P(f3), P(l3), P(img), W, H, D, float(step), float(ratio), P(out))
    want = out[..., 3].astype(np.int32)
    got = orc.jfa_pass(labels, lab4, seeds, step, ratio)
    assert np.array_equal(got, want)


def test_centroid_slot_mapping(ref):
    for W, H in ((240, 160), (320, 240), (146, 120), (640, 480), (1280, 720)):
        for kp in (187, 936, 1947, 2000):
            for i in list(range(0, kp, 7)) + [kp - 1, -1]:
                tx, ty = ctypes.c_int(), ctypes.c_int()
                ref.ref_centroid_target(float(i), W, H, float(kp), ctypes.byref(tx), ctypes.byref(ty))
                slot = kp if i < 0 else i
                assert (tx.value, ty.value) == (slot % W, slot // W)


def test_aver_exception(ref, orc, asv):
    W, H, D, kp = 37, 13, 7, 60
    rgb = small_clip(asv, W, H, D, seed=9)[0]
    lab4 = orc.rgb2lab(rgb)
    rng = np.random.default_rng(4)
    sums = np.zeros((kp + 1, 7), np.int64)
    cnt = rng.integers(1, 400, kp + 1)
    dead = [0, 1, 5, 6, 30, kp - 1]              # includes seed 0 (reads texel W-1) and the last seed
    cnt[dead] = 0
    for i in range(kp + 1):
        c = int(cnt[i])
        if c == 0:
            continue
        xs = rng.integers(0, W, c); ys = rng.integers(0, H, c); zs = rng.integers(0, D, c)
        sums[i, :4] = [(2 * xs + 1).sum(), (2 * ys + 1).sum(), (2 * zs + 1).sum(), c]
        sums[i, 4:] = rng.integers(0, 256, (c, 3)).sum(0)
    pos0 = np.zeros((kp, 3), np.float32)
    slab0 = np.zeros((kp, 3), np.float32)
    got_pos, got_col = orc.finalize((D, H, W), sums, lab4, pos0, slab0)
    sp = np.zeros((D, H, W, 4), np.float32)
    scol = np.zeros((D, H, W, 4), np.float32)
    for i in range(kp + 1):                         # texels of slice 0 hold the sums (slot i at (i % W, i // W))
        y, x = divmod(i, W)
        sp[0, y, x] = [np.float32(sums[i, 0]) * np.float32(0.5), np.float32(sums[i, 1]) * np.float32(0.5),
                       np.float32(sums[i, 2]) * np.float32(0.5), np.float32(sums[i, 3])]
        scol[0, y, x] = [np.float32(sums[i, 4]), np.float32(sums[i, 5]), np.float32(sums[i, 6]),
                         np.float32(sums[i, 3])]
    img = np.ascontiguousarray(lab4[..., :3].astype(np.float32))
    for i in range(kp):
        p4 = np.zeros(4, np.float32)
        c3 = np.zeros(3, np.float32)
        ref.ref_aver_exception(P(sp), P(scol), P(img), W, H, D, i, P(p4), P(c3))
        assert np.array_equal(p4[:3], got_pos[i]), i
        assert np.array_equal(c3, got_col[i]), i
        assert p4[3] == i


@pytest.fixture(scope="module")
def ref_host():
    from oracle import build_ref
    path = build_ref.build_host()
    if path is None:
        pytest.skip("reference tree not present")
    lib = ctypes.CDLL(path)
    V = ctypes.c_void_p
    for f in (lib.ref_enforce_connectivity, lib.ref_label_connected3D):
        f.argtypes = [V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, V]
        f.restype = ctypes.c_int
    return lib


def connectivity_cases(rng):
    """label volumes: noisy, blocky (nearest of random centres), with -1, degenerate shapes"""
    out = []
    for (D, H, W) in ((7, 13, 17), (1, 9, 11), (5, 1, 19), (6, 12, 1), (3, 2, 2), (9, 20, 24)):
        out.append((rng.integers(-1, 4, (D, H, W)).astype(np.int32), 40))
        c = rng.integers(0, [W, H, D], (6, 3))
        zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
        dist = [(xx - cx) ** 2 + (yy - cy) ** 2 + 2 * (zz - cz) ** 2 for cx, cy, cz in c]
        blocky = np.argmin(np.stack(dist), 0).astype(np.int32)
        noisy = blocky.copy()
        flip = rng.random(blocky.shape) < 0.05
        noisy[flip] = rng.integers(-1, 6, int(flip.sum()))
        out.append((blocky, D * H * W // 6))
        out.append((noisy, D * H * W // 6))
    return out


def test_connectivity_matches_reference(ref_host, orc):
    rng = np.random.default_rng(29)
    for labels, supsz in connectivity_cases(rng):
        D, H, W = labels.shape
        for fn in (ref_host.ref_enforce_connectivity, ref_host.ref_label_connected3D):
            want = np.empty_like(labels)
            n = fn(P(labels), W, H, D, supsz, P(want))
            got, m = orc.enforce_connectivity(labels, supsz)
            assert m == n
            assert np.array_equal(got, want), (labels.shape, supsz)


def test_connectivity_on_jfa_labels(ref_host, orc, asv):
    rgb, fwd, bwd = small_clip(asv, W=48, H=36, D=10, seed=4, jitter=0.3, drift=1.0)
    _, raw, _, info = orc.run_clip(rgb, fwd, bwd, 60, iters=3, nthreads=4)
    supsz = raw.size // 60
    want = np.empty_like(raw)
    n = ref_host.ref_enforce_connectivity(P(raw), 48, 36, 10, supsz, P(want))
    got, m = orc.enforce_connectivity(raw, supsz)
    assert m == n and np.array_equal(got, want)


@pytest.fixture(scope="module")
def ref_grid(ref_host):
    V = ctypes.c_void_p
    ref_host.ref_init_seeds.argtypes = [ctypes.c_int] * 5 + [V, ctypes.c_int, V]
    ref_host.ref_init_seeds.restype = ctypes.c_int
    ref_host.ref_sequence_label.argtypes = [V, ctypes.c_long, V, ctypes.c_int, ctypes.c_int]
    return ref_host


GRID_SHAPES = [(240, 160, 30, 200), (320, 240, 85, 1000), (1280, 720, 30, 2000), (64, 48, 12, 60),
               (37, 23, 9, 25), (17, 9, 3, 2), (2, 2, 2, 1), (40, 30, 2, 30), (160, 128, 8, 30000),
               (64, 64, 64, 32767), (640, 480, 120, 2000), (50, 50, 5, 3000), (90, 50, 8, 120)]


@pytest.mark.parametrize("middlebury", [0, 1])
def test_seed_grid_matches_reference(ref_grid, orc, middlebury):
    """Image::init_seeds compiled from the reference tree against the restatement:
    the same seeds, ids, base step s and grid counts."""
    for (W, H, D, K) in GRID_SHAPES:
        g5 = np.zeros(5, np.int32)
        n = ref_grid.ref_init_seeds(W, H, D, K, middlebury, None, 0, P(g5))
        want = np.zeros((max(n, 1), 4), np.float32)
        ref_grid.ref_init_seeds(W, H, D, K, middlebury, P(want), n, P(g5))
        s4, g = orc.grid_seeds(W, H, D, K, middlebury=middlebury)
        assert (g.s, g.dNum, g.hNum, g.wNum, g.Kp) == tuple(g5), (W, H, D, K)
        assert np.array_equal(s4, want[:n]), (W, H, D, K)


def sequence_label_cases(rng):
    """label volumes with the voxel count of every label (as the centroid pass
    gives them): more than 3 labels absent (dead seeds), or all present with
    label -1 in places; some with long runs of one label"""
    out = []
    for case in range(24):
        D, H, W = int(rng.integers(1, 6)), int(rng.integers(1, 12)), int(rng.integers(2, 14))
        kp = int(rng.integers(9, 40))
        many_dead = case % 2 == 0
        if many_dead:
            used = np.sort(rng.choice(kp, kp - 4 - int(rng.integers(0, 3)), replace=False))
            labels = used[rng.integers(0, used.size, (D, H, W))].astype(np.int32)
        else:
            labels = rng.integers(0, kp, (D, H, W)).astype(np.int32)
            labels.ravel()[:kp] = np.arange(kp) if labels.size >= kp else labels.ravel()[:kp]
        if case % 3 == 0:
            labels[:, :, : W // 2] = labels[0, 0, 0]                 # runs of one label
        labels[rng.random(labels.shape) < 0.1] = -1
        counts = np.bincount(np.where(labels < 0, kp, labels).ravel(), minlength=kp + 1).astype(np.int64)
        out.append((labels, counts, kp))
    return out


def test_sequence_label_matches_reference(ref_grid, orc):
    """Image::sequence_label compiled from the reference tree against the
    restatement's post-processing: the > 3 dead-seed remap (with its
    unchanging last_label) and the raster-order fill of label -1."""
    seen = set()
    for labels, counts, kp in sequence_label_cases(np.random.default_rng(41)):
        dead = int((counts[:kp] < 1).sum())
        if dead in (1, 2, 3):
            continue                                   # that branch is a shader (label_replace.gs)
        sums = np.zeros((kp + 1, 7), np.int64)
        sums[:, 3] = counts
        got, stats = orc.postprocess(labels, sums, kp)
        want = labels.copy()
        ref_grid.ref_sequence_label(P(want), want.size, P(counts), kp, 1 if dead > 3 else 0)
        assert stats[0] == dead
        assert np.array_equal(got, want)
        seen.add("remap" if dead > 3 else "fill")
    assert seen == {"remap", "fill"}


@pytest.mark.parametrize("W,H,D,K,mb", [(64, 48, 12, 60, 0), (37, 23, 9, 25, 0), (120, 80, 15, 300, 0),
                                        (50, 50, 5, 3000, 0), (64, 48, 12, 60, 1), (240, 160, 30, 200, 0)])
def test_density_placement_matches_reference(ref_grid, orc, asv, W, H, D, K, mb):
    """The host parts of Image::initialization compiled from the reference tree
    (cell ranges, the cell-id grid, the redistribution over the density sums)
    against the restatement, given the restatement's density sums (the sums
    themselves come from derivative_t / density_grid, pinned above)."""
    from oracle.oracle import GridInfo
    V = ctypes.c_void_p
    ref_grid.ref_initialization.argtypes = [ctypes.c_int] * 5 + [V, V, V, ctypes.c_int]
    ref_grid.ref_initialization.restype = ctypes.c_int
    rgb, _, _ = asv.synth_clip(W, H, D, n_ellipses=5, noise_sigma=4.0, seed=W * D + K)
    s4, g = orc.grid_seeds(W, H, D, K, middlebury=mb)
    adj, dens = orc.density_adjust(rgb, s4, g)
    grid = np.empty((D, H, W), np.float32)
    seeds = np.zeros((g.Kp, 4), np.float32)
    dens = np.ascontiguousarray(dens, np.float32)
    n = ref_grid.ref_initialization(W, H, D, K, mb, P(dens), P(grid), P(seeds), g.Kp)
    assert n == adj.shape[0]
    assert np.array_equal(seeds[:n], adj)
    lib = orc.load()
    lib.orc_grid_cell_tables.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, V,
                                         ctypes.POINTER(GridInfo), V, V, V]
    xc, yc, zc = np.empty(W, np.int32), np.empty(H, np.int32), np.empty(D, np.int32)
    lib.orc_grid_cell_tables(W, H, D, P(np.ascontiguousarray(s4)), ctypes.byref(g), P(xc), P(yc), P(zc))
    cell = (zc[:, None, None] * g.hNum + yc[None, :, None]) * g.wNum + xc[None, None, :]
    assert np.array_equal(grid, cell.astype(np.float32))


def few_dead_cases(rng):
    """label volumes with 1 to 3 seeds absent (dead), every other seed present,
    label -1 in half of them: (labels, counts, kp, dead ids)"""
    out = []
    for case in range(18):
        D, H, W = int(rng.integers(1, 6)), int(rng.integers(1, 10)), int(rng.integers(2, 12))
        kp = int(rng.integers(6, 30))
        ndead = 1 + case % 3
        dead = np.sort(rng.choice(kp, ndead, replace=False))
        used = np.setdiff1d(np.arange(kp), dead)
        labels = used[rng.integers(0, used.size, (D, H, W))].astype(np.int32)
        labels.ravel()[:used.size] = used[: labels.size]             # every live seed present
        if case % 2:
            labels[rng.random(labels.shape) < 0.1] = -1
        counts = np.bincount(np.where(labels < 0, kp, labels).ravel(), minlength=kp + 1).astype(np.int64)
        if int((counts[:kp] < 1).sum()) == ndead:
            out.append((labels, counts, kp, dead))
    return out


def reference_few_dead(ref, ref_grid, labels, counts, kp, dead):
    """check_dead_seeds' 1-3 dead branch with the reference's own code: one
    label_replace pass per dead seed (GPU-AS/Image.cpp:1647-1672: seeds in
    order, last_seed_index counting down from K'), then sequence_label's fill
    of label -1 when -1 is present"""
    D, H, W = labels.shape
    vol = np.zeros(labels.shape + (4,), np.float32)
    vol[..., 3] = labels
    last = kp
    for d in dead:
        last -= 1
        nxt = np.empty_like(vol)
        ref.ref_label_replace(P(vol), W, H, D, int(d), last, P(nxt))
        vol = nxt
    want = vol[..., 3].astype(np.int32)
    if counts[kp] > 0:
        ref_grid.ref_sequence_label(P(want), want.size, P(counts), kp, 0)
    return want


def test_few_dead_seeds_match_reference(ref, ref_grid, orc):
    """1 to 3 dead seeds: label_replace.gs compiled from the reference tree and
    its host loop, against the restatement's post-processing."""
    V = ctypes.c_void_p
    ref.ref_label_replace.argtypes = [V] + [ctypes.c_int] * 5 + [V]
    seen = set()
    for labels, counts, kp, dead in few_dead_cases(np.random.default_rng(47)):
        sums = np.zeros((kp + 1, 7), np.int64)
        sums[:, 3] = counts
        got, stats = orc.postprocess(labels, sums, kp)
        want = reference_few_dead(ref, ref_grid, labels, counts, kp, dead)
        assert stats[0] == len(dead)
        assert np.array_equal(got, want)
        seen.add(len(dead))
    assert seen == {1, 2, 3}


@pytest.mark.parametrize("W,H,D,K", [(48, 40, 30, 60), (64, 48, 30, 150), (37, 23, 20, 25), (1280, 720, 30, 2000)])
def test_stream_window_placement_matches_reference(ref_grid, orc, asv, W, H, D, K):
    """The streaming program's per-window grid (initialization_grid) and density
    placement (the host parts of initialization_adjust), compiled from the
    reference tree, against the restatement (the same grid and placement
    functions serve the windows)."""
    V = ctypes.c_void_p
    ref_grid.ref_stream_initialization.argtypes = [ctypes.c_int] * 4 + [V, V, V, ctypes.c_int, V]
    ref_grid.ref_stream_initialization.restype = ctypes.c_int
    s4, g = orc.grid_seeds(W, H, D, K)
    g5 = np.zeros(5, np.int32)
    grid_only = np.zeros((g.Kp, 4), np.float32)
    n = ref_grid.ref_stream_initialization(W, H, D, K, None, None, P(grid_only), g.Kp, P(g5))
    assert (g.s, g.dNum, g.hNum, g.wNum, g.Kp) == tuple(g5)
    assert np.array_equal(grid_only[:n], s4)
    if W * H * D > 4_000_000:
        return                                        # the grid only at 720p (the placement needs a clip)
    rgb, _, _ = asv.synth_clip(W, H, D, n_ellipses=5, noise_sigma=4.0, drift_amp=2.0, seed=W + D + K)
    adj, dens = orc.density_adjust(rgb, s4, g)
    dens = np.ascontiguousarray(dens, np.float32)
    grid = np.empty((D, H, W), np.float32)
    seeds = np.zeros((g.Kp, 4), np.float32)
    n = ref_grid.ref_stream_initialization(W, H, D, K, P(dens), P(grid), P(seeds), g.Kp, P(g5))
    assert n == adj.shape[0] and np.array_equal(seeds[:n], adj)


LADDER_S = list(range(1, 130)) + [150, 200, 255, 256, 257, 400, 511, 512, 1000]


def reference_ladder(lib, s):
    """the (step, ratio) uniforms of every flood pass of one Lloyd iteration,
    and the ratio, from Image::init_variables and Image::flood compiled whole"""
    V = ctypes.c_void_p
    lib.ref_flood_ladder.argtypes = [ctypes.c_int, V, V, ctypes.c_int, V]
    lib.ref_flood_ladder.restype = ctypes.c_int
    steps = np.zeros(64, np.float32)
    ratios = np.zeros(64, np.float32)
    r = np.zeros(1, np.float32)
    n = lib.ref_flood_ladder(s, P(steps), P(ratios), 64, P(r))
    assert 0 < n <= 64
    return steps[:n], ratios[:n], r[0]


def test_flood_ladder_matches_reference(ref_host, orc):
    """JFA pass ladder (1, floor(s/2) halving, then 2, 1) and the per-pass ratio
    uniform, against the reference's own Image::flood for every base step s"""
    for s in LADDER_S:
        steps, ratios, r = reference_ladder(ref_host, s)
        want_r = orc.ratio(s, 8.0)
        assert np.float32(want_r) == r, s
        got_steps, rmul = orc.ladder(s)
        assert np.array_equal(np.float32(got_steps), steps), (s, got_steps, steps)
        assert np.array_equal(np.float32(rmul) * np.float32(want_r), ratios), s


def test_labels_txt_matches_reference(ref_host, asv, tmp_path):
    """asv_write_labels_txt against Image::print_sv_txt compiled from the
    reference tree (GPU-AS/Image.cpp:1780-1806): byte-identical files for
    random volumes with -1, 1- to 5-digit labels and degenerate shapes."""
    ref_host.ref_print_sv_txt.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_char_p]
    rng = np.random.default_rng(31)
    for k, (D, H, W, hi) in enumerate([(3, 5, 7, 20), (2, 4, 6, 99999), (1, 1, 1, 5), (4, 9, 3, 12000),
                                       (2, 1, 13, 1500)]):
        lab = rng.integers(-1, hi, (D, H, W)).astype(np.int32)
        lab.ravel()[0] = -1
        stem = str(tmp_path / f"ref{k}")
        ref_host.ref_print_sv_txt(P(lab), W, H, D, stem.encode())
        ours = str(tmp_path / f"ours{k}.txt")
        asv.write_labels_txt(ours, lab)
        assert open(ours, "rb").read() == open(stem + ".txt", "rb").read()


def test_stream_scheduler_matches_reference(ref_host, orc):
    """The streaming program's block partition (streamGPU-AS/Render.cpp:
    199-241) and post_and_next's kept seeds (:519-540), both compiled from the
    reference tree, against the restatement the streaming oracle runs."""
    lib = orc.load()
    V = ctypes.c_void_p
    ref_host.ref_stream_blocks.argtypes = [ctypes.c_int, V, ctypes.c_int]
    ref_host.ref_stream_keep.argtypes = [V, ctypes.c_int, ctypes.c_int, V]
    lib.orc_stream_blocks.argtypes = [ctypes.c_int, ctypes.c_int, V, ctypes.c_int]
    lib.orc_stream_keep.argtypes = [V, ctypes.c_int, ctypes.c_int, V]
    for D in list(range(2, 400)) + [899, 900, 901, 1777]:
        a, b = np.zeros(512, np.int32), np.zeros(512, np.int32)
        na = ref_host.ref_stream_blocks(D, P(a), 512)
        nb = lib.orc_stream_blocks(D, 30, P(b), 512)
        assert na == nb and np.array_equal(a[:2 * na], b[:2 * nb]), D
    rng = np.random.default_rng(37)
    for bs in (30, 42, 12):
        for n in (0, 1, 7, 500, 3000):
            info = np.zeros((max(n, 1), 4), np.float32)
            info[:, 0] = rng.integers(0, 1280, info.shape[0]) + 0.5
            info[:, 1] = rng.integers(0, 720, info.shape[0]) + 0.5
            info[:, 2] = rng.integers(0, bs, info.shape[0]) + 0.5
            info[::5, 2] = bs - bs // 3 + np.float32(0.0)             # exactly on the threshold
            info[:, 3] = np.arange(info.shape[0])
            ka, kb = np.zeros((max(n, 1), 4), np.float32), np.zeros((max(n, 1), 4), np.float32)
            ma = ref_host.ref_stream_keep(P(info), n, bs, P(ka))
            mb = lib.orc_stream_keep(P(info), n, bs, P(kb))
            assert ma == mb and np.array_equal(ka[:ma], kb[:mb]), (bs, n)
