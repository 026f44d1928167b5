"""Golden fixtures from the reference's own shaders (tests/golden/make_golden.py):
the CPU restatement and the CUDA path must reproduce them exactly."""
import os

import numpy as np
import pytest

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(G, name))


def test_oracle_rgb2lab(orc):
    f = load("rgb2lab_sample.npz")
    assert np.array_equal(orc.rgb2lab(f["rgb"])[:, :3].astype(np.float32), f["lab"])


def test_oracle_derivative(orc):
    f = load("derivative.npz")
    assert np.array_equal(orc.gradient_half(f["rgb"]), f["gradient"].astype(np.float16).view(np.uint16))


@pytest.mark.parametrize("step", [1, 3, 7])
def test_oracle_flood(orc, step):
    f = load(f"flood_step{step}.npz")
    lab4 = orc.rgb2lab(f["rgb"])
    got = orc.jfa_pass(f["labels"], lab4, f["seeds"], int(f["step"]), np.float32(f["ratio"]))
    assert np.array_equal(got, f["out"])


def test_oracle_aver_exception(orc):
    f = load("aver_exception.npz")
    rgb = f["rgb"]
    D, H, W, _ = rgb.shape
    kp = f["pos"].shape[0]
    pos, col = orc.finalize((D, H, W), f["sums"], orc.rgb2lab(rgb), np.zeros((kp, 3), np.float32),
                            np.zeros((kp, 3), np.float32))
    assert np.array_equal(pos, f["pos"][:, :3])
    assert np.array_equal(col, f["col"])


@pytest.mark.gpu
def test_cuda_rgb2lab(asv):
    f = load("rgb2lab_sample.npz")
    rgb = f["rgb"].reshape(2, 64, 128, 3)
    img = asv.Image(lloyd_iters=1)
    img.init_gpu(rgb, 100)
    img.RGB2LAB()
    assert np.array_equal(img.lab()[..., :3].reshape(-1, 3).astype(np.float32), f["lab"])


@pytest.mark.gpu
@pytest.mark.parametrize("step", [1, 3, 7])
def test_cuda_flood(asv, step):
    f = load(f"flood_step{step}.npz")
    rgb = f["rgb"]
    D, H, W, _ = rgb.shape
    img = asv.Image(lloyd_iters=1)
    img.init_gpu(rgb, 20)
    img.RGB2LAB()
    assert img.info().Kp == f["seeds"].shape[0]
    img.set_seeds(f["seeds"])
    got = img.jfa_pass(f["labels"], int(f["step"]), float(np.float32(f["ratio"])))
    assert np.array_equal(got, f["out"])


def _connectivity_cases():
    f = load("connectivity.npz")
    i = 0
    while f"labels_{i}" in f:
        yield f[f"labels_{i}"], int(f[f"supsz_{i}"]), f[f"out_{i}"], int(f[f"n_{i}"])
        i += 1


def test_oracle_connectivity(orc):
    for labels, supsz, out, n in _connectivity_cases():
        got, m = orc.enforce_connectivity(labels, supsz)
        assert m == n and np.array_equal(got, out)


@pytest.mark.gpu
def test_cuda_connectivity(asv):
    with asv.Image(lloyd_iters=1) as img:
        for labels, supsz, out, n in _connectivity_cases():
            got, m = img.enforce_connectivity_labels(labels, supsz)
            assert m == n and np.array_equal(got, out), labels.shape


def test_oracle_seed_grid():
    """the restatement's seed grid against Image::init_seeds' own output"""
    from oracle import oracle
    f = load("seed_grid.npz")
    n = 0
    for key in f.files:
        if not key.startswith("shape_"):
            continue
        W, H, D, K, mb = (int(v) for v in f[key])
        tag = key[len("shape_"):]
        s4, g = oracle.grid_seeds(W, H, D, K, middlebury=mb)
        assert (g.s, g.dNum, g.hNum, g.wNum, g.Kp) == tuple(int(v) for v in f["grid_" + tag])
        assert np.array_equal(s4, f["seeds_" + tag])
        n += 1
    assert n >= 20


@pytest.mark.parametrize("fixture", ["sequence_label.npz", "few_dead.npz"])
def test_oracle_sequence_label(orc, fixture):
    """the restatement's post-processing against the reference's own output:
    Image::sequence_label (> 3 dead seeds, the -1 fill) and label_replace.gs
    with its host loop (1-3 dead seeds)"""
    f = load(fixture)
    n = 0
    for key in f.files:
        if not key.startswith("labels_"):
            continue
        i = key[len("labels_"):]
        labels, counts, kp = f[key], f["counts_" + i], int(f["kp_" + i])
        sums = np.zeros((kp + 1, 7), np.int64)
        sums[:, 3] = counts
        got, _ = orc.postprocess(labels, sums, kp)
        assert np.array_equal(got, f["out_" + i]), i
        n += 1
    assert n >= 10


def test_oracle_density_placement(asv):
    """the restatement's seed redistribution and cell-id grid against the host
    parts of Image::initialization's own output"""
    import ctypes
    from oracle import oracle
    from oracle.oracle import GridInfo
    f = load("density_placement.npz")
    lib = oracle.load()
    V = ctypes.c_void_p
    lib.orc_grid_cell_tables.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, V,
                                         ctypes.POINTER(GridInfo), V, V, V]
    n = 0
    while f"case_{n}" in f:
        W, H, D, K, mb = (int(v) for v in f[f"case_{n}"])
        rgb, _, _ = asv.synth_clip(W, H, D, n_ellipses=5, noise_sigma=4.0, seed=W * D + K)
        s4, g = oracle.grid_seeds(W, H, D, K, middlebury=mb)
        adj, _ = oracle.density_adjust(rgb, s4, g)
        assert np.array_equal(adj, f[f"seeds_{n}"]), (W, H, D, K, mb)
        xc, yc, zc = np.empty(W, np.int32), np.empty(H, np.int32), np.empty(D, np.int32)
        s4c = np.ascontiguousarray(s4)
        lib.orc_grid_cell_tables(W, H, D, s4c.ctypes.data_as(V), ctypes.byref(g), xc.ctypes.data_as(V),
                                 yc.ctypes.data_as(V), zc.ctypes.data_as(V))
        cell = (zc[:, None, None] * g.hNum + yc[None, :, None]) * g.wNum + xc[None, None, :]
        assert np.array_equal(f[f"grid_{n}"], cell.astype(np.float32))
        n += 1
    assert n >= 5



def test_oracle_flood_ladder(orc):
    """the restatement's JFA ladder and ratio against Image::flood's own uniforms"""
    f = load("flood_ladder.npz")
    assert f["s"].size >= 100
    for i, s in enumerate(f["s"]):
        r = np.float32(orc.ratio(int(s), 8.0))
        assert r == f["ratio"][i]
        steps, rmul = orc.ladder(int(s))
        n = int(f["count"][i])
        assert len(steps) == n, s
        assert np.array_equal(np.float32(steps), f["steps"][i, :n]), s
        assert np.array_equal(np.float32(rmul) * r, f["ratios"][i, :n]), s


def test_labels_txt(asv, tmp_path):
    """asv_write_labels_txt against the bytes Image::print_sv_txt wrote"""
    f = load("labels_txt.npz")
    n = 0
    while f"labels_{n}" in f:
        p = str(tmp_path / f"k{n}.txt")
        asv.write_labels_txt(p, f[f"labels_{n}"])
        assert open(p, "rb").read() == f[f"txt_{n}"].tobytes()
        n += 1
    assert n == 4


def test_oracle_stream_scheduler(orc):
    """the oracle's block partition and kept seeds against the reference's
    compiled streaming Render.cpp"""
    import ctypes
    f = load("stream_scheduler.npz")
    lib = orc.load()
    V = ctypes.c_void_p
    lib.orc_stream_blocks.argtypes = [ctypes.c_int, ctypes.c_int, V, ctypes.c_int]
    lib.orc_stream_keep.argtypes = [V, ctypes.c_int, ctypes.c_int, V]
    for i, D in enumerate(f["D"]):
        iv = np.zeros(512, np.int32)
        n = lib.orc_stream_blocks(int(D), 30, iv.ctypes.data_as(V), 512)
        assert n == f["blocks"][i] and np.array_equal(iv[:2 * n], f["intervals"][i, :2 * n]), D
    info = np.ascontiguousarray(f["info"])
    kept = np.zeros_like(info)
    k = lib.orc_stream_keep(info.ctypes.data_as(V), info.shape[0], 30, kept.ctypes.data_as(V))
    assert k == f["kept"].shape[0] and np.array_equal(kept[:k], f["kept"])
