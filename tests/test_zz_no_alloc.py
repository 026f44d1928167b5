"""asv_check_dead_seeds_noalloc: the post-processing entry point that does
no device allocation, for hosts that own all device memory (their own pool)
or cannot afford cudaMalloc's device synchronization mid-pipeline.

Each case is checked against the oracle's post-processing (orc.postprocess,
the restatement of check_dead_seeds / sequence_label pinned to the
reference's own code) and against the context path
(asv_check_dead_seeds_host), which allocates its scratch with the context;
all of them compute integer labels, so the tolerance is exact equality.  Each
case calls the entry point twice in a row, because its scratch persists
between calls.  The shapes cover a volume of whole 2048-voxel chunks, one
with a partial last chunk, and one of more than 1024 chunks (the chunk scan
carries across its 1024-thread rounds), with Kp above 1024 and dead seeds on
both sides of the 1024-seed rounds of the seed scan.  This file is collected
last so that a run stopping at the first failure has run every other test;
it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

from conftest import small_clip

pytestmark = pytest.mark.gpu


def _cases(raw, kp, rng):
    out = [raw]
    a = raw.copy()
    a[rng.random(a.shape) < 0.03] = -1
    out.append(a)                                              # -1 fill only
    b = raw.copy()
    b[np.isin(b, [2, kp - 1])] = 0
    b.ravel()[0] = -1
    out.append(b)                                              # 2 dead seeds + -1 at voxel 0
    c = raw.copy()
    c[np.isin(c, [1, 3, 5, 7, 9])] = 4
    c[rng.random(c.shape) < 0.01] = -1
    out.append(c)                                              # 5 dead seeds: raster remap
    return out


def _oracle(orc, raw, kp):
    counts = np.zeros((kp + 1, 7), np.int64)
    counts[:, 3] = np.bincount(np.where(raw < 0, kp, raw).ravel(), minlength=kp + 1)
    want, _ = orc.postprocess(raw, counts, kp)
    return want


def _noalloc(lib, torch, raw, kp, twice=True):
    D, H, W = raw.shape
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    d_raw = torch.from_numpy(np.ascontiguousarray(raw)).to(dev)
    d_out = torch.empty_like(d_raw)
    outs = []
    for _ in range(2 if twice else 1):
        d_out.fill_(-7)
        st = lib.asv_check_dead_seeds_noalloc(d_raw.data_ptr(), d_out.data_ptr(), W, H, D, kp, stream)
        torch.cuda.synchronize(dev)
        assert st == 0
        outs.append(d_out.cpu().numpy())
    return outs


def test_noalloc_matches_oracle_and_context_path(asv, orc):
    torch = pytest.importorskip("torch")
    lib = asv.load()
    W, H, D, K = 64, 48, 12, 60
    rgb, fwd, bwd = small_clip(asv, W, H, D, seed=21)
    img = asv.Image(lloyd_iters=3)
    img.segment(rgb, fwd, bwd, K)
    kp = img.info().Kp
    for raw in _cases(img.raw_labels(), kp, np.random.default_rng(3)):
        want = _oracle(orc, raw, kp)
        assert np.array_equal(img.check_dead_seeds_host(raw), want)
        for got in _noalloc(lib, torch, raw, kp):
            assert np.array_equal(got, want)
    img.close()


@pytest.mark.parametrize("D,H,W,kp", [(9, 23, 37, 40), (30, 240, 320, 1500)])
def test_noalloc_ragged_and_large(asv, orc, D, H, W, kp):
    """a partial last chunk (7659 voxels); 2.3 M voxels = 1125 chunks with
    Kp = 1500: dead seeds at 3, 1023, 1024, 1025 and 1499, -1 voxels"""
    torch = pytest.importorskip("torch")
    lib = asv.load()
    rng = np.random.default_rng(D + kp)
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    nbx, nby = (W + 6) // 7, (H + 4) // 5
    base = (((zz // 3) * nby + yy // 5) * nbx + xx // 7) % kp           # blocky, every label present
    base = base.astype(np.int32)
    assert np.unique(base).size == kp
    cases = [base]
    a = base.copy()
    a[rng.random(a.shape) < 0.02] = -1
    cases.append(a)
    b = base.copy()
    b[np.isin(b, [3, 1023 % kp, 1024 % kp, 1025 % kp, kp - 1])] = 0
    b[rng.random(b.shape) < 0.01] = -1
    cases.append(b)                                                   # > 3 dead: remap
    c = base.copy()
    c[np.isin(c, [kp - 1, 1])] = 2
    cases.append(c)                                                   # 2 dead, no -1
    for raw in cases:
        want = _oracle(orc, raw, kp)
        for got in _noalloc(lib, torch, raw, kp):
            assert np.array_equal(got, want)


def test_noalloc_out_of_range_read_as_minus_one(asv, orc):
    torch = pytest.importorskip("torch")
    lib = asv.load()
    rng = np.random.default_rng(5)
    kp = 50
    raw = rng.integers(0, kp, (6, 20, 30)).astype(np.int32)
    raw[raw == 7] = 0                                                 # one dead seed
    bad = rng.random(raw.shape) < 0.02
    raw[bad] = rng.integers(kp, 1000, int(bad.sum()))
    raw.ravel()[5] = -9
    clean = np.where((raw < 0) | (raw >= kp), -1, raw).astype(np.int32)
    want = _oracle(orc, clean, kp)
    for got in _noalloc(lib, torch, raw, kp):
        assert np.array_equal(got, want)


def test_noalloc_rejects_bad_arguments(asv):
    torch = pytest.importorskip("torch")
    lib = asv.load()
    d = torch.zeros(64, dtype=torch.int32, device="cuda:0")
    e = torch.zeros(64, dtype=torch.int32, device="cuda:0")
    # 2^25 + 1 voxels, and Kp beyond the label range: refused before any GPU work
    assert lib.asv_check_dead_seeds_noalloc(d.data_ptr(), e.data_ptr(), 8193, 4096, 1, 10, None) == 1
    assert lib.asv_check_dead_seeds_noalloc(d.data_ptr(), e.data_ptr(), 4, 2, 2, 32768, None) == 1
    assert lib.asv_check_dead_seeds_noalloc(None, e.data_ptr(), 4, 2, 2, 10, None) == 1
    # in place, and overlapping by one voxel: refused
    assert lib.asv_check_dead_seeds_noalloc(d.data_ptr(), d.data_ptr(), 4, 2, 2, 10, None) == 1
    assert lib.asv_check_dead_seeds_noalloc(d.data_ptr(), d.data_ptr() + 4 * 15, 4, 2, 2, 10, None) == 1
    # adjacent but disjoint: accepted
    assert lib.asv_check_dead_seeds_noalloc(d.data_ptr(), d.data_ptr() + 4 * 16, 4, 2, 2, 10, None) == 0
    torch.cuda.synchronize()
