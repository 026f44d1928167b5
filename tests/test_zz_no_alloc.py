"""asv_check_dead_seeds_noalloc: the post-processing entry point that does
no device allocation, for hosts that own all device memory (their own pool)
or cannot afford cudaMalloc's device synchronization mid-pipeline.

It is checked against the context path (asv_check_dead_seeds_host), which
allocates its scratch with the context; both compute integer labels, so the
tolerance is exact equality.  Each case calls the entry point twice in a row,
because its scratch persists between calls.  This file is collected last so
that a run stopping at the first failure has run every other test; it also
passes on its own in a fresh process.
"""
import numpy as np
import pytest

from conftest import small_clip

pytestmark = pytest.mark.gpu


def _cases(raw, kp):
    rng = np.random.default_rng(3)
    out = [raw]
    a = raw.copy()
    a[rng.random(a.shape) < 0.03] = -1
    out.append(a)                                              # -1 fill only
    b = raw.copy()
    b[np.isin(b, [2, kp - 1])] = 0
    b[0, 0, 0] = -1
    out.append(b)                                              # 2 dead seeds + -1 at voxel 0
    c = raw.copy()
    c[np.isin(c, [1, 3, 5, 7, 9])] = 4
    c[rng.random(c.shape) < 0.01] = -1
    out.append(c)                                              # 5 dead seeds: raster remap
    return out


def test_noalloc_matches_context_path(asv):
    torch = pytest.importorskip("torch")
    lib = asv.load()
    W, H, D, K = 64, 48, 12, 60
    rgb, fwd, bwd = small_clip(asv, W, H, D, seed=21)
    img = asv.Image(lloyd_iters=3)
    img.segment(rgb, fwd, bwd, K)
    kp = img.info().Kp
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for raw in _cases(img.raw_labels(), kp):
        want = img.check_dead_seeds_host(raw)
        d_raw = torch.from_numpy(np.ascontiguousarray(raw)).to(dev)
        d_out = torch.empty_like(d_raw)
        for _ in range(2):
            d_out.fill_(-7)
            st = lib.asv_check_dead_seeds_noalloc(d_raw.data_ptr(), d_out.data_ptr(), W, H, D, kp,
                                                  stream)
            torch.cuda.synchronize(dev)
            assert st == 0
            assert np.array_equal(d_out.cpu().numpy(), want)
    img.close()


def test_noalloc_rejects_oversize(asv):
    torch = pytest.importorskip("torch")
    lib = asv.load()
    d = torch.zeros(16, dtype=torch.int32, device="cuda:0")
    # 2^25 + 1 voxels, and Kp beyond the label range: refused before any GPU work
    assert lib.asv_check_dead_seeds_noalloc(d.data_ptr(), d.data_ptr(), 8193, 4096, 1, 10, None) == 1
    assert lib.asv_check_dead_seeds_noalloc(d.data_ptr(), d.data_ptr(), 4, 2, 2, 32768, None) == 1
    assert lib.asv_check_dead_seeds_noalloc(None, d.data_ptr(), 4, 2, 2, 10, None) == 1
