"""NumPy restatement of the supervoxel quality measures (asv_evaluate).

TEST INFRASTRUCTURE ONLY: the oracle for anisotropic_supervoxel_gb300's
asv_evaluate.  The definitions (LIBSVX's 3D undersegmentation error, 3D
segmentation accuracy, 3D boundary recall and mean duration, Xu & Corso,
CVPR 2012; LIBSVX's own code is not available, so parity with it is
unpinned) are the ones stated in include/asv.h; the sums run in the same
order as the library's host code, so the results are equal as doubles.
"""
import numpy as np


def _boundary(a):
    b = np.zeros(a.shape, bool)
    for ax in range(3):
        d = np.diff(a, axis=ax) != 0
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, -1)
        hi[ax] = slice(1, None)
        b[tuple(lo)] |= d
        b[tuple(hi)] |= d
    return b


def evaluate(labels, truth):
    labels = np.asarray(labels, np.int64)
    truth = np.asarray(truth, np.int64)
    rows, NG = int(labels.max()) + 2, int(truth.max()) + 1
    c = np.bincount(((labels + 1) * NG + truth).ravel(), minlength=rows * NG).reshape(rows, NG)
    ssz, gsz = c.sum(1), c.sum(0)
    arg = np.where(c.max(1) > 0, c.argmax(1), -1)          # ties: the smaller truth id
    under = np.zeros(NG, np.int64)
    cover = np.zeros(NG, np.int64)
    for s in range(rows):
        for g in np.nonzero(c[s])[0]:
            under[g] += ssz[s]
        if arg[s] >= 0:
            cover[arg[s]] += c[s, arg[s]]
    ue = sa = 0.0
    ng = 0
    for g in range(NG):
        if gsz[g]:
            ue += float(under[g] - gsz[g]) / float(gsz[g])
            sa += float(cover[g]) / float(gsz[g])
            ng += 1
    D = labels.shape[0]
    dur, nlab = 0.0, 0
    z = np.arange(D)[:, None, None] * np.ones(labels.shape, np.int64)
    for s in range(1, rows):
        if ssz[s]:
            zs = z[labels == s - 1]
            dur += float(zs.max() - zs.min() + 1)
            nlab += 1
    sb = _boundary(labels)
    gb = _boundary(truth)
    near = np.zeros(sb.shape, bool)
    Dd, H, W = sb.shape
    pad = np.pad(sb, 1)
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                near |= pad[dz:dz + Dd, dy:dy + H, dx:dx + W]
    tb, rec = int(gb.sum()), int((gb & near).sum())
    nsv = int((ssz > 0).sum())
    return {"undersegmentation": ue / ng if ng else 0.0, "segmentation_accuracy": sa / ng if ng else 0.0,
            "boundary_recall": rec / tb if tb else 1.0, "mean_duration": dur / nlab if nlab else 0.0,
            "supervoxels": nsv, "truth_segments": ng, "truth_boundary": tb, "recalled": rec}
