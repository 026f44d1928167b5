"""NumPy restatement of the device optical flow (asv_compute_flow).

TEST INFRASTRUCTURE ONLY: the oracle for anisotropic_supervoxel_gb300's
csrc/asv_flow.cu, never called by the library.  Every step uses the same
float32 operations in the same order as the CUDA kernels (built with
-fmad=false), so the two agree bit for bit: grey conversion, the binomial
pyramid, the polynomial expansion (Farneback 2003) with a 5x5 Gaussian
window (sigma 1.1), per-iteration matrices from the bilinearly sampled
destination expansion, 13x13 box sums, the 2x2 solve, and the bilinear
upsampling between levels.

The reference (GPU-AS/Image.cpp:643-686) calls OpenCV's CUDA Farneback, which
is not available here: this restates the method, not OpenCV's code, so parity
with the reference's flow is unpinned.
"""
import numpy as np

N = 2
BOX = 6
MAX_LEVELS = 5
F = np.float32


def consts():
    """(g[3][5] float32, ginv[5][6] float32) as the library computes them."""
    sigma = 1.1
    u = np.arange(-N, N + 1)
    g = np.exp(-(u * u).astype(np.float64) / (2.0 * sigma * sigma))
    gt = np.stack([g, u * g, u * u * g]).astype(np.float32)
    G = np.zeros((6, 12))
    for v in range(-N, N + 1):
        for uu in range(-N, N + 1):
            w = g[uu + N] * g[v + N]
            B = np.array([1.0, uu, v, uu * uu, v * v, uu * v], np.float64)
            for i in range(6):
                for j in range(6):
                    G[i, j] += w * B[i] * B[j]
    for i in range(6):
        G[i, 6 + i] = 1.0
    for c in range(6):
        piv = c
        for r in range(c + 1, 6):
            if abs(G[r, c]) > abs(G[piv, c]):
                piv = r
        G[[c, piv]] = G[[piv, c]]
        d = G[c, c]
        for j in range(12):
            G[c, j] /= d
        for r in range(6):
            if r != c:
                f = G[r, c]
                for j in range(12):
                    G[r, j] -= f * G[c, j]
    return gt, G[1:6, 6:12].astype(np.float32)


def levels(W, H):
    out, w, h = [], W, H
    while len(out) < MAX_LEVELS:
        out.append((w, h))
        nw, nh = (w + 1) // 2, (h + 1) // 2
        if nw < 16 or nh < 16:
            break
        w, h = nw, nh
    return out


def gray(rgb):
    r = rgb.astype(np.int64)
    return ((r[..., 0] * 4899 + r[..., 1] * 9617 + r[..., 2] * 1868 + 8192) >> 14).astype(F)


def down(img, Wo, Ho):
    D, Hi, Wi = img.shape
    w = F([1, 4, 6, 4, 1])
    x = np.arange(Wo)
    y = np.arange(Ho)
    acc = np.zeros((D, Ho, Wo), F)
    for j in range(-2, 3):
        yy = np.clip(2 * y + j, 0, Hi - 1)
        row = np.zeros((D, Ho, Wo), F)
        for i in range(-2, 3):
            xx = np.clip(2 * x + i, 0, Wi - 1)
            row = (row + w[i + 2] * img[:, yy][:, :, xx]).astype(F)
        acc = (acc + w[j + 2] * row).astype(F)
    return (acc * F(1.0 / 256.0)).astype(F)


def expand(img, gt, gi):
    """polynomial expansion planes (b1, b2, a11, a22, a12)"""
    D, H, W = img.shape
    x = np.arange(W)
    s = [np.zeros(img.shape, F) for _ in range(3)]
    for u in range(-N, N + 1):
        f = img[:, :, np.clip(x + u, 0, W - 1)]
        for p in range(3):
            s[p] = (s[p] + gt[p][u + N] * f).astype(F)
    y = np.arange(H)
    m = [np.zeros(img.shape, F) for _ in range(6)]
    for v in range(-N, N + 1):
        yy = np.clip(y + v, 0, H - 1)
        h0, h1, h2 = s[0][:, yy], s[1][:, yy], s[2][:, yy]
        g, vg, vvg = gt[0][v + N], gt[1][v + N], gt[2][v + N]
        m[0] = (m[0] + g * h0).astype(F)
        m[1] = (m[1] + g * h1).astype(F)
        m[2] = (m[2] + vg * h0).astype(F)
        m[3] = (m[3] + g * h2).astype(F)
        m[4] = (m[4] + vvg * h0).astype(F)
        m[5] = (m[5] + vg * h1).astype(F)
    out = []
    for k in range(5):
        r = np.zeros(img.shape, F)
        for e in range(6):
            r = (r + gi[k][e] * m[e]).astype(F)
        out.append((F(0.5) * r).astype(F) if k == 4 else r)
    return out


def pairs(D):
    return [(z, z + 1) for z in range(D - 1)] + [(z, z - 1) for z in range(1, D)]


def update(poly, flow, W, H, D):
    P = len(pairs(D))
    M = [np.zeros((P, H, W), F) for _ in range(5)]
    yy, xx = np.mgrid[0:H, 0:W]
    for p, (src, dst) in enumerate(pairs(D)):
        dx, dy = flow[0][p], flow[1][p]
        qx = (xx.astype(F) + dx).astype(F)
        qy = (yy.astype(F) + dy).astype(F)
        ok = (qx >= 0) & (qy >= 0) & (qx <= F(W - 1)) & (qy <= F(H - 1))
        x0 = np.minimum(np.where(ok, qx, 0).astype(np.int64), max(W - 2, 0))
        y0 = np.minimum(np.where(ok, qy, 0).astype(np.int64), max(H - 2, 0))
        x1 = np.minimum(x0 + 1, W - 1)
        y1 = np.minimum(y0 + 1, H - 1)
        fx = (qx - x0.astype(F)).astype(F)
        fy = (qy - y0.astype(F)).astype(F)
        one = F(1)
        w00 = ((one - fx) * (one - fy)).astype(F)
        w01 = (fx * (one - fy)).astype(F)
        w10 = ((one - fx) * fy).astype(F)
        w11 = (fx * fy).astype(F)
        q = []
        for k in range(5):
            Pd = poly[k][dst]
            v = (w00 * Pd[y0, x0]).astype(F)
            v = (v + (w01 * Pd[y0, x1]).astype(F)).astype(F)
            v = (v + (w10 * Pd[y1, x0]).astype(F)).astype(F)
            v = (v + (w11 * Pd[y1, x1]).astype(F)).astype(F)
            q.append(v)
        a11 = (F(0.5) * (poly[2][src] + q[2])).astype(F)
        a22 = (F(0.5) * (poly[3][src] + q[3])).astype(F)
        a12 = (F(0.5) * (poly[4][src] + q[4])).astype(F)
        db1 = (F(-0.5) * (q[0] - poly[0][src])).astype(F)
        db1 = (db1 + (a11 * dx).astype(F)).astype(F)
        db1 = (db1 + (a12 * dy).astype(F)).astype(F)
        db2 = (F(-0.5) * (q[1] - poly[1][src])).astype(F)
        db2 = (db2 + (a12 * dx).astype(F)).astype(F)
        db2 = (db2 + (a22 * dy).astype(F)).astype(F)
        o = [((a11 * a11).astype(F) + (a12 * a12).astype(F)).astype(F),
             ((a11 * a12).astype(F) + (a12 * a22).astype(F)).astype(F),
             ((a12 * a12).astype(F) + (a22 * a22).astype(F)).astype(F),
             ((a11 * db1).astype(F) + (a12 * db2).astype(F)).astype(F),
             ((a12 * db1).astype(F) + (a22 * db2).astype(F)).astype(F)]
        for k in range(5):
            M[k][p] = np.where(ok, o[k], F(0))
    return M


def box(a, axis):
    n = a.shape[axis]
    s = np.zeros(a.shape, F)
    idx = np.arange(n)
    for o in range(-BOX, BOX + 1):
        j = idx + o
        valid = (j >= 0) & (j < n)
        t = np.take(a, np.clip(j, 0, n - 1), axis=axis)
        shape = [1] * a.ndim
        shape[axis] = n
        s = (s + np.where(valid.reshape(shape), t, F(0))).astype(F)
    return s


def solve(M):
    g11, g12, g22, h1, h2 = M
    det = ((g11 * g22).astype(F) - (g12 * g12).astype(F)).astype(F)
    idet = (F(1) / (det + F(1e-3))).astype(F)
    fx = (((g22 * h1).astype(F) - (g12 * h2).astype(F)).astype(F) * idet).astype(F)
    fy = (((g11 * h2).astype(F) - (g12 * h1).astype(F)).astype(F) * idet).astype(F)
    return [fx, fy]


def upsample(flow, Wc, Hc, W, H):
    sx, sy = F(Wc) / F(W), F(Hc) / F(H)
    yy, xx = np.mgrid[0:H, 0:W]
    cx = np.minimum(np.maximum(((xx.astype(F) + F(0.5)) * sx - F(0.5)).astype(F), F(0)), F(Wc - 1))
    cy = np.minimum(np.maximum(((yy.astype(F) + F(0.5)) * sy - F(0.5)).astype(F), F(0)), F(Hc - 1))
    x0, y0 = cx.astype(np.int64), cy.astype(np.int64)
    x1, y1 = np.minimum(x0 + 1, Wc - 1), np.minimum(y0 + 1, Hc - 1)
    fx, fy = (cx - x0.astype(F)).astype(F), (cy - y0.astype(F)).astype(F)
    one = F(1)
    out = []
    for c, s in ((0, sx), (1, sy)):
        Fc = flow[c]
        v = (((one - fx) * (one - fy)).astype(F) * Fc[:, y0, x0]).astype(F)
        v = (v + ((fx * (one - fy)).astype(F) * Fc[:, y0, x1]).astype(F)).astype(F)
        v = (v + (((one - fx) * fy).astype(F) * Fc[:, y1, x0]).astype(F)).astype(F)
        v = (v + ((fx * fy).astype(F) * Fc[:, y1, x1]).astype(F)).astype(F)
        out.append((v / s).astype(F))
    return out


def compute_flow(rgb, iters=10):
    """fwd, bwd [D,H,W,2] float32 of an RGB8 clip [D,H,W,3] (texture orientation)"""
    D, H, W, _ = rgb.shape
    gt, gi = consts()
    lv = levels(W, H)
    imgs = [gray(rgb)]
    for (w, h) in lv[1:]:
        imgs.append(down(imgs[-1], w, h))
    polys = [expand(im, gt, gi) for im in imgs]
    P = len(pairs(D))
    flow = None
    for k in range(len(lv) - 1, -1, -1):
        w, h = lv[k]
        if flow is None:
            flow = [np.zeros((P, h, w), F), np.zeros((P, h, w), F)]
        else:
            flow = upsample(flow, lv[k + 1][0], lv[k + 1][1], w, h)
        for _ in range(iters):
            M = update(polys[k], flow, w, h, D)
            M = [box(box(m, 2), 1) for m in M]
            flow = solve(M)
    fwd = np.zeros((D, H, W, 2), F)
    bwd = np.zeros((D, H, W, 2), F)
    for p, (src, dst) in enumerate(pairs(D)):
        tgt = fwd if dst == src + 1 else bwd
        tgt[src, :, :, 0] = flow[0][p]
        tgt[src, :, :, 1] = flow[1][p]
    return fwd, bwd
