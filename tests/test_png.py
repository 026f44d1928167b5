"""PNG frame input/output (csrc/asv_png.cpp) against an independent codec.

The independent codec here is Python's own zlib (a different DEFLATE implementation) plus a
NumPy restatement of the PNG filters and Adam7 passes: test images are
encoded here with every zlib strategy (stored, fixed, dynamic Huffman, RLE,
Huffman-only), every colour type and bit depth, random row filters and
interlacing, then decoded by the library; the library's own PNG output is
decoded here.  Host code only: no GPU.
"""
import os
import struct
import zlib

import numpy as np
import pytest

import anisotropic_supervoxel_gb300 as asv

SIG = b"\x89PNG\r\n\x1a\n"
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
COMBOS = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8),
          (4, 8), (4, 16), (6, 8), (6, 16)]


def _chunk(kind, data):
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xffffffff)


def _pack_row(samples, depth):
    """one scanline's samples (1-D, channel-interleaved) to bytes"""
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    per = 8 // depth
    n = len(samples)
    out = bytearray((n * depth + 7) // 8)
    for i, v in enumerate(samples):
        out[i // per] |= int(v) << (8 - depth * (i % per + 1))
    return bytes(out)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter(row, prev, f, bpp):
    out = bytearray(len(row))
    for i in range(len(row)):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i] if prev is not None else 0
        c = prev[i - bpp] if (prev is not None and i >= bpp) else 0
        pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][f]
        out[i] = (row[i] - pred) & 0xff
    return bytes([f]) + bytes(out)


def _unfilter(data, h, rb, bpp):
    rows, prev, at = [], None, 0
    for _ in range(h):
        f = data[at]
        cur = bytearray(data[at + 1:at + 1 + rb])
        at += 1 + rb
        for i in range(rb):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i] if prev is not None else 0
            c = prev[i - bpp] if (prev is not None and i >= bpp) else 0
            cur[i] = (cur[i] + [0, a, b, (a + b) >> 1, _paeth(a, b, c)][f]) & 0xff
        rows.append(bytes(cur))
        prev = cur
    return rows


def make_png(samples, depth, ctype, interlace=0, plte=None, comp=None, rng=None, idat_pieces=1,
             ancillary=True, filters=None):
    """PNG bytes of samples [H, W, C] (C = channels of ctype)"""
    rng = rng or np.random.default_rng(0)
    H, W, C = samples.shape
    bpp = max(1, C * depth // 8)
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    raw = bytearray()
    for (x0, y0, dx, dy) in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        prev = None
        for y in range(sub.shape[0]):
            row = _pack_row(sub[y].reshape(-1), depth)
            f = int(rng.integers(0, 5)) if filters is None else filters
            raw += _filter(row, prev, f, bpp)
            prev = row
    level, strategy = comp or (6, zlib.Z_DEFAULT_STRATEGY)
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    z = co.compress(bytes(raw)) + co.flush()
    out = SIG + _chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, ctype, 0, 0, interlace))
    if ancillary:
        out += _chunk(b"tEXt", b"Comment\x00test frame")
    if plte is not None:
        out += _chunk(b"PLTE", plte.astype(np.uint8).tobytes())
    step = max(1, -(-len(z) // idat_pieces))
    for at in range(0, len(z), step):
        out += _chunk(b"IDAT", z[at:at + step])
    return out + _chunk(b"IEND", b"")


def expected_bgr(samples, depth, ctype, plte=None):
    H, W, _ = samples.shape
    if ctype in (0, 4):
        g = samples[..., 0].astype(np.int64)
        g = g >> 8 if depth == 16 else (g * 255 // ((1 << depth) - 1) if depth < 8 else g)
        return np.repeat(g[..., None], 3, axis=2).astype(np.uint8)
    if ctype == 3:
        return plte[samples[..., 0]][..., ::-1].astype(np.uint8)
    rgb = samples[..., :3].astype(np.int64)
    if depth == 16:
        rgb = rgb >> 8
    return rgb[..., ::-1].astype(np.uint8)


def random_image(rng, W, H, depth, ctype, smooth=False):
    C = CHANNELS[ctype]
    top = (1 << depth) if ctype != 3 else None
    plte = None
    if ctype == 3:
        npal = int(rng.integers(1, (1 << depth) + 1))
        plte = rng.integers(0, 256, (npal, 3))
        top = npal
    if smooth:
        yy, xx = np.mgrid[0:H, 0:W]
        base = ((xx * 7 + yy * 3) // 5) % top
        s = np.repeat(base[..., None], C, axis=2) + rng.integers(0, 2, (H, W, C))
        s = np.minimum(s, top - 1)
    else:
        s = rng.integers(0, top, (H, W, C))
    return s.astype(np.int64), plte


def _write(tmp_path, name, data):
    p = tmp_path / name
    p.write_bytes(data)
    return str(p)


STRATEGIES = [(0, zlib.Z_DEFAULT_STRATEGY), (6, zlib.Z_FIXED), (9, zlib.Z_DEFAULT_STRATEGY),
              (6, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE), (1, zlib.Z_FILTERED)]


@pytest.mark.parametrize("ctype,depth", COMBOS)
@pytest.mark.parametrize("interlace", [0, 1])
def test_decode_every_format(tmp_path, ctype, depth, interlace):
    rng = np.random.default_rng(1000 * ctype + 10 * depth + interlace)
    for k, comp in enumerate(STRATEGIES):
        for (W, H) in [(1, 1), (3, 2), (13, 9), (37, 21)]:
            s, plte = random_image(rng, W, H, depth, ctype, smooth=bool(k % 2))
            data = make_png(s, depth, ctype, interlace, plte, comp, rng, idat_pieces=1 + k % 3)
            p = _write(tmp_path, f"f{k}_{W}x{H}.png", data)
            assert asv.png_info(p) == (W, H)
            got = asv.read_png(p)
            want = expected_bgr(s, depth, ctype, plte)
            assert np.array_equal(got, want), (ctype, depth, interlace, comp, W, H)


def test_decode_large_dynamic(tmp_path):
    """a large frame with skewed statistics: long Huffman codes (over 10
    bits) and long-distance matches"""
    rng = np.random.default_rng(7)
    W, H = 640, 360
    yy, xx = np.mgrid[0:H, 0:W]
    img = np.stack([(xx // 40 * 37) % 256, (yy // 30 * 53) % 256, ((xx + yy) // 50 * 19) % 256], -1)
    noise = rng.random((H, W)) < 0.03
    img[noise] = rng.integers(0, 256, (int(noise.sum()), 3))
    for filt in (None, 0):
        data = make_png(img.astype(np.int64), 8, 2, 0, None, (9, zlib.Z_DEFAULT_STRATEGY), rng, 5,
                        filters=filt)
        p = _write(tmp_path, "big.png", data)
        assert np.array_equal(asv.read_png(p), img[..., ::-1].astype(np.uint8))


def _decode_here(data):
    """the library's PNG output decoded independently: chunk CRCs, zlib,
    NumPy unfiltering"""
    assert data[:8] == SIG
    at, idat, hdr = 8, b"", None
    while at < len(data):
        (n,) = struct.unpack(">I", data[at:at + 4])
        kind, body = data[at + 4:at + 8], data[at + 8:at + 8 + n]
        (crc,) = struct.unpack(">I", data[at + 8 + n:at + 12 + n])
        assert crc == zlib.crc32(kind + body) & 0xffffffff
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
        at += 12 + n
    W, H, depth, ctype, _, _, inter = hdr
    assert (depth, ctype, inter) == (8, 2, 0)
    raw = zlib.decompress(idat)
    rows = _unfilter(raw, H, 3 * W, 3)
    return np.frombuffer(b"".join(rows), np.uint8).reshape(H, W, 3)


@pytest.mark.parametrize("kind", ["noise", "flat", "render", "tiny"])
def test_encode_decodes_with_zlib(tmp_path, kind):
    rng = np.random.default_rng(3)
    if kind == "noise":
        img = rng.integers(0, 256, (45, 67, 3), dtype=np.uint8)
    elif kind == "flat":
        img = np.full((40, 300, 3), 17, np.uint8)
    elif kind == "tiny":
        img = rng.integers(0, 256, (1, 1, 3), dtype=np.uint8)
    else:
        lab = (np.arange(64)[None, :, None] // 9 + np.arange(48)[None, None, :] // 7 * 10).repeat(1, 0)
        lab = np.broadcast_to(lab.transpose(0, 2, 1), (1, 48, 64)).astype(np.int32)
        img = asv.render_rgb(lab, int(lab.max()) + 1)[0]
    p = str(tmp_path / "o.png")
    asv.write_png(p, img)
    data = open(p, "rb").read()
    assert np.array_equal(_decode_here(data), img)
    assert np.array_equal(asv.read_png(p), img[..., ::-1])
    if kind in ("flat", "render"):
        assert len(data) < img.nbytes // 10          # piecewise-constant frames compress


def _corrupt_chunk(data, kind, fn):
    """applies fn to the body of the first chunk `kind` and re-signs it"""
    at = 8
    while at < len(data):
        (n,) = struct.unpack(">I", data[at:at + 4])
        k, body = data[at + 4:at + 8], data[at + 8:at + 8 + n]
        if k == kind:
            nb = fn(body)
            return data[:at] + _chunk(k, nb) + data[at + 12 + n:]
        at += 12 + n
    raise AssertionError(kind)


def test_errors(tmp_path):
    rng = np.random.default_rng(5)
    s, _ = random_image(rng, 20, 10, 8, 2)
    good = make_png(s, 8, 2, 0, None, (6, zlib.Z_DEFAULT_STRATEGY), rng)
    ok = _write(tmp_path, "ok.png", good)
    assert asv.read_png(ok).shape == (10, 20, 3)

    def bad(name, data, exc=ValueError, match="malformed"):
        p = _write(tmp_path, name, data)
        with pytest.raises(exc, match=match):
            asv.read_png(p)

    bad("sig.png", b"\x88" + good[1:])
    flip = bytearray(good)
    flip[40] ^= 1                                        # inside IHDR/tEXt: CRC mismatch
    bad("crc.png", bytes(flip))
    bad("trunc.png", good[:len(good) // 2])
    bad("noiend.png", good[:-12])
    bad("adler.png", _corrupt_chunk(good, b"IDAT", lambda b: b[:-1] + bytes([b[-1] ^ 0xff])))
    bad("zhdr.png", _corrupt_chunk(good, b"IDAT", lambda b: bytes([0x79]) + b[1:]))
    raw = zlib.decompress(_idat(good))
    bad("filter.png", _corrupt_chunk(good, b"IDAT", lambda b: zlib.compress(bytes([5]) + raw[1:])))
    bad("short.png", _corrupt_chunk(good, b"IDAT", lambda b: zlib.compress(raw[:-3])))
    bad("long.png", _corrupt_chunk(good, b"IDAT", lambda b: zlib.compress(raw + b"\x00\x00")))
    crit = good[:-12] + _chunk(b"ABCD", b"xyz") + good[-12:]
    bad("crit.png", crit, match="unsupported")
    pal = make_png(np.zeros((2, 2, 1), np.int64) + 3, 8, 3, 0, np.zeros((2, 3)), None, rng)
    bad("pal.png", pal)                                   # index 3 of a 2-entry palette
    with pytest.raises(OSError):
        asv.read_png(str(tmp_path / "missing.png"))
    huge = _corrupt_chunk(good, b"IHDR", lambda b: struct.pack(">II", 16384, 16384) + b[8:])
    p = _write(tmp_path, "huge.png", huge)
    with pytest.raises(ValueError, match="malformed"):          # 2^28 pixels claimed by a tiny stream
        asv.read_png(p)
    s2, _ = random_image(rng, 21, 10, 8, 2)
    other = _write(tmp_path, "other.png", make_png(s2, 8, 2, 0, None, None, rng))
    with pytest.raises(ValueError, match="size"):
        asv.read_frames([ok, other])


def _idat(data):
    at, z = 8, b""
    while at < len(data):
        (n,) = struct.unpack(">I", data[at:at + 4])
        if data[at + 4:at + 8] == b"IDAT":
            z += data[at + 8:at + 8 + n]
        at += 12 + n
    return z


def test_fuzz_corrupt_streams(tmp_path):
    """random damage inside the zlib stream (chunk CRCs re-signed so the
    damage reaches the inflater): every file decodes or is refused, and a
    decoded frame is the right size"""
    rng = np.random.default_rng(11)
    s, _ = random_image(rng, 31, 17, 8, 6, smooth=True)
    for it in range(300):
        comp = STRATEGIES[it % len(STRATEGIES)]
        good = make_png(s, 8, 6, it % 2, None, comp, rng)

        def damage(b):
            b = bytearray(b)
            for _ in range(int(rng.integers(1, 4))):
                b[int(rng.integers(0, len(b)))] ^= 1 << int(rng.integers(0, 8))
            if rng.random() < 0.2:
                b = b[:int(rng.integers(0, len(b)))]
            return bytes(b)
        p = _write(tmp_path, "fz.png", _corrupt_chunk(good, b"IDAT", damage))
        try:
            out = asv.read_png(p)
            assert out.shape == (17, 31, 3)
        except ValueError:
            pass


def test_sanitized_fuzz(tmp_path):
    """the decoder built with AddressSanitizer and UndefinedBehaviorSanitizer
    (tests/png_fuzz.cpp) runs 100 000 damaged files made from a corpus of
    every colour type, bit depth, interlacing and zlib strategy: no
    out-of-bounds access, no undefined behaviour, every case a status code"""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "anisotropic_supervoxel_gb300", "csrc")
    inc = os.path.join(os.path.dirname(csrc), "..", "include")
    exe = str(tmp_path / "png_fuzz")
    build = subprocess.run([gxx, "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
                            "-fopenmp", "-I", csrc, "-I", inc,
                            os.path.join(os.path.dirname(os.path.abspath(__file__)), "png_fuzz.cpp"),
                            "-o", exe], capture_output=True, text=True)
    if build.returncode != 0:
        pytest.skip("sanitizer runtime unavailable: " + build.stderr[-200:])
    corpus = tmp_path / "corpus"
    corpus.mkdir()
    rng = np.random.default_rng(17)
    n = 0
    for ctype, depth in COMBOS:
        for interlace in (0, 1):
            for W, H in ((1, 1), (7, 5), (33, 17)):
                comp = STRATEGIES[n % len(STRATEGIES)]
                s, plte = random_image(rng, W, H, depth, ctype, smooth=bool(n % 2))
                (corpus / f"c{n:03d}.png").write_bytes(make_png(s, depth, ctype, interlace, plte, comp, rng,
                                                                idat_pieces=1 + n % 3))
                n += 1
    run = subprocess.run([exe, str(corpus), "100000", "7"], capture_output=True, text=True, timeout=600,
                         env=dict(os.environ, ASAN_OPTIONS="detect_leaks=1"))
    assert run.returncode == 0, run.stderr[-2000:]
    counts = [int(v) for v in run.stdout.split()[3:4] + run.stdout.split()[5:]]
    ok, fails = counts[0], counts[1:]
    assert ok > 5000 and sum(fails) > 50000 and ok + sum(fails) == 100000, run.stdout
    assert fails[0] == fails[1] == fails[2] == fails[6] == fails[7] == 0, run.stdout   # only -3, -4, -5


def test_frames_and_render_files(tmp_path):
    rng = np.random.default_rng(2)
    frames = rng.integers(0, 256, (5, 12, 16, 3), dtype=np.uint8)
    for t in range(5):
        asv.write_png(str(tmp_path / f"{t:03d}.png"), frames[t][..., ::-1])    # BGR frames stored as RGB
    (tmp_path / "notes.txt").write_text("not a frame")
    paths = asv.list_frames(str(tmp_path))
    assert [os.path.basename(p) for p in paths] == [f"{t:03d}.png" for t in range(5)]
    assert np.array_equal(asv.read_frames(paths), frames)
    buf = np.zeros_like(frames)
    assert asv.read_frames(paths, out=buf) is buf and np.array_equal(buf, frames)
    with pytest.raises(ValueError):
        asv.read_frames(paths, out=np.zeros((4, 12, 16, 3), np.uint8))

    lab = rng.integers(-1, 30, (3, 12, 16)).astype(np.int32)
    rgb = asv.render_rgb(lab, 30)
    pre = str(tmp_path / "r_")
    asv.write_render_ppm(pre, lab, 30)
    asv.write_render_png(pre, lab, 30)
    asv.write_render_png(pre, lab, 30, start_index=20)
    for t in range(3):
        ppm = open(f"{pre}{t:05d}.ppm", "rb").read()
        body = np.frombuffer(ppm[len(b"P6\n16 12\n255\n"):], np.uint8).reshape(12, 16, 3)
        assert np.array_equal(body, rgb[t])
        assert np.array_equal(asv.read_png(f"{pre}{t + 1:05d}.png"), rgb[t][..., ::-1])
        assert np.array_equal(asv.read_png(f"{pre}00020_{t + 21:05d}.png"), rgb[t][..., ::-1])
    assert np.all(rgb[lab[:, ::-1] < 0] == 0)             # -1 is black (frames are un-flipped)
