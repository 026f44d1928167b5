"""BMP and binary PNM frame input (csrc/asv_frames.cpp) against files built here.

The Render::run frame loop reads every file of the sorted folder with
cv::imread(path, 1) (GPU-AS/Render.cpp:151-157, 229-238), so a folder of
BMP or PPM frames is as valid an input as PNG.  Each test writes a frame with
`struct` and NumPy from the published file layouts and checks the decoded
8-bit BGR pixels, top row first.  Host code only: no GPU.
"""
import os
import struct

import numpy as np
import pytest

import anisotropic_supervoxel_gb300 as asv
from anisotropic_supervoxel_gb300 import _lib

F_FORMAT, F_UNSUPPORTED, F_SIZE = -3, -4, -5


def _bmp(pixel_rows, W, H, bpp, comp=0, palette=None, masks=None, top_down=False, hdr=40):
    """a BMP file: pixel_rows are the stored rows (bytes, unpadded) in file order"""
    stride = ((W * bpp + 31) // 32) * 4
    body = b"".join(r + b"\0" * (stride - len(r)) for r in pixel_rows)
    extra = b""
    if masks is not None:
        extra = struct.pack("<3I", *masks)
    pal = b"" if palette is None else b"".join(struct.pack("<4B", b, g, r, 0) for (b, g, r) in palette)
    info = struct.pack("<IiiHHIIiiII", hdr, W, -H if top_down else H, 1, bpp, comp, len(body), 2835, 2835,
                       0 if palette is None else len(palette), 0)
    info += b"\0" * (hdr - 40)
    off = 14 + hdr + len(extra) + len(pal)
    head = b"BM" + struct.pack("<IHHI", off + len(body), 0, 0, off)
    return head + info + extra + pal + body


def _write(tmp_path, name, data):
    p = os.path.join(tmp_path, name)
    with open(p, "wb") as f:
        f.write(data)
    return p


def _decode(path):
    return asv.read_frame(path)


def test_bmp24_bottom_up_padded(tmp_path):
    rng = np.random.default_rng(1)
    W, H = 7, 5                                   # 21-byte rows padded to 24
    img = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    rows = [img[H - 1 - r].tobytes() for r in range(H)]
    p = _write(tmp_path, "a.bmp", _bmp(rows, W, H, 24))
    assert asv.frame_info(p) == (W, H)
    np.testing.assert_array_equal(_decode(p), img)


def test_bmp24_top_down_and_v5_header(tmp_path):
    rng = np.random.default_rng(2)
    W, H = 9, 4
    img = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    rows = [img[r].tobytes() for r in range(H)]
    p = _write(tmp_path, "b.bmp", _bmp(rows, W, H, 24, top_down=True, hdr=124))
    np.testing.assert_array_equal(_decode(p), img)


def test_bmp32_alpha_dropped(tmp_path):
    rng = np.random.default_rng(3)
    W, H = 6, 3
    img = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    alpha = rng.integers(0, 256, (H, W, 1), dtype=np.uint8)
    bgra = np.concatenate([img, alpha], axis=2)
    rows = [bgra[H - 1 - r].tobytes() for r in range(H)]
    p = _write(tmp_path, "c.bmp", _bmp(rows, W, H, 32))
    np.testing.assert_array_equal(_decode(p), img)


def test_bmp32_bitfields(tmp_path):
    rng = np.random.default_rng(4)
    W, H = 5, 4
    img = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)   # stored as R<<24 | G<<16 | B<<8
    px = (img[..., 2].astype(np.uint32) << 24) | (img[..., 1].astype(np.uint32) << 16) | (img[..., 0].astype(np.uint32) << 8)
    rows = [px[H - 1 - r].astype("<u4").tobytes() for r in range(H)]
    p = _write(tmp_path, "d.bmp", _bmp(rows, W, H, 32, comp=3, masks=(0xff000000, 0x00ff0000, 0x0000ff00)))
    np.testing.assert_array_equal(_decode(p), img)


@pytest.mark.parametrize("layout", ["555", "565"])
def test_bmp16(tmp_path, layout):
    rng = np.random.default_rng(5)
    W, H = 11, 3                                  # 22-byte rows padded to 24
    if layout == "555":
        bits, masks, comp = (5, 5, 5), None, 0
    else:
        bits, masks, comp = (5, 6, 5), (0xf800, 0x07e0, 0x001f), 3
    r = rng.integers(0, 1 << bits[0], (H, W)).astype(np.uint32)
    g = rng.integers(0, 1 << bits[1], (H, W)).astype(np.uint32)
    b = rng.integers(0, 1 << bits[2], (H, W)).astype(np.uint32)
    px = (r << (bits[1] + bits[2])) | (g << bits[2]) | b
    rows = [px[H - 1 - y].astype("<u2").tobytes() for y in range(H)]
    p = _write(tmp_path, "e.bmp", _bmp(rows, W, H, 16, comp=comp, masks=masks))
    want = np.stack([b << (8 - bits[2]), g << (8 - bits[1]), r << (8 - bits[0])], axis=2).astype(np.uint8)
    np.testing.assert_array_equal(_decode(p), want)


@pytest.mark.parametrize("bpp", [1, 4, 8])
def test_bmp_palette(tmp_path, bpp):
    rng = np.random.default_rng(10 + bpp)
    W, H = 13, 6
    n = 1 << bpp
    palette = [tuple(int(v) for v in rng.integers(0, 256, 3)) for _ in range(n)]
    idx = rng.integers(0, n, (H, W))
    rows = []
    for y in range(H - 1, -1, -1):
        out = bytearray((W * bpp + 7) // 8)
        per = 8 // bpp
        for x in range(W):
            out[x // per] |= int(idx[y, x]) << (8 - bpp * (x % per + 1))
        rows.append(bytes(out))
    p = _write(tmp_path, "f.bmp", _bmp(rows, W, H, bpp, palette=palette))
    want = np.array(palette, np.uint8)[idx]
    np.testing.assert_array_equal(_decode(p), want)


def test_bmp_refused_and_truncated(tmp_path):
    W, H = 4, 2
    rows = [bytes(W) for _ in range(H)]
    rle = _write(tmp_path, "rle.bmp", _bmp(rows, W, H, 8, comp=1, palette=[(0, 0, 0)] * 256))
    lib = _lib.load()
    out = np.zeros((H, W, 3), np.uint8)
    assert lib.asv_frame_read_bgr(os.fsencode(rle), out.ctypes.data, W, H) == F_UNSUPPORTED
    full = _bmp([bytes(3 * W)] * H, W, H, 24)
    cut = _write(tmp_path, "cut.bmp", full[:-5])
    assert lib.asv_frame_read_bgr(os.fsencode(cut), out.ctypes.data, W, H) == F_FORMAT
    ok = _write(tmp_path, "ok.bmp", full)
    assert lib.asv_frame_read_bgr(os.fsencode(ok), out.ctypes.data, W + 1, H) == F_SIZE


def test_pnm_p6_p5_comments_and_16bit(tmp_path):
    rng = np.random.default_rng(6)
    W, H = 10, 7
    rgb = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    p6 = _write(tmp_path, "g.ppm", b"P6\n# made here\n%d %d\n# max\n255\n" % (W, H) + rgb.tobytes())
    assert asv.frame_info(p6) == (W, H)
    np.testing.assert_array_equal(_decode(p6), rgb[..., ::-1])
    grey = rng.integers(0, 256, (H, W), dtype=np.uint8)
    p5 = _write(tmp_path, "h.pgm", b"P5 %d %d 255\n" % (W, H) + grey.tobytes())
    np.testing.assert_array_equal(_decode(p5), np.repeat(grey[..., None], 3, axis=2))
    wide = rng.integers(0, 65536, (H, W, 3), dtype=np.uint16)
    p16 = _write(tmp_path, "i.ppm", b"P6\n%d %d\n65535\n" % (W, H) + wide.astype(">u2").tobytes())
    np.testing.assert_array_equal(_decode(p16), (wide >> 8).astype(np.uint8)[..., ::-1])
    lib = _lib.load()
    out = np.zeros((H, W, 3), np.uint8)
    odd = _write(tmp_path, "j.ppm", b"P6\n%d %d\n1023\n" % (W, H) + bytes(2 * 3 * W * H))
    assert lib.asv_frame_read_bgr(os.fsencode(odd), out.ctypes.data, W, H) == F_UNSUPPORTED
    short = _write(tmp_path, "k.ppm", b"P6\n%d %d\n255\n" % (W, H) + rgb.tobytes()[:-1])
    assert lib.asv_frame_read_bgr(os.fsencode(short), out.ctypes.data, W, H) == F_FORMAT


def test_mixed_folder_matches_png(tmp_path):
    """a folder of BMP, PPM and PNG frames of one size reads like the PNG frames"""
    rng = np.random.default_rng(7)
    W, H = 12, 8
    frames = rng.integers(0, 256, (3, H, W, 3), dtype=np.uint8)
    _write(tmp_path, "000.bmp", _bmp([frames[0][H - 1 - r].tobytes() for r in range(H)], W, H, 24))
    _write(tmp_path, "001.ppm", b"P6\n%d %d\n255\n" % (W, H) + frames[1][..., ::-1].tobytes())
    asv.write_png(os.path.join(tmp_path, "002.png"), frames[2][..., ::-1])   # RGB in, BGR out
    _write(tmp_path, "notes.txt", b"not a frame")
    paths = asv.list_frames(str(tmp_path))
    assert [os.path.basename(p) for p in paths] == ["000.bmp", "001.ppm", "002.png"]
    np.testing.assert_array_equal(asv.read_frames(paths), frames)
