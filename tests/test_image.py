"""Image output (dr_image_*): the reference's float -> byte rule, the block-major -> row-major walk,
PNG and PFM files.  The PNG writer is pinned against the reference's own Images::saveBufferPNG
(lodepng, built into oracle/_ref): both files decode to identical pixels.  CPU only."""
import struct
import zlib

import numpy as np
import pytest

import dumbray_gb300 as dr
import _oracle as O


def _decode_png(path):
    """Minimal PNG reader for 8-bit RGBA, non-interlaced files (all filter types)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        if typ == b"IHDR":
            w, h, depth, ctype, _, _, inter = struct.unpack(">IIBBBBB", body)
            assert (depth, ctype, inter) == (8, 6, 0)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    out = np.zeros((h, 4 * w), np.int32)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        prev = out[y - 1] if y else np.zeros(4 * w, np.int32)
        cur = np.zeros(4 * w, np.int32)
        for i in range(4 * w):
            a = cur[i - 4] if i >= 4 else 0
            b = prev[i]
            c = prev[i - 4] if i >= 4 else 0
            if f == 0:
                pred = 0
            elif f == 1:
                pred = a
            elif f == 2:
                pred = b
            elif f == 3:
                pred = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            cur[i] = (line[i] + pred) & 0xFF
        out[y] = cur
    return out.reshape(h, w, 4).astype(np.uint8)


def _test_image(h=19, w=23, seed=0):
    rng = np.random.default_rng(seed)
    img = rng.uniform(-0.3, 1.4, (h, w, 4)).astype(np.float32)
    img[0, 0] = [0.0, 1.0, 255.0 / 255.0, 254.999 / 255.0]
    img[0, 1] = [1.0 / 255.0, -0.0, 0.9999999, 1e-9]
    return img


def _reference_rule(img):
    v = np.float32(255.0) * img.astype(np.float32)
    return np.where(v > 255, 255, np.where(v < 0, 0, np.trunc(v))).astype(np.uint8)


def test_rgba8_matches_the_reference_rule():
    img = _test_image()
    assert np.array_equal(dr.to_rgba8(img), _reference_rule(img))


def test_png_round_trip(tmp_path):
    img = _test_image(37, 70000 // 37 // 4 + 5)   # rows long enough to span several stored blocks
    p = tmp_path / "a.png"
    dr.write_png(img, p)
    assert np.array_equal(_decode_png(p), _reference_rule(img))


@pytest.mark.skipif(not O.reference_available(), reason="reference library not built here")
def test_png_pixels_equal_reference_saveBufferPNG(tmp_path):
    """Images::saveBufferPNG of the reference (through its BlockBuffer and lodepng) and
    dr_image_write_png decode to the same RGBA bytes."""
    L = O.reference()
    if not hasattr(L, "dref_save_png"):
        pytest.skip("reference library predates its PNG export")
    img = _test_image(21, 34, seed=3)
    ours, ref = tmp_path / "ours.png", tmp_path / "ref.png"
    dr.write_png(img, ours)
    assert L.dref_save_png(img.ctypes.data, img.shape[1], img.shape[0], str(ref).encode()) == 0
    assert np.array_equal(_decode_png(ours), _decode_png(ref))


def test_pfm_round_trip(tmp_path):
    img = _test_image(9, 13, seed=1)
    p = tmp_path / "a.pfm"
    dr.write_pfm(img, p)
    data = open(p, "rb").read()
    head = b"PF\n13 9\n-1.0\n"
    assert data.startswith(head)
    px = np.frombuffer(data[len(head):], "<f4").reshape(9, 13, 3)[::-1]
    assert np.array_equal(px, img[..., :3])


def test_image_from_blocks_matches_python_layout():
    W, H = 37, 21
    img = np.random.default_rng(2).standard_normal((H, W, 4)).astype(np.float32)
    fb = dr.image_to_blockmajor(img)
    assert np.array_equal(dr.image_from_blocks(fb, W, H), img)


def test_image_argument_errors(tmp_path):
    with pytest.raises(ValueError):
        dr.write_png(np.zeros((4, 4, 3), np.float32), tmp_path / "x.png")
    with pytest.raises(dr.DumbRayError):
        dr.write_png(np.zeros((4, 4, 4), np.float32), tmp_path / "no_such_dir" / "x.png")
