"""dr_png_read (texture PNG decoding) against the reference's lodepng::decode to 8-bit RGBA.

Inputs come from a small PNG writer here (numpy + zlib): every colour type and bit depth, random
row filters, tRNS palettes and colour keys, Adam7 interlacing, stored / fixed / dynamic deflate
blocks, image data split over several IDAT chunks.  Expected pixels are computed independently in
numpy; the reference decoder, when built, must agree byte for byte too."""
import ctypes
import struct
import zlib

import numpy as np
import pytest

import dumbray_gb300 as dr
import _oracle as O

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunk(kind, data):
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def _pack_rows(img, depth):
    """img: (h, w, ch) integer samples -> list of row byte strings."""
    h, w, ch = img.shape
    rows = []
    for y in range(h):
        flat = img[y].reshape(-1).astype(np.uint32)
        if depth == 16:
            rows.append(flat.astype(">u2").tobytes())
        elif depth == 8:
            rows.append(flat.astype(np.uint8).tobytes())
        else:
            per = 8 // depth
            nbytes = (len(flat) * depth + 7) // 8
            out = bytearray(nbytes)
            for i, v in enumerate(flat):
                out[i // per] |= int(v) << (8 - depth * (i % per + 1))
            rows.append(bytes(out))
    return rows


def _filter_rows(rows, bpp, rng):
    out = bytearray()
    prev = bytes(len(rows[0])) if rows else b""
    for row in rows:
        f = int(rng.integers(0, 5))
        cur = np.frombuffer(row, np.uint8).astype(np.int32)
        p = np.frombuffer(prev, np.uint8).astype(np.int32)
        enc = np.zeros_like(cur)
        for i in range(len(cur)):
            a = cur[i - bpp] if i >= bpp else 0
            b = p[i]
            c = p[i - bpp] if i >= bpp else 0
            if f == 0:
                pred = 0
            elif f == 1:
                pred = a
            elif f == 2:
                pred = b
            elif f == 3:
                pred = (a + b) >> 1
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            enc[i] = (cur[i] - pred) & 255
        out += bytes([f]) + enc.astype(np.uint8).tobytes()
        prev = row
    return bytes(out)


def make_png(img, ctype, depth, palette=None, trns=None, interlace=False, level=6, seed=0, idat_split=3):
    rng = np.random.default_rng(seed)
    h, w, ch = img.shape
    bpp = max(1, ch * depth // 8)
    if interlace:
        raw = b""
        for (x0, y0, dx, dy) in ADAM7:
            sub = img[y0::dy, x0::dx]
            if sub.shape[0] and sub.shape[1]:
                raw += _filter_rows(_pack_rows(sub, depth), bpp, rng)
    else:
        raw = _filter_rows(_pack_rows(img, depth), bpp, rng)
    z = zlib.compress(raw, level)
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 1 if interlace else 0))
    if palette is not None:
        out += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        out += _chunk(b"tRNS", trns)
    k = max(1, len(z) // idat_split)
    for i in range(0, len(z), k):
        out += _chunk(b"IDAT", z[i:i + k])
    return out + _chunk(b"IEND", b"")


def expected_rgba(img, ctype, depth, palette=None, trns=None):
    h, w, _ = img.shape
    out = np.zeros((h, w, 4), np.uint8)

    def to8(v):
        v = v.astype(np.int64)
        if depth == 16:
            return (v >> 8).astype(np.uint8)
        if depth == 8:
            return v.astype(np.uint8)
        return ((v * 255) // ((1 << depth) - 1)).astype(np.uint8)

    if ctype == 3:
        pal = np.full((len(palette), 4), 255, np.uint8)
        pal[:, :3] = palette
        if trns is not None:
            a = np.frombuffer(trns, np.uint8)
            pal[:len(a), 3] = a
        return pal[img[..., 0]]
    if ctype in (0, 4):
        g = to8(img[..., 0])
        out[..., 0] = out[..., 1] = out[..., 2] = g
        if ctype == 4:
            out[..., 3] = to8(img[..., 1])
        else:
            key = struct.unpack(">H", trns[:2])[0] if trns else None
            out[..., 3] = np.where(img[..., 0] == key, 0, 255) if key is not None else 255
        return out
    for k in range(3):
        out[..., k] = to8(img[..., k])
    if ctype == 6:
        out[..., 3] = to8(img[..., 3])
    else:
        if trns:
            key = struct.unpack(">HHH", trns[:6])
            match = (img[..., 0] == key[0]) & (img[..., 1] == key[1]) & (img[..., 2] == key[2])
            out[..., 3] = np.where(match, 0, 255)
        else:
            out[..., 3] = 255
    return out


CASES = []
for ctype, depths in ((0, (1, 2, 4, 8, 16)), (2, (8, 16)), (3, (1, 2, 4, 8)), (4, (8, 16)), (6, (8, 16))):
    for depth in depths:
        for interlace in (False, True):
            CASES.append((ctype, depth, interlace))


def _case(ctype, depth, interlace, seed, w=13, h=11, level=6, with_trns=True):
    rng = np.random.default_rng(seed)
    ch = CHANNELS[ctype]
    top = (1 << depth) if ctype != 3 else min(1 << depth, 7)
    img = rng.integers(0, top, size=(h, w, ch))
    palette = trns = None
    if ctype == 3:
        palette = rng.integers(0, 256, size=(top, 3))
        if with_trns:
            trns = bytes(rng.integers(0, 256, size=top - 2).astype(np.uint8))
    elif ctype == 0 and with_trns:
        trns = struct.pack(">H", int(img[3, 4, 0]))
    elif ctype == 2 and with_trns:
        trns = struct.pack(">HHH", *[int(v) for v in img[2, 5]])
    data = make_png(img, ctype, depth, palette, trns, interlace, level=level, seed=seed)
    return data, expected_rgba(img, ctype, depth, palette, trns)


def _ours(path):
    L = dr.lib()
    w, h = ctypes.c_int32(), ctypes.c_int32()
    dr.check(L.dr_png_read(str(path).encode(), ctypes.byref(w), ctypes.byref(h), None))
    out = np.zeros((h.value, w.value, 4), np.uint8)
    dr.check(L.dr_png_read(str(path).encode(), ctypes.byref(w), ctypes.byref(h), out.ctypes.data))
    return out


def _ref(path):
    L = O.reference()
    if not hasattr(L, "dref_png_decode"):
        return None
    L.dref_png_decode.restype = ctypes.c_int
    L.dref_png_decode.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    w, h = ctypes.c_int(), ctypes.c_int()
    assert L.dref_png_decode(str(path).encode(), ctypes.byref(w), ctypes.byref(h), None) == 0
    out = np.zeros((h.value, w.value, 4), np.uint8)
    assert L.dref_png_decode(str(path).encode(), ctypes.byref(w), ctypes.byref(h), out.ctypes.data) == 0
    return out


@pytest.mark.parametrize("ctype,depth,interlace", CASES)
def test_png_decoding(tmp_path, ctype, depth, interlace):
    for level, seed in ((0, 1), (1, 2), (9, 3)):   # stored, fixed-Huffman-heavy, dynamic blocks
        data, want = _case(ctype, depth, interlace, seed, level=level)
        path = tmp_path / f"t{level}.png"
        path.write_bytes(data)
        got = _ours(path)
        assert np.array_equal(got, want)
        if O.reference_available():
            ref = _ref(path)
            if ref is not None:
                assert np.array_equal(got, ref)


def test_png_larger_and_own_writer(tmp_path):
    """A larger image (long back-references) and the files dr_image_write_png writes."""
    rng = np.random.default_rng(5)
    img = (rng.integers(0, 4, size=(96, 160, 4)) * 60).astype(np.int64)   # repetitive: many matches
    data = make_png(img, 6, 8, level=9, seed=7)
    (tmp_path / "big.png").write_bytes(data)
    assert np.array_equal(_ours(tmp_path / "big.png"), img.astype(np.uint8))
    rgba = rng.uniform(0, 1, size=(9, 7, 4)).astype(np.float32)
    dr.write_png(rgba, tmp_path / "own.png")
    assert np.array_equal(_ours(tmp_path / "own.png"), dr.to_rgba8(rgba))


def test_png_errors(tmp_path):
    (tmp_path / "x.png").write_bytes(b"not a png at all")
    good, _ = _case(2, 8, False, 1)
    (tmp_path / "trunc.png").write_bytes(good[:60])
    for name in ("x.png", "trunc.png", "missing.png"):
        with pytest.raises(dr.DumbRayError):
            _ours(tmp_path / name)
