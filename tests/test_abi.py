"""The C ABI library loads and exports every entry point include/dr_api.h declares; argument
validation paths that need no device work."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import dumbray_gb300 as dr

HEADER = Path(__file__).resolve().parent.parent / "include" / "dr_api.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(dr_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("dr_scene_create", "dr_cast", "dr_render_blocks", "dr_renderer_create", "dr_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    L = dr.lib()
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_block_count():
    L = dr.lib()
    assert L.dr_version() >= 100
    assert L.dr_block_count(1920, 1080) == 240 * 68
    assert L.dr_block_count(256, 256) == 32 * 16
    assert L.dr_block_count(0, 10) == 0
    assert dr.block_count(1920, 1080) == 16320


def test_argument_errors_are_reported_without_device_work():
    L = dr.lib()
    assert L.dr_scene_create(None, None, None, 0, None, 0, None, 0, None, None) == dr.DR_E_ARG
    assert b"out is NULL" in L.dr_last_error()
    h = ctypes.c_void_p()
    assert L.dr_scene_create(None, None, None, -1, None, 0, None, 0, None, ctypes.byref(h)) == dr.DR_E_ARG
    tris = np.zeros((2, 3, 3), np.float32)
    bad = np.array([0, 3], np.int32)
    m = (dr.DrMaterial * 1)(dr.lambert())
    assert L.dr_scene_create(tris.ctypes.data, None, bad.ctypes.data, 2, ctypes.addressof(m), 1, None, 0, None,
                             ctypes.byref(h)) == dr.DR_E_ARG
    assert b"material id out of range" in L.dr_last_error()
    assert L.dr_renderer_create(-5, ctypes.byref(h)) == dr.DR_E_ARG
    assert L.dr_cast(None, None, None, None, 0, 1, None, None, None) == dr.DR_E_ARG
    assert L.dr_render_blocks(None, None, None, None, 0, 0, None, None) == dr.DR_E_ARG
    with pytest.raises(dr.DumbRayError):
        dr.check(dr.DR_E_ARG)


def test_block_major_layout_matches_reference_formula():
    """BlockBasedFrameBuffer<8,16>::blockPixelLocation (BlockBasedFrameBuffer.impl.cuh:125-142)."""
    W, H = 37, 21
    img = np.arange(H * W * 4, dtype=np.float32).reshape(H, W, 4)
    fb = dr.image_to_blockmajor(img)
    bw = (W + 7) // 8
    for block in range(dr.block_count(W, H)):
        for pid in range(128):
            by, bx = divmod(block, bw)
            oy, ox = divmod(pid, 8)
            x, y = bx * 8 + ox, by * 16 + oy
            if x < W and y < H:
                assert np.array_equal(fb[block * 128 + pid], img[y, x])
    assert np.array_equal(dr.blockmajor_to_image(fb, W, H), img)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No CPU fallback: without the built library every entry into the API raises."""
    monkeypatch.setattr(dr, "_lib", None)
    monkeypatch.setattr(dr, "LIB_PATH", tmp_path / "libdumbray_gb300.so")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        dr.lib()
    with pytest.raises(RuntimeError, match="missing"):
        dr.Scene(np.zeros((1, 3, 3), np.float32), materials=[dr.lambert()])
    with pytest.raises(RuntimeError, match="missing"):
        dr.Renderer()


def test_exceptions_do_not_cross_the_c_abi():
    """Host allocation failures inside an entry point come back as status codes (no std::terminate):
    dr_image_write_png sizes its row buffer from width x height before it reads a pixel."""
    L = dr.lib()
    px = np.zeros(16, np.float32)
    fn = L.dr_image_write_png
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p]
    assert fn(px.ctypes.data, 1 << 30, 1 << 30, b"never-written.png") == dr.DR_E_NOMEM
    assert L.dr_last_error() == b"dr_image_write_png: out of host memory"
    assert fn(px.ctypes.data, 0x7FFFFFFF, 0x7FFFFFFF, b"never-written.png") == dr.DR_E_STATE
    assert L.dr_last_error().startswith(b"dr_image_write_png: ")
