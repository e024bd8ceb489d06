"""Mutated inputs to the host parsers that read untrusted files: the .dumb scene loader (Dson text,
includes), the OBJ reader behind it and the PNG texture decoder.  Seeded mutations of the committed
scene-file fixtures (truncations, deleted / duplicated spans, random bytes, inserted tokens such as
huge numbers or stray OBJ records; PNG chunks re-checksummed so the mutations reach inflate and
unfiltering) must load or fail with a status code and a message — never crash or hang."""
import ctypes
import random
import shutil
import struct
import zlib
from pathlib import Path

import pytest

import dumbray_gb300 as dr

GOLD = Path(__file__).resolve().parent / "golden"
TOKENS = list('{}[]",:-.0123456789eE ') + ["1e30", "-1e30", "nan", "inf", "99999999999", "-7", '""', "[]", "{}", "\n",
                                           "f 1 2 3", "v 1 2 3", "vt 0 0", "g x", "usemtl a"]
ALLOWED = {dr.DR_OK, dr.DR_E_ARG, dr.DR_E_NOMEM, dr.DR_E_STATE}


def _mutate(b: bytes, rng: random.Random) -> bytes:
    b = bytearray(b)
    if not b:
        return bytes(b)
    k, i = rng.randrange(6), rng.randrange(len(b))
    if k == 0:
        return bytes(b[:i])
    if k == 1:
        del b[i:min(len(b), i + rng.randrange(1, 40))]
        return bytes(b)
    if k == 2:
        j = min(len(b), i + rng.randrange(1, 80))
        return bytes(b[:j] + b[i:j] + b[j:])
    if k == 3:
        b[i] = rng.randrange(256)
        return bytes(b)
    t = rng.choice(TOKENS).encode()
    if k == 4:
        return bytes(b[:i] + t + b[i:])
    return bytes(b[:i] + t + b[min(len(b), i + rng.randrange(1, 8)):])


def _fix_crcs(b: bytes) -> bytes:
    if len(b) < 8:
        return b
    out, i = bytearray(b[:8]), 8
    while i + 12 <= len(b):
        n = struct.unpack(">I", b[i:i + 4])[0]
        if i + 12 + n > len(b):
            break
        kind, data = b[i + 4:i + 8], b[i + 8:i + 8 + n]
        out += b[i:i + 8] + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)
        i += 12 + n
    return bytes(out + b[i:])


def _load(path: Path) -> int:
    L = dr.lib()
    h = ctypes.c_void_p()
    s = L.dr_scene_file_load(str(path).encode(), ctypes.byref(h))
    assert s in ALLOWED, (s, L.dr_last_error())
    if s == dr.DR_OK:
        counts = (ctypes.c_int32 * 8)()
        assert L.dr_scene_file_counts(h, counts) == dr.DR_OK
        L.dr_scene_file_destroy(h)
    else:
        assert L.dr_last_error()
    return s


@pytest.mark.timeout(300)
@pytest.mark.parametrize("fixture,files", [("scene_file", ["scene.dumb", "materials.dumb", "props.obj"]),
                                           ("scene_file_tex", ["scene.dumb", "textured.obj", "checker.png"])])
def test_mutated_scene_files_load_or_fail_cleanly(tmp_path, fixture, files):
    rng = random.Random(fixture)
    seen = set()
    for it in range(120):
        work = tmp_path / f"m{it}"
        shutil.copytree(GOLD / fixture, work)
        name = rng.choice(files)
        data = (work / name).read_bytes()
        for _ in range(rng.randrange(1, 4)):
            data = _mutate(data, rng)
        if name.endswith(".png") and rng.random() < 0.7:
            data = _fix_crcs(data)
        (work / name).write_bytes(data)
        seen.add(_load(work / "scene.dumb"))
        shutil.rmtree(work)
    assert dr.DR_E_ARG in seen   # the mutations do reach the error paths
