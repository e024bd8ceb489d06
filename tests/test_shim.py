"""The reference-side drop-in GB300Renderer (tests/shim/GB300Renderer.cu), compiled against the
reference sources into one shared object with the reference's own objects (as inside a DumbRay
build) and linked with this library.

CPU: it compiles, links with no undefined symbol, exports the harness entry points, and its set-up
fails with NULL (no crash) where there is no GPU.
GPU: renderBlocksGPU (BlockRenderer.cuh:43-44) on a device BlockBasedFrameBuffer<8,16> replica
writes the same pixels as dr_render_blocks on the same inputs - the scene converted from the
reference objects (materials, lights, textures, texture corners through their stored state), the
camera from the reference lens and transform - read back through the reference's own
FrameBuffer::updateHostBlocks; two worker threads on their own streams over disjoint block ranges
give the one-thread frame."""
import ctypes
import subprocess
import sys
import threading
from pathlib import Path

import numpy as np
import pytest

import dumbray_gb300 as dr
import _oracle as O

ROOT = Path(__file__).resolve().parent.parent
SHIM = ROOT / "tests" / "shim"
LIB = SHIM / "_build" / "libgb300shim.so"
GOLD = ROOT / "tests" / "golden"
sys.path.insert(0, str(GOLD))
from make_golden import render_scene, texture_scene  # noqa: E402

needs_ref = pytest.mark.skipif(not O.reference_available(), reason="reference library not built here")
vp, ci = ctypes.c_void_p, ctypes.c_int

_lib = None


def shim():
    global _lib
    if _lib is None:
        r = subprocess.run(["bash", str(SHIM / "build_shim.sh")], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        L = ctypes.CDLL(str(LIB))
        L.dshim_create.restype = vp
        L.dshim_create.argtypes = [vp, ci, ci, ci, ci, ci, ci, ci, ctypes.c_uint]
        L.dshim_render.restype = ci
        L.dshim_render.argtypes = [vp, ci, ci, ci, vp]
        L.dshim_read.restype = ci
        L.dshim_read.argtypes = [vp, ci, ci, vp]
        L.dshim_camera.restype = ci
        L.dshim_camera.argtypes = [vp, vp]
        L.dshim_error.restype = ctypes.c_char_p
        L.dshim_error.argtypes = [vp]
        L.dshim_destroy.argtypes = [vp]
        L.dref_scene_destroy.argtypes = [vp]
        L.dshim_set_tight_octree.argtypes = [vp, ci]
        _lib = L
    return _lib


class RefScene:
    """A reference TriScene + camera built through the reference's constructors (dref_scene_create_uv of
    the reference objects inside the shim's own shared object)."""

    def __init__(self, tris, mat, mats, lights, cam, uv=None, textures=()):
        L = shim()
        self.t = np.ascontiguousarray(tris, np.float32)
        self.m = np.ascontiguousarray(mat, np.int32)
        self.mrec = np.ascontiguousarray(np.stack([O.ref_material_record(x) for x in mats]))
        self.lrec = np.ascontiguousarray(np.stack([O.ref_light_record(x) for x in lights]))
        self.crec = O.ref_camera_record(cam)
        self.uv = None if uv is None else np.ascontiguousarray(uv, np.float32).reshape(-1, 3, 2)
        L.dref_scene_create_uv.restype = vp
        L.dref_scene_create_uv.argtypes = [vp, vp, vp, vp, ci, vp, ci, vp, ci, vp]
        self.h = L.dref_scene_create_uv(self.t.ctypes.data, None, None if self.uv is None else self.uv.ctypes.data,
                                        self.m.ctypes.data, len(self.t), self.mrec.ctypes.data, len(self.mrec),
                                        self.lrec.ctypes.data, len(self.lrec), self.crec.ctypes.data)
        if textures:
            self.imgs = [np.ascontiguousarray(x, np.float32) for x, _ in textures]
            whf = np.array([[im.shape[1], im.shape[0], int(f)] for im, (_, f) in zip(self.imgs, textures)], np.int32)
            ptrs = (ctypes.c_void_p * len(self.imgs))(*[im.ctypes.data for im in self.imgs])
            L.dref_scene_set_textures.argtypes = [vp, ci, vp, vp]
            L.dref_scene_set_textures(self.h, len(self.imgs), whf.ctypes.data, ptrs)

    def close(self):
        if self.h:
            shim().dref_scene_destroy(self.h)
            self.h = None


@needs_ref
def test_shim_builds_links_and_exports():
    L = shim()
    for name in ("dshim_create", "dshim_render", "dshim_read", "dshim_camera", "dshim_error", "dshim_destroy"):
        assert hasattr(L, name)
    out = subprocess.run(["nm", "-DC", str(LIB)], capture_output=True, text=True).stdout
    assert "GB300Renderer::renderBlocksGPU" in out and "DumbRenderer::renderBlocksCPU" in out


@needs_ref
def test_shim_set_up_fails_cleanly_without_a_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    tris, mat, mats, lights, cam = render_scene("diffuse")
    rs = RefScene(tris, mat, mats, lights, cam)
    assert shim().dshim_create(rs.h, 32, 32, 1, 1, 2, 1, 0, 0) is None
    rs.close()


def _scenes():
    out = {}
    for kind in ("diffuse", "metal", "ss", "fresnel", "default", "spot", "spot_open"):
        tris, mat, mats, lights, cam = render_scene(kind)
        out[kind] = (tris, mat, mats, lights, cam, None, ())
    tris, mat, mats, lights, cam = render_scene("diffuse")
    seg = dr.camera(dr.LENS_SPHERICAL_SEGMENT, position=(0.0, 0.0, -0.95), angle=(70.0, 50.0), focal_distance=2.0,
                    softness=0.01, filter=(1.0, 0.9, 0.8))
    out["segment_lens"] = (tris, mat, mats, lights, seg, None, ())
    out["perspective_lens"] = (tris, mat, mats, lights, dr.camera(dr.LENS_DEFAULT_PERSPECTIVE, position=(0.0, 0.0, -0.95),
                                                                 angle=55.0), None, ())
    for kind in ("tex_normal", "tex_alpha"):
        tris, mat, mats, lights, cam, uv, textures = texture_scene(kind)
        out[kind] = (tris, mat, mats, lights, cam, uv, textures)
    return out


SCENES = _scenes()


def _direct(sc_args, cam, W, H, fsaa, bounces, seed, cuda, box_epsilon=0.0):
    import torch
    tris, mat, mats, lights, _, uv, textures = sc_args
    sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights, box_epsilon=box_epsilon)
    if textures:
        sc.set_textures(textures, uv)
    fb = dr.new_frame_buffer(W, H, cuda)
    r = dr.Renderer(1 << 16)
    p = dr.render_params(W, H, dr.MODE_REFERENCE, samples=fsaa, max_bounces=bounces, iteration=0, seed=seed)
    r.render_blocks(sc, cam, fb, 0, dr.block_count(W, H), p)
    torch.cuda.synchronize()
    out = fb.cpu().numpy()
    r.close()
    sc.close()
    return out


def _same(a, b, tol_rel=2e-3, max_bad=0.002):
    a = a[:, :3].astype(np.float64)
    b = b[:, :3].astype(np.float64)
    assert np.isfinite(a).all()
    bad = np.abs(a - b) > tol_rel * np.maximum(np.abs(b), 0.01)
    assert bad.mean() <= max_bad, f"{bad.mean():.5f} of channels differ"
    assert abs(a.mean() - b.mean()) <= 1e-4 * max(abs(b.mean()), 1e-3)


@needs_ref
@pytest.mark.gpu
@pytest.mark.parametrize("kind", list(SCENES))
def test_render_blocks_gpu_matches_direct_call(cuda, kind):
    import torch
    L = shim()
    tris, mat, mats, lights, cam, uv, textures = SCENES[kind]
    rs = RefScene(tris, mat, mats, lights, cam, uv, textures)
    W, H, fsaa, bounces, seed = 40, 36, (2, 2), 3, 9
    h = L.dshim_create(rs.h, W, H, fsaa[0], fsaa[1], bounces, 1, dr.BOXING_HEIGHT, seed)
    assert h, "harness set-up failed"
    try:
        nb = dr.block_count(W, H)
        s = torch.cuda.Stream()
        assert L.dshim_render(h, 0, 0, nb, ctypes.c_void_p(s.cuda_stream)) == 1, L.dshim_error(h)
        got = np.zeros((nb * 128, 4), np.float32)
        assert L.dshim_read(h, 0, nb, got.ctypes.data) == 1
        c = dr.DrCamera()
        assert L.dshim_camera(h, ctypes.byref(c)) == 1
        if cam.lens != dr.LENS_SPHERICAL_SEGMENT:
            # the reference lens's stored focal factor, as the library computes it from the angle
            x = np.float32(0.5) / np.tan(np.float32(cam.angle[0]) / np.float32(2 * 57.29577951308233))
            assert abs(c.lens_x - float(x)) <= 4 * np.spacing(np.float32(x))
        want = _direct(SCENES[kind], c, W, H, fsaa, bounces, seed, cuda)
        # in-image pixels only: neither renderer writes the padding of the last block row, and the
        # reference's host buffer (and so its device replica) starts uninitialised there
        _same(dr.blockmajor_to_image(got, W, H).reshape(-1, 4), dr.blockmajor_to_image(want, W, H).reshape(-1, 4))
        assert float(dr.blockmajor_to_image(got, W, H)[..., :3].mean()) > 0
    finally:
        L.dshim_destroy(h)
        rs.close()


@needs_ref
@pytest.mark.gpu
def test_two_worker_threads_on_disjoint_blocks(cuda):
    """As BlockRenderer runs two GPU worker threads per device, each with its own stream and
    DeviceBlockManager: slots 0 and 1 render alternate block ranges concurrently."""
    import torch
    L = shim()
    tris, mat, mats, lights, cam, uv, textures = SCENES["metal"]
    rs = RefScene(tris, mat, mats, lights, cam)
    W, H = 96, 64
    nb = dr.block_count(W, H)
    ranges = [(a, min(nb, a + 5)) for a in range(0, nb, 5)]

    def frame(threads):
        h = L.dshim_create(rs.h, W, H, 2, 2, 3, 1, dr.BOXING_HEIGHT, 5)
        assert h
        try:
            streams = [torch.cuda.Stream() for _ in range(threads)]
            errs = []

            def work(slot):
                for a, b in ranges[slot::threads]:
                    if L.dshim_render(h, slot, a, b, ctypes.c_void_p(streams[slot].cuda_stream)) != 1:
                        errs.append(L.dshim_error(h))

            ts = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
            for t in ts:
                t.start()
            for t in ts:
                t.join()
            assert not errs, errs
            out = np.zeros((nb * 128, 4), np.float32)
            assert L.dshim_read(h, 0, nb, out.ctypes.data) == 1
            return out
        finally:
            L.dshim_destroy(h)

    one = frame(1)
    two = frame(2)
    _same(two, one)
    rs.close()


@needs_ref
@pytest.mark.gpu
def test_tight_octree_option(cuda):
    """setTightOctree(true): the converted scene takes the physical-mode padding; the frame equals
    dr_render_blocks on a scene built with that padding."""
    import torch
    L = shim()
    tris, mat, mats, lights, cam, uv, textures = SCENES["metal"]
    rs = RefScene(tris, mat, mats, lights, cam)
    W, H = 40, 36
    h = L.dshim_create(rs.h, W, H, 2, 2, 3, 1, dr.BOXING_HEIGHT, 9)
    assert h
    try:
        L.dshim_set_tight_octree(h, 1)
        nb = dr.block_count(W, H)
        s = torch.cuda.Stream()
        assert L.dshim_render(h, 0, 0, nb, ctypes.c_void_p(s.cuda_stream)) == 1, L.dshim_error(h)
        got = np.zeros((nb * 128, 4), np.float32)
        assert L.dshim_read(h, 0, nb, got.ctypes.data) == 1
        c = dr.DrCamera()
        assert L.dshim_camera(h, ctypes.byref(c)) == 1
        want = _direct(SCENES["metal"], c, W, H, (2, 2), 3, 9, cuda, box_epsilon=dr.PHYSICAL_TREE)
        _same(dr.blockmajor_to_image(got, W, H).reshape(-1, 4), dr.blockmajor_to_image(want, W, H).reshape(-1, 4))
    finally:
        L.dshim_destroy(h)
        rs.close()
