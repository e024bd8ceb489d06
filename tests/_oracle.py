"""ctypes bindings of the CPU oracle (oracle/_build/libdroracle.so) and, when it has been built, of
the reference DumbRay host path (oracle/_ref/libdumbref.so).  Test infrastructure only."""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

import dumbray_gb300 as dr

ROOT = Path(__file__).resolve().parent.parent
ORACLE_LIB = ROOT / "oracle" / "_build" / "libdroracle.so"
REF_LIB = ROOT / "oracle" / "_ref" / "libdumbref.so"

_o = None
_r = None
vp, ci = ctypes.c_void_p, ctypes.c_int


def oracle():
    global _o
    if _o is None:
        if not ORACLE_LIB.exists():
            subprocess.run(["bash", str(ROOT / "oracle" / "build_oracle.sh")], check=True, capture_output=True)
        L = ctypes.CDLL(str(ORACLE_LIB))
        L.dro_scene_create.restype = vp
        L.dro_scene_create.argtypes = [vp, vp, vp, ci, vp, ci, vp, ci, ci, ci, ci]
        L.dro_scene_set_triangle_params.argtypes = [vp, vp, vp, vp]
        L.dro_scene_freeze_sampling.argtypes = [vp, ci]
        L.dro_scene_set_textures.argtypes = [vp, vp, ci, vp]
        L.dro_scene_destroy.argtypes = [vp]
        L.dro_node_count.restype = ctypes.c_longlong
        L.dro_node_count.argtypes = [vp]
        L.dro_tree_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                                     ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ci)]
        L.dro_tree_canonical.restype = ctypes.c_longlong
        L.dro_tree_canonical.argtypes = [vp, vp, vp, vp, ctypes.c_longlong, ctypes.c_longlong]
        L.dro_cast.argtypes = [vp, vp, vp, vp, ci, ci, ci, vp, vp, vp, vp]
        L.dro_render_blocks.argtypes = [vp, vp, vp, vp, ci, ci, ci]
        L.dro_rng_u32.restype = ctypes.c_uint32
        L.dro_rng_u32.argtypes = [ctypes.c_uint32] * 5
        _o = L
    return _o


def reference_available() -> bool:
    return REF_LIB.exists()


def reference():
    global _r
    if _r is None:
        L = ctypes.CDLL(str(REF_LIB))
        L.dref_octree_create.restype = vp
        L.dref_octree_create.argtypes = [vp, vp, vp, ci]
        L.dref_octree_node_count.restype = ci
        L.dref_octree_node_count.argtypes = [vp]
        L.dref_octree_destroy.argtypes = [vp]
        L.dref_octree_cast.argtypes = [vp, vp, vp, ci, ci, ci, vp, vp]
        L.dref_scene_create.restype = vp
        L.dref_scene_create.argtypes = [vp, vp, vp, ci, vp, ci, vp, ci, vp]
        L.dref_scene_destroy.argtypes = [vp]
        L.dref_render.restype = ctypes.c_double
        L.dref_render.argtypes = [vp, ci, ci, ci, ci, ci, ci, ci, ci, vp]
        if hasattr(L, "dref_obj_read"):
            L.dref_obj_read.restype = vp
            L.dref_obj_read.argtypes = [ctypes.c_char_p]
            L.dref_obj_meshes.restype = ci
            L.dref_obj_meshes.argtypes = [vp]
            L.dref_obj_names.restype = ci
            L.dref_obj_names.argtypes = [vp]
            L.dref_obj_name.restype = ctypes.c_char_p
            L.dref_obj_name.argtypes = [vp, ci]
            L.dref_obj_triangles.restype = ci
            L.dref_obj_triangles.argtypes = [vp, ci, vp, vp, vp]
            L.dref_obj_free.argtypes = [vp]
        if hasattr(L, "dref_save_png"):
            L.dref_save_png.restype = ci
            L.dref_save_png.argtypes = [vp, ci, ci, ctypes.c_char_p]
        if hasattr(L, "dref_dumb_load"):
            L.dref_dumb_load.restype = vp
            L.dref_dumb_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ci]
            L.dref_dumb_free.argtypes = [vp]
            L.dref_dumb_counts.argtypes = [vp, vp]
            L.dref_dumb_geometry.argtypes = [vp, vp, vp, vp]
            L.dref_dumb_material.argtypes = [vp, ci, vp]
            L.dref_dumb_light.argtypes = [vp, ci, vp]
            L.dref_dumb_camera.argtypes = [vp, vp]
            L.dref_dumb_settings.argtypes = [vp, vp]
            L.dref_record_material.argtypes = [vp, vp]
            L.dref_record_light.argtypes = [vp, vp]
            L.dref_record_lens.argtypes = [vp, vp]
            L.dref_dumb_render.restype = ctypes.c_double
            L.dref_dumb_render.argtypes = [vp, ci, ci, ci, ci, vp]
        _r = L
    return _r


class OracleScene:
    def __init__(self, tris, normals=None, mat_id=None, materials=(), lights=(), threads=8):
        L = oracle()
        self.tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 3, 3)
        self.nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32)
        self.mat = None if mat_id is None else np.ascontiguousarray(mat_id, dtype=np.int32)
        mats = list(materials)
        lts = list(lights)
        self._marr = (dr.DrMaterial * max(1, len(mats)))(*mats)
        self._larr = (dr.DrLight * max(1, len(lts)))(*lts)
        self.h = L.dro_scene_create(self.tris.ctypes.data, None if self.nrm is None else self.nrm.ctypes.data,
                                    None if self.mat is None else self.mat.ctypes.data, len(self.tris),
                                    ctypes.addressof(self._marr), len(mats), ctypes.addressof(self._larr), len(lts), 0, 0,
                                    threads)

    def set_triangle_params(self, albedo=None, emission=None, roughness=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float32) for a in (albedo, emission, roughness)]
        oracle().dro_scene_set_triangle_params(self.h, *[None if a is None else a.ctypes.data for a in arrs])
        self._keep = arrs

    def freeze_sampling(self, freeze=True):
        """Light selection keeps the current per-triangle emission power (as the device library's
        sampling tables do when parameters are written in place), or follows it again."""
        oracle().dro_scene_freeze_sampling(self.h, 1 if freeze else 0)

    def set_textures(self, textures, uv=None):
        """As dumbray_gb300.Scene.set_textures."""
        self._tex = [np.ascontiguousarray(t, dtype=np.float32) for t, _ in textures]
        arr = (dr.DrTexture * max(1, len(self._tex)))()
        for i, (img, (_, filt)) in enumerate(zip(self._tex, textures)):
            arr[i].width, arr[i].height, arr[i].filtering = img.shape[1], img.shape[0], int(filt)
            arr[i].rgba = img.ctypes.data
        self._uv = None if uv is None else np.ascontiguousarray(uv, dtype=np.float32).reshape(-1, 3, 2)
        oracle().dro_scene_set_textures(self.h, ctypes.addressof(arr), len(self._tex),
                                        None if self._uv is None else self._uv.ctypes.data)

    def node_count(self):
        return oracle().dro_node_count(self.h)

    def stats(self):
        n, l, r = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        d = ctypes.c_int()
        oracle().dro_tree_stats(self.h, ctypes.byref(n), ctypes.byref(l), ctypes.byref(r), ctypes.byref(d))
        return dict(nodes=n.value, leaves=l.value, refs=r.value, depth=d.value)

    def canonical(self):
        s = self.stats()
        box = np.zeros((s["nodes"], 6), np.float32)
        cnt = np.zeros(s["nodes"], np.int32)
        tri = np.zeros(max(1, s["refs"]), np.int32)
        k = oracle().dro_tree_canonical(self.h, box.ctypes.data, cnt.ctypes.data, tri.ctypes.data, s["nodes"], s["refs"])
        return box[:k], cnt[:k], tri[: s["refs"]]

    def cast(self, o, d, ignore=None, cull=True, threads=8):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = len(o)
        idx = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        nb = np.zeros(n, np.int32)
        nt = np.zeros(n, np.int32)
        ig = None if ignore is None else np.ascontiguousarray(ignore, np.int32)
        oracle().dro_cast(self.h, o.ctypes.data, d.ctypes.data, None if ig is None else ig.ctypes.data, n, 1 if cull else 0,
                          threads, idx.ctypes.data, t.ctypes.data, nb.ctypes.data, nt.ctypes.data)
        return idx, t, nb, nt

    def render_blocks(self, cam, params, fb=None, start=0, end=None, threads=8):
        nb = dr.block_count(params.width, params.height)
        end = nb if end is None else end
        if fb is None:
            fb = np.zeros((nb * dr.BLOCK_SIZE, 4), np.float32)
        oracle().dro_render_blocks(self.h, ctypes.byref(cam), ctypes.byref(params), fb.ctypes.data, start, end, threads)
        return fb

    def __del__(self):
        try:
            oracle().dro_scene_destroy(self.h)
        except Exception:
            pass


def ref_cast(tris, o, d, cull=True, threads=8):
    """The reference's own Octree::cast (oracle/_ref)."""
    L = reference()
    tris = np.ascontiguousarray(tris, np.float32)
    h = L.dref_octree_create(tris.ctypes.data, None, None, len(tris))
    try:
        n = len(o)
        idx = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        L.dref_octree_cast(h, o.ctypes.data, d.ctypes.data, n, 1 if cull else 0, threads, idx.ctypes.data, t.ctypes.data)
        return idx, t, L.dref_octree_node_count(h)
    finally:
        L.dref_octree_destroy(h)


def ref_material_record(m: dr.DrMaterial) -> np.ndarray:
    """Constructor record (48 floats) for oracle/ref_driver.cu's ref_material."""
    r = np.zeros(48, np.float32)
    r[16:20] = list(m.texture)
    r[20:28] = [m.tiling[k][j] for k in range(4) for j in range(2)]
    r[28:36] = [m.offset[k][j] for k in range(4) for j in range(2)]
    r[36:39] = list(m.normal_color)
    r[39] = m.alpha_threshold
    if m.type == dr.MAT_DUMB_BASED:
        r[:9] = [0, *m.fresnel, m.specular, *m.color, m.metal]
    elif m.type == dr.MAT_SIMPLE_STOCHASTIC:
        r[:7] = [1, *m.color, m.diffuse, m.smoothness, m.shininess]
    elif m.type == dr.MAT_FRESNEL:
        r[:4] = [2, *m.color]
    elif m.type == dr.MAT_DEFAULT:
        r[:7] = [3, *m.color, m.diffuse, m.smoothness, m.shininess]
    else:
        raise ValueError("material has no reference counterpart")
    return r


def ref_light_record(l: dr.DrLight) -> np.ndarray:
    """Constructor record for oracle/ref_driver.cu's ref_light."""
    r = np.zeros(16, np.float32)
    if l.type == dr.LIGHT_SPHERICAL:
        r[:8] = [0, *l.color, *l.position, l.radius]
    elif l.type == dr.LIGHT_SOFT_DIRECTIONAL:
        r[:9] = [1, *l.color, *l.direction, l.distance, l.softness]
    elif l.type == dr.LIGHT_DIRECTIONAL:
        r[:8] = [2, *l.color, *l.direction, l.distance]
    else:
        flags = (1 if l.emit_from_sphere else 0) | (2 if l.cast_shadows else 0) | (int(l.samples) << 2)
        r[:16] = [3, *l.color, *l.position, *l.direction, l.luminosity, l.hotspot_angle, l.falloff_angle,
                  l.falloff_power, l.emitter_size, flags]
    return r


def ref_camera_record(c: dr.DrCamera) -> np.ndarray:
    """Only identity camera orientation is expressible here (reference Transform with zero Euler angles)."""
    assert tuple(c.right) == (1.0, 0.0, 0.0) and tuple(c.up) == (0.0, 1.0, 0.0) and tuple(c.forward) == (0.0, 0.0, 1.0)
    r = np.zeros(16, np.float32)
    r[0] = c.lens
    r[1], r[2] = c.angle[0], c.angle[1]
    r[3], r[4] = c.focal_distance, c.softness
    r[5:8] = list(c.filter)
    r[8:11] = list(c.position)
    return r


def ref_render(tris, mat_id, materials, lights, cam, width, height, fsaa=(1, 1), max_bounces=2, cull=True, iterations=1,
               threads=8, normals=None, uv=None, textures=()):
    """Reference DumbRenderer on CPU threads; returns (row-major RGBA image, seconds).  ``uv``: corner
    texture coordinates [n, 3, 2]; ``textures``: [(rgba float [h, w, 4], filtering)]."""
    L = reference()
    tris = np.ascontiguousarray(tris, np.float32)
    mat = np.ascontiguousarray(mat_id, np.int32)
    mrec = np.ascontiguousarray(np.stack([ref_material_record(m) for m in materials]))
    lrec = np.ascontiguousarray(np.stack([ref_light_record(l) for l in lights]))
    crec = ref_camera_record(cam)
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
    uvs = None if uv is None else np.ascontiguousarray(uv, np.float32).reshape(-1, 3, 2)
    L.dref_scene_create_uv.restype = vp
    L.dref_scene_create_uv.argtypes = [vp, vp, vp, vp, ci, vp, ci, vp, ci, vp]
    h = L.dref_scene_create_uv(tris.ctypes.data, None if nrm is None else nrm.ctypes.data,
                               None if uvs is None else uvs.ctypes.data, mat.ctypes.data, len(tris),
                               mrec.ctypes.data, len(mrec), lrec.ctypes.data, len(lrec), crec.ctypes.data)
    if textures:
        imgs = [np.ascontiguousarray(t, np.float32) for t, _ in textures]
        whf = np.array([[im.shape[1], im.shape[0], int(f)] for im, (_, f) in zip(imgs, textures)], np.int32)
        ptrs = (ctypes.c_void_p * len(imgs))(*[im.ctypes.data for im in imgs])
        L.dref_scene_set_textures.argtypes = [vp, ci, vp, vp]
        L.dref_scene_set_textures(h, len(imgs), whf.ctypes.data, ptrs)
    try:
        img = np.zeros((height, width, 4), np.float32)
        sec = L.dref_render(h, width, height, fsaa[0], fsaa[1], max_bounces, 1 if cull else 0, iterations, threads,
                            img.ctypes.data)
        return img, sec
    finally:
        L.dref_scene_destroy(h)


def ref_read_obj(path):
    """The reference's MeshReader::readObj + bake (oracle/_ref): None if it fails, else
    (names, [(xyz, nrm, uv) per mesh])."""
    L = reference()
    h = L.dref_obj_read(str(path).encode())
    if not h:
        return None
    try:
        names = [L.dref_obj_name(h, i).decode(errors="replace") for i in range(L.dref_obj_names(h))]
        meshes = []
        for i in range(L.dref_obj_meshes(h)):
            n = L.dref_obj_triangles(h, i, None, None, None)
            arrs = [np.zeros((n, 3, 3), np.float32) for _ in range(3)]
            L.dref_obj_triangles(h, i, *(a.ctypes.data for a in arrs))
            meshes.append(tuple(arrs))
        return names, meshes
    finally:
        L.dref_obj_free(h)


# ---- scene files through the reference's own loader (DumbRenderContext::fromFile) ----------------

class RefSceneFileError(RuntimeError):
    pass


def _ref_dumb_open(path):
    L = reference()
    err = ctypes.create_string_buffer(8192)
    h = L.dref_dumb_load(str(path).encode(), err, len(err))
    if not h:
        raise RefSceneFileError(err.value.decode(errors="replace"))
    return L, h


def ref_scene_file_dump(path):
    """What the reference's loader built, as canonical float dumps: geometry (xyz, normals, material
    ids in push order), per-material / per-light dumps, camera (lens + transform) and settings."""
    L, h = _ref_dumb_open(path)
    try:
        c = np.zeros(3, np.int32)
        L.dref_dumb_counts(h, c.ctypes.data)
        n = int(c[0])
        xyz = np.zeros((n, 9), np.float32)
        nrm = np.zeros((n, 9), np.float32)
        mat = np.zeros(n, np.int32)
        L.dref_dumb_geometry(h, xyz.ctypes.data, nrm.ctypes.data, mat.ctypes.data)
        mats = np.zeros((int(c[1]), 48), np.float32)
        for i in range(int(c[1])):
            L.dref_dumb_material(h, i, mats[i].ctypes.data)
        lights = np.zeros((int(c[2]), 16), np.float32)
        for i in range(int(c[2])):
            L.dref_dumb_light(h, i, lights[i].ctypes.data)
        cam = np.zeros(32, np.float32)
        L.dref_dumb_camera(h, cam.ctypes.data)
        settings = np.zeros(8, np.int32)
        L.dref_dumb_settings(h, settings.ctypes.data)
        uv = np.zeros((n, 6), np.float32)
        L.dref_dumb_texcoords.argtypes = [vp, vp]
        L.dref_dumb_texcoords(h, uv.ctypes.data)
        L.dref_dumb_texture_count.restype = ci
        L.dref_dumb_texture_count.argtypes = [vp]
        L.dref_dumb_texture.argtypes = [vp, ci, vp, vp]
        textures = []
        for i in range(L.dref_dumb_texture_count(h)):
            whf = np.zeros(3, np.int32)
            L.dref_dumb_texture(h, i, whf.ctypes.data, None)
            img = np.zeros((whf[1], whf[0], 4), np.float32)
            L.dref_dumb_texture(h, i, whf.ctypes.data, img.ctypes.data)
            textures.append((img, int(whf[2])))
        return dict(xyz=xyz, nrm=nrm, mat=mat, materials=mats, lights=lights, camera=cam[:29], settings=settings[:6],
                    uv=uv, textures=textures)
    finally:
        L.dref_dumb_free(h)


def scene_file_dump(f):
    """The same dumps for a dumbray_gb300.SceneFile: materials, lights and the lens go through the
    reference's constructors (dref_record_*), the transform fields are the camera's own."""
    L = reference()
    n = len(f.tris)
    mats = np.zeros((len(f.materials), 48), np.float32)
    for i, m in enumerate(f.materials):
        rec = ref_material_record(m)
        L.dref_record_material(rec.ctypes.data, mats[i].ctypes.data)
    lights = np.zeros((len(f.lights), 16), np.float32)
    for i, l in enumerate(f.lights):
        rec = ref_light_record(l)
        L.dref_record_light(rec.ctypes.data, lights[i].ctypes.data)
    c = f.camera
    crec = np.zeros(16, np.float32)
    crec[0] = c.lens
    crec[1:3] = list(c.angle)
    crec[3], crec[4] = c.focal_distance, c.softness
    crec[5:8] = list(c.filter)
    cam = np.zeros(32, np.float32)
    L.dref_record_lens(crec.ctypes.data, cam.ctypes.data)
    cam[8:11], cam[11:14], cam[14:17] = list(c.right), list(c.up), list(c.forward)
    cam[17:20], cam[20:23], cam[23:26] = list(c.row_x), list(c.row_y), list(c.row_z)
    cam[26:29] = list(c.position)
    p = f.params
    settings = np.array([p.boxing, p.max_bounces, p.samples_x, p.samples_y, 1, p.cull_backfaces], np.int32)
    return dict(xyz=f.tris.reshape(n, 9), nrm=f.normals.reshape(n, 9), mat=f.mat_id, materials=mats, lights=lights,
                camera=cam[:29], settings=settings, uv=f.uv.reshape(n, 6), textures=list(f.textures))


def ref_dumb_render(path, width, height, iterations, threads=8):
    """Reference DumbRenderer render of a scene file loaded by the reference (its camera and renderer
    settings); returns (row-major RGBA image, seconds)."""
    L, h = _ref_dumb_open(path)
    try:
        img = np.zeros((height, width, 4), np.float32)
        sec = L.dref_dumb_render(h, width, height, iterations, threads, img.ctypes.data)
        if sec < 0:
            raise RefSceneFileError("reference render failed")
        return img, sec
    finally:
        L.dref_dumb_free(h)
