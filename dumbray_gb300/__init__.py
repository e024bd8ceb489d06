"""dumbray_gb300 - GB300-native (sm_103a) implementation of DumbRay's rendering hot path.

Python host mirror of the C ABI in ``include/dr_api.h``.  Every call goes through the native
library ``dumbray_gb300/_build/libdumbray_gb300.so`` (built in-tree by ``dumbray_gb300.build``);
there is no CPU fallback: if the library is missing, importing the API raises.

Interfaces mirrored from the reference (paths relative to the DumbRay checkout):
  * ``Scene``        - TriScene = Octree<Renderable<BakedTriFace>> + materials + lights
                       (__source__/DataStructures/Objects/Scene/Scene.cuh:13-68)
  * ``cast``         - Octree::cast (.../Raycasters/Octree/Octree.impl.cuh:174-212)
  * ``BlockRenderer``- DumbRenderer's renderBlocksGPU and its configuration setters
                       (__source__/DataStructures/Renderers/DumbRenderer/DumbRenderer.cuh:9-64)
  * frame buffer     - BlockBasedFrameBuffer<8,16> layout helpers (BlockBasedFrameBuffer.impl.cuh:108-156)
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from . import scenes  # noqa: F401  (input generators)

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_build" / "libdumbray_gb300.so"

DR_OK, DR_E_ARG, DR_E_CUDA, DR_E_CAPACITY, DR_E_TIMEOUT, DR_E_NOMEM, DR_E_STATE = range(7)
MAT_DUMB_BASED, MAT_SIMPLE_STOCHASTIC, MAT_LAMBERT, MAT_MIRROR, MAT_GLOSSY, MAT_FRESNEL, MAT_DEFAULT = range(7)
LIGHT_SPHERICAL, LIGHT_SOFT_DIRECTIONAL, LIGHT_DIRECTIONAL, LIGHT_SPOTLIGHT = range(4)
LENS_DEFAULT_PERSPECTIVE, LENS_SIMPLE_STOCHASTIC, LENS_SPHERICAL_SEGMENT, LENS_PINHOLE, LENS_FISHEYE, LENS_SPHERICAL = range(6)
MODE_REFERENCE, MODE_PHYSICAL = 0, 1
PHYSICAL_TREE = -1.0   # Scene(box_epsilon=...): octree padding scaled to the scene (physical-mode scenes)
BOXING_HEIGHT, BOXING_WIDTH, BOXING_MIN, BOXING_MAX = range(4)
BLOCK_W, BLOCK_H = 8, 16
BLOCK_SIZE = BLOCK_W * BLOCK_H

_F3 = ctypes.c_float * 3


class DrBuildParams(ctypes.Structure):
    _fields_ = [("max_depth", ctypes.c_int32), ("split_threshold", ctypes.c_int32), ("threads", ctypes.c_int32),
                ("box_epsilon", ctypes.c_float), ("device_build", ctypes.c_int32)]


class DrMaterial(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("color", _F3), ("fresnel", _F3), ("specular", ctypes.c_float),
                ("metal", ctypes.c_float), ("diffuse", ctypes.c_float), ("smoothness", ctypes.c_float),
                ("shininess", ctypes.c_float), ("roughness", ctypes.c_float), ("emission", _F3),
                ("texture", ctypes.c_int32 * 4), ("tiling", (ctypes.c_float * 2) * 4), ("offset", (ctypes.c_float * 2) * 4),
                ("normal_color", _F3), ("alpha_threshold", ctypes.c_float)]


class DrTexture(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("filtering", ctypes.c_int32),
                ("rgba", ctypes.c_void_p)]


TEX_COLOR, TEX_FRESNEL, TEX_NORMAL, TEX_ALPHA = range(4)
FILTER_NONE, FILTER_BILINEAR = 0, 1


def textured(m: "DrMaterial", channel: int, texture: int, tiling=(1.0, 1.0), offset=(0.0, 0.0)) -> "DrMaterial":
    """Gives material ``m`` texture ``texture`` (0-based index into the textures passed to
    Scene.set_textures) on ``channel`` (TEX_COLOR / TEX_FRESNEL / TEX_NORMAL / TEX_ALPHA); sets the
    reference's defaults for the normal-map colour (1, 1, 1) and the alpha threshold (0.5) if unset."""
    m.texture[channel] = texture + 1
    m.tiling[channel][:] = tiling
    m.offset[channel][:] = offset
    if channel == TEX_NORMAL and not any(m.normal_color):
        m.normal_color[:] = (1.0, 1.0, 1.0)
    if channel == TEX_ALPHA and m.alpha_threshold == 0.0:
        m.alpha_threshold = 0.5
    return m


class DrLight(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("color", _F3), ("position", _F3), ("direction", _F3),
                ("radius", ctypes.c_float), ("distance", ctypes.c_float), ("softness", ctypes.c_float),
                ("luminosity", ctypes.c_float), ("hotspot_angle", ctypes.c_float), ("falloff_angle", ctypes.c_float),
                ("falloff_power", ctypes.c_float), ("emitter_size", ctypes.c_float),
                ("emit_from_sphere", ctypes.c_int32), ("cast_shadows", ctypes.c_int32), ("samples", ctypes.c_int32)]


class DrCamera(ctypes.Structure):
    _fields_ = [("lens", ctypes.c_int32), ("angle", ctypes.c_float * 2), ("focal_distance", ctypes.c_float),
                ("softness", ctypes.c_float), ("filter", _F3), ("position", _F3), ("right", _F3), ("up", _F3),
                ("forward", _F3), ("origin_rows", ctypes.c_int32), ("row_x", _F3), ("row_y", _F3), ("row_z", _F3),
                ("lens_x", ctypes.c_float)]


class DrRenderParams(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("samples_x", ctypes.c_int32), ("samples_y", ctypes.c_int32), ("max_bounces", ctypes.c_int32),
                ("cull_backfaces", ctypes.c_int32), ("boxing", ctypes.c_int32), ("iteration", ctypes.c_int32),
                ("seed", ctypes.c_uint32)]


class DrBatchItem(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("camera", DrCamera), ("params", DrRenderParams), ("fb", ctypes.c_void_p),
                ("start_block", ctypes.c_int32), ("end_block", ctypes.c_int32)]


class DumbRayError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"dumbray_gb300 status {status}: {message}")
        self.status = status


_lib = None


PROGRESS_CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_void_p)


def lib() -> ctypes.CDLL:
    """The native library (loaded once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"native library {LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                           "(or python -m dumbray_gb300.build); there is no CPU fallback")
    L = ctypes.CDLL(str(LIB_PATH))
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    P = ctypes.POINTER
    L.dr_last_error.restype = ctypes.c_char_p
    L.dr_version.restype = i32
    L.dr_block_count.restype = i32
    L.dr_block_count.argtypes = [i32, i32]
    L.dr_scene_create.restype = i32
    L.dr_scene_create.argtypes = [vp, vp, vp, i32, vp, i32, vp, i32, vp, P(vp)]
    L.dr_scene_set_triangle_params.restype = i32
    L.dr_scene_set_triangle_params.argtypes = [vp, vp, vp, vp]
    L.dr_scene_triangle_params_device.restype = i32
    L.dr_scene_triangle_params_device.argtypes = [vp, P(vp), P(vp)]
    L.dr_scene_stats.restype = i32
    L.dr_scene_stats.argtypes = [vp, P(i64), P(i64), P(i64), P(i32)]
    L.dr_scene_export_tree.restype = i32
    L.dr_scene_export_tree.argtypes = [vp, vp, vp, vp, vp]
    L.dr_scene_destroy.restype = None
    L.dr_scene_destroy.argtypes = [vp]
    L.dr_octree_create_host.restype = i32
    L.dr_octree_create_host.argtypes = [vp, i32, vp, P(vp)]
    L.dr_octree_stats.restype = i32
    L.dr_octree_stats.argtypes = [vp, P(i64), P(i64), P(i64), P(i32)]
    L.dr_octree_export.restype = i32
    L.dr_octree_export.argtypes = [vp, vp, vp, vp, vp]
    L.dr_octree_group_planes.restype = i32
    L.dr_octree_group_planes.argtypes = [vp, vp, vp]
    L.dr_octree_destroy.restype = None
    L.dr_octree_destroy.argtypes = [vp]
    L.dr_cast.restype = i32
    L.dr_cast.argtypes = [vp, vp, vp, vp, i32, i32, vp, vp, vp]
    L.dr_cast_counted.restype = i32
    L.dr_cast_counted.argtypes = [vp, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp]
    L.dr_renderer_create.restype = i32
    L.dr_renderer_create.argtypes = [i32, P(vp)]
    L.dr_renderer_destroy.restype = None
    L.dr_renderer_destroy.argtypes = [vp]
    L.dr_renderer_launch_count.restype = i64
    L.dr_renderer_launch_count.argtypes = [vp]
    L.dr_renderer_set_profiling.restype = i32
    L.dr_renderer_set_profiling.argtypes = [vp, i32]
    L.dr_renderer_kernel_times.restype = i32
    L.dr_renderer_kernel_times.argtypes = [vp, vp, vp]
    L.dr_renderer_kernel_busy.restype = i32
    L.dr_renderer_kernel_busy.argtypes = [vp, vp]
    L.dr_renderer_set_lanes.restype = i32
    L.dr_renderer_set_lanes.argtypes = [vp, i32]
    L.dr_renderer_lanes.restype = i32
    L.dr_renderer_lanes.argtypes = [vp]
    L.dr_renderer_set_block_shape.restype = i32
    L.dr_renderer_set_block_shape.argtypes = [vp, i32]
    L.dr_renderer_block_shape.restype = i32
    L.dr_renderer_block_shape.argtypes = [vp]
    L.dr_renderer_set_counting.restype = i32
    L.dr_renderer_set_counting.argtypes = [vp, i32]
    L.dr_renderer_counters.restype = i32
    L.dr_renderer_counters.argtypes = [vp, vp]
    L.dr_renderer_wave_counts.restype = i32
    L.dr_renderer_wave_counts.argtypes = [vp, vp, vp, i32]
    L.dr_render_adjoint.restype = i32
    L.dr_render_adjoint.argtypes = [vp, vp, vp, vp, i32, i32, vp, vp, vp, vp]
    L.dr_batch_create.restype = i32
    L.dr_batch_create.argtypes = [vp, i32, P(vp)]
    L.dr_batch_set_iteration.restype = i32
    L.dr_batch_set_iteration.argtypes = [vp, i32]
    L.dr_batch_render.restype = i32
    L.dr_batch_render.argtypes = [vp, vp, i32, vp]
    L.dr_batch_paths.restype = i64
    L.dr_batch_paths.argtypes = [vp]
    L.dr_batch_destroy.restype = None
    L.dr_batch_destroy.argtypes = [vp]
    L.dr_render_blocks.restype = i32
    L.dr_render_blocks.argtypes = [vp, vp, vp, vp, i32, i32, vp, vp]
    for fn in ("dr_image_from_blocks", "dr_image_to_rgba8"):
        getattr(L, fn).restype = i32
        getattr(L, fn).argtypes = [vp, i32, i32, vp]
    for fn in ("dr_image_write_png", "dr_image_write_pfm"):
        getattr(L, fn).restype = i32
        getattr(L, fn).argtypes = [vp, i32, i32, ctypes.c_char_p]
    L.dr_obj_read.restype = i32
    L.dr_obj_read.argtypes = [ctypes.c_char_p, P(vp)]
    L.dr_mesh_file_objects.restype = i32
    L.dr_mesh_file_objects.argtypes = [vp]
    L.dr_mesh_file_object_name.restype = ctypes.c_char_p
    L.dr_mesh_file_object_name.argtypes = [vp, i32]
    L.dr_mesh_file_object_triangles.restype = i32
    L.dr_mesh_file_object_triangles.argtypes = [vp, i32]
    L.dr_mesh_file_object_data.restype = i32
    L.dr_mesh_file_object_data.argtypes = [vp, i32, vp, vp, vp]
    L.dr_mesh_file_destroy.restype = None
    L.dr_mesh_file_destroy.argtypes = [vp]
    L.dr_png_read.restype = i32
    L.dr_png_read.argtypes = [ctypes.c_char_p, P(i32), P(i32), vp]
    L.dr_scene_set_textures.restype = i32
    L.dr_scene_set_textures.argtypes = [vp, vp, i32, vp]
    L.dr_scene_file_load.restype = i32
    L.dr_scene_file_load.argtypes = [ctypes.c_char_p, P(vp)]
    L.dr_scene_file_counts.restype = i32
    L.dr_scene_file_counts.argtypes = [vp, vp]
    L.dr_scene_file_geometry.restype = i32
    L.dr_scene_file_geometry.argtypes = [vp, vp, vp, vp]
    L.dr_scene_file_materials.restype = i32
    L.dr_scene_file_materials.argtypes = [vp, vp]
    L.dr_scene_file_lights.restype = i32
    L.dr_scene_file_lights.argtypes = [vp, vp]
    L.dr_scene_file_camera.restype = i32
    L.dr_scene_file_camera.argtypes = [vp, vp]
    L.dr_scene_file_render_params.restype = i32
    L.dr_scene_file_render_params.argtypes = [vp, vp]
    L.dr_scene_file_textures.restype = i32
    L.dr_scene_file_textures.argtypes = [vp]
    L.dr_scene_file_texture.restype = i32
    L.dr_scene_file_texture.argtypes = [vp, i32, P(i32), P(i32), P(i32), vp]
    L.dr_scene_file_texcoords.restype = i32
    L.dr_scene_file_texcoords.argtypes = [vp, vp]
    L.dr_scene_file_create_scene.restype = i32
    L.dr_scene_file_create_scene.argtypes = [vp, vp, P(vp)]
    L.dr_scene_file_destroy.restype = None
    L.dr_scene_file_destroy.argtypes = [vp]
    L.dr_progressive_create.restype = i32
    L.dr_progressive_create.argtypes = [vp, vp, vp, i32, P(vp)]
    L.dr_progressive_set_target.restype = i32
    L.dr_progressive_set_target.argtypes = [vp, i32]
    L.dr_progressive_set_view.restype = i32
    L.dr_progressive_set_view.argtypes = [vp, vp, vp]
    L.dr_progressive_set_callbacks.restype = i32
    L.dr_progressive_set_callbacks.argtypes = [vp, PROGRESS_CALLBACK, PROGRESS_CALLBACK, PROGRESS_CALLBACK, vp]
    for fn in ("dr_progressive_start", "dr_progressive_stop"):
        getattr(L, fn).restype = i32
        getattr(L, fn).argtypes = [vp]
    L.dr_progressive_wait.restype = i32
    L.dr_progressive_wait.argtypes = [vp, i32, i32]
    L.dr_progressive_completed.restype = i32
    L.dr_progressive_completed.argtypes = [vp]
    L.dr_progressive_read.restype = i32
    L.dr_progressive_read.argtypes = [vp, vp, i32, i32, P(i32)]
    L.dr_progressive_save_png.restype = i32
    L.dr_progressive_save_png.argtypes = [vp, ctypes.c_char_p]
    L.dr_progressive_render_seconds.restype = ctypes.c_double
    L.dr_progressive_render_seconds.argtypes = [vp]
    L.dr_progressive_destroy.restype = None
    L.dr_progressive_destroy.argtypes = [vp]
    _lib = L
    return L


def check(status: int) -> None:
    if status != DR_OK:
        raise DumbRayError(status, lib().dr_last_error().decode(errors="replace"))


def block_count(width: int, height: int) -> int:
    return ((width + BLOCK_W - 1) // BLOCK_W) * ((height + BLOCK_H - 1) // BLOCK_H)


# ---- material / light / camera constructors ------------------------------------------------------

def dumb_based(fresnel=(0.2, 0.2, 0.2), specular=8.0, diffuse=(0.2, 0.2, 0.2), metal=0.5) -> DrMaterial:
    """DumbBasedShader(fresnel, specular, diffuse, metal) (DumbBasedShader.impl.cuh:5-16)."""
    m = DrMaterial()
    m.type = MAT_DUMB_BASED
    m.fresnel[:] = fresnel
    m.specular = specular
    m.color[:] = diffuse
    m.metal = metal
    return m


def simple_stochastic(color=(1.0, 1.0, 1.0), diffuse=0.05, smoothness=0.95, shininess=2.0) -> DrMaterial:
    """SimpleStochasticShader(color, diffuse, smoothness, shininess) (SimpleStochasticShader.impl.cuh:4-11)."""
    m = DrMaterial()
    m.type = MAT_SIMPLE_STOCHASTIC
    m.color[:] = color
    m.diffuse = diffuse
    m.smoothness = smoothness
    m.shininess = shininess
    return m


def lambert(albedo=(0.7, 0.7, 0.7), emission=(0.0, 0.0, 0.0)) -> DrMaterial:
    m = DrMaterial()
    m.type = MAT_LAMBERT
    m.color[:] = albedo
    m.emission[:] = emission
    return m


def mirror(reflectance=(0.9, 0.9, 0.9)) -> DrMaterial:
    m = DrMaterial()
    m.type = MAT_MIRROR
    m.color[:] = reflectance
    return m


def glossy(albedo=(0.8, 0.8, 0.8), roughness=0.2) -> DrMaterial:
    m = DrMaterial()
    m.type = MAT_GLOSSY
    m.color[:] = albedo
    m.roughness = roughness
    return m


def spherical_light(color, position, radius) -> DrLight:
    """SphericalLightEmitter(color, position, radius)."""
    l = DrLight()
    l.type = LIGHT_SPHERICAL
    l.color[:] = color
    l.position[:] = position
    l.radius = radius
    return l


def soft_directional_light(color, direction, distance, softness) -> DrLight:
    """SimpleSoftDirectionalLight(color, direction, distance, softness)."""
    l = DrLight()
    l.type = LIGHT_SOFT_DIRECTIONAL
    l.color[:] = color
    l.direction[:] = direction
    l.distance = distance
    l.softness = softness
    return l


def fresnel_shader(color=(1.0, 1.0, 1.0)) -> DrMaterial:
    """Shaders::FresnelShader(color) (FresnelShader.impl.cuh:5-19): no indirect samples."""
    m = DrMaterial()
    m.type = MAT_FRESNEL
    m.color[:] = color
    return m


def default_shader(color=(1.0, 1.0, 1.0), diffuse=0.7, smoothness=0.2, shininess=8.0) -> DrMaterial:
    """DefaultShaderGeneric(color, diffuse, smoothness, shine) (DefaultShader.impl.cuh:3-10)."""
    m = DrMaterial()
    m.type = MAT_DEFAULT
    m.color[:] = color
    m.diffuse = diffuse
    m.smoothness = smoothness
    m.shininess = shininess
    return m


def spotlight(color=(1.0, 1.0, 1.0), luminosity=1500.0, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0),
              hotspot_angle=16.0, falloff_angle=64.0, falloff_power=1.0, emitter_size=0.25, emit_from_sphere=False,
              cast_shadows=True, samples=1) -> DrLight:
    """Lights::Spotlight(...) with the reference's defaults (Spotlight.cuh:7-11)."""
    l = DrLight()
    l.type = LIGHT_SPOTLIGHT
    l.color[:] = color
    l.luminosity = luminosity
    l.position[:] = position
    l.direction[:] = direction
    l.hotspot_angle, l.falloff_angle, l.falloff_power = hotspot_angle, falloff_angle, falloff_power
    l.emitter_size = emitter_size
    l.emit_from_sphere = 1 if emit_from_sphere else 0
    l.cast_shadows = 1 if cast_shadows else 0
    l.samples = samples
    return l


def directional_light(color, direction, distance) -> DrLight:
    """SimpleDirectionalLight(color, direction, distance)."""
    l = DrLight()
    l.type = LIGHT_DIRECTIONAL
    l.color[:] = color
    l.direction[:] = direction
    l.distance = distance
    return l


def camera(lens: int, position=(0.0, 0.0, 0.0), target=None, angle=(60.0, 60.0), focal_distance=128.0, softness=1.0,
           filter=(1.0, 1.0, 1.0), basis=None) -> DrCamera:
    """Camera = lens + transform.  ``basis`` = (right, up, forward) or derived from ``target``; the
    default is the identity orientation (+z forward), i.e. a reference Transform with zero Euler angles."""
    c = DrCamera()
    c.lens = lens
    c.angle[:] = angle if hasattr(angle, "__len__") else (angle, angle)
    c.focal_distance = focal_distance
    c.softness = softness
    c.filter[:] = filter
    c.position[:] = position
    if basis is None and target is not None:
        _, r, u, f = scenes.camera_basis(position, target)
        basis = (r, u, f)
    if basis is None:
        basis = ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0))
    c.right[:] = [float(v) for v in basis[0]]
    c.up[:] = [float(v) for v in basis[1]]
    c.forward[:] = [float(v) for v in basis[2]]
    return c


def render_params(width, height, mode=MODE_REFERENCE, samples=(1, 1), max_bounces=2, cull_backfaces=True,
                  boxing=BOXING_HEIGHT, iteration=1, seed=0) -> DrRenderParams:
    p = DrRenderParams()
    p.mode, p.width, p.height = mode, width, height
    p.samples_x, p.samples_y = samples
    p.max_bounces = max_bounces
    p.cull_backfaces = 1 if cull_backfaces else 0
    p.boxing = boxing
    p.iteration = iteration
    p.seed = seed & 0xFFFFFFFF
    return p


def _ptr(t) -> int:
    """Device pointer of a CUDA torch tensor (contiguous), or 0 for None."""
    if t is None:
        return 0
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return t.data_ptr()


def _stream_ptr(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


class Scene:
    """Triangles + materials + lights, octree built on the host and uploaded once (immutable).

    ``max_depth`` / ``split_threshold`` / ``box_epsilon`` = 0 build the reference's octree
    (depth 24, 8 triangles per leaf, 1.28e-3 box padding): casts and traversal counts then match the
    reference's.  ``box_epsilon=PHYSICAL_TREE`` (any negative value) pads boxes by 2^-18 x the largest
    absolute coordinate instead, for scenes rendered in the physical mode only: the same closest hits
    up to float32 near-ties, with far fewer duplicated leaf references on finely tessellated meshes."""

    def __init__(self, tris, normals=None, mat_id=None, materials=(), lights=(), max_depth=0, split_threshold=0,
                 threads=0, box_epsilon=0.0, device_build=False):
        L = lib()
        self.tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 3, 3)
        self.n = len(self.tris)
        self._nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3, 3)
        self._mat = None if mat_id is None else np.ascontiguousarray(mat_id, dtype=np.int32)
        mats = list(materials)
        lts = list(lights)
        self.materials, self.lights = mats, lts
        marr = (DrMaterial * max(1, len(mats)))(*mats)
        larr = (DrLight * max(1, len(lts)))(*lts)
        bp = DrBuildParams(max_depth, split_threshold, threads, box_epsilon, 1 if device_build else 0)
        h = ctypes.c_void_p()
        check(L.dr_scene_create(self.tris.ctypes.data, None if self._nrm is None else self._nrm.ctypes.data,
                                None if self._mat is None else self._mat.ctypes.data, self.n,
                                ctypes.addressof(marr) if mats else None, len(mats),
                                ctypes.addressof(larr) if lts else None, len(lts), ctypes.byref(bp), ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("scene destroyed")
        return self._h

    def stats(self):
        L = lib()
        nodes, leaves, refs = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        depth = ctypes.c_int32()
        check(L.dr_scene_stats(self.handle, ctypes.byref(nodes), ctypes.byref(leaves), ctypes.byref(refs), ctypes.byref(depth)))
        return dict(nodes=nodes.value, leaves=leaves.value, refs=refs.value, depth=depth.value)

    def export_tree(self):
        s = self.stats()
        box = np.zeros((s["nodes"], 6), np.float32)
        child = np.zeros(s["nodes"], np.int32)
        leaf = np.zeros((s["nodes"], 2), np.int32)
        refs = np.zeros(max(1, s["refs"]), np.int32)
        check(lib().dr_scene_export_tree(self.handle, box.ctypes.data, child.ctypes.data, leaf.ctypes.data, refs.ctypes.data))
        return box, child, leaf, refs[: s["refs"]]

    def triangle_params_device(self):
        """(albedo_ptr, emission_ptr): device float[n][3] arrays the kernels read (writable in place)."""
        a, e = ctypes.c_void_p(), ctypes.c_void_p()
        check(lib().dr_scene_triangle_params_device(self.handle, ctypes.byref(a), ctypes.byref(e)))
        return a.value, e.value

    def set_triangle_params(self, albedo=None, emission=None, roughness=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float32) for a in (albedo, emission, roughness)]
        check(lib().dr_scene_set_triangle_params(self.handle, *[None if a is None else a.ctypes.data for a in arrs]))

    def set_textures(self, textures, uv=None):
        """dr_scene_set_textures: ``textures`` = [(rgba float [h, w, 4], filtering)], ``uv`` = float
        [n, 3, 2] corner texture coordinates (None: zeros)."""
        imgs = [np.ascontiguousarray(t, dtype=np.float32) for t, _ in textures]
        arr = (DrTexture * max(1, len(imgs)))()
        for i, (img, (_, filt)) in enumerate(zip(imgs, textures)):
            arr[i].width, arr[i].height, arr[i].filtering = img.shape[1], img.shape[0], int(filt)
            arr[i].rgba = img.ctypes.data
        u = None if uv is None else np.ascontiguousarray(uv, dtype=np.float32).reshape(-1, 3, 2)
        check(lib().dr_scene_set_textures(self.handle, ctypes.addressof(arr) if imgs else None, len(imgs),
                                          None if u is None else u.ctypes.data))

    def close(self):
        if self._h is not None:
            lib().dr_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tight_box_epsilon(tris) -> float:
    """Octree box padding scaled to the scene: 2^-18 x the largest absolute coordinate (what
    ``box_epsilon=PHYSICAL_TREE`` selects).  The leaf-box acceptance test of the traversal must
    tolerate the float rounding of hit points (a few units of 2^-24 x the larger of |origin| and
    |hit point|), so this keeps a margin of 2^5 for ray origins up to 2x the scene's extent."""
    m = float(np.max(np.abs(np.asarray(tris, dtype=np.float32)))) if len(tris) else 1.0
    return max(m, 1e-30) * 2.0 ** -18


def build_octree_host(tris, max_depth=0, split_threshold=0, threads=0, box_epsilon=0.0, device_build=False):
    """Host-only octree build (dr_octree_create_host); returns (stats, box, child, leaf, refs) with
    node 0 = root, as dr_scene_export_tree."""
    L = lib()
    t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 3, 3)
    bp = DrBuildParams(max_depth, split_threshold, threads, box_epsilon, 1 if device_build else 0)
    h = ctypes.c_void_p()
    check(L.dr_octree_create_host(t.ctypes.data, len(t), ctypes.byref(bp), ctypes.byref(h)))
    try:
        nodes, leaves, refs = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        depth = ctypes.c_int32()
        check(L.dr_octree_stats(h, ctypes.byref(nodes), ctypes.byref(leaves), ctypes.byref(refs), ctypes.byref(depth)))
        box = np.zeros((nodes.value, 6), np.float32)
        child = np.zeros(nodes.value, np.int32)
        leaf = np.zeros((nodes.value, 2), np.int32)
        ref = np.zeros(max(1, refs.value), np.int32)
        check(L.dr_octree_export(h, box.ctypes.data, child.ctypes.data, leaf.ctypes.data, ref.ctypes.data))
        stats = dict(nodes=nodes.value, leaves=leaves.value, refs=refs.value, depth=depth.value)
        return stats, box, child, leaf, ref[: refs.value]
    finally:
        L.dr_octree_destroy(h)


def octree_group_planes_host(tris, split_threshold=0, box_epsilon=0.0):
    """Host-only octree build and its group-test planes (dr_octree_group_planes): returns
    (box, child, leaf, gbox, gbox_ref) with box/child/leaf as build_octree_host (node 0 = root) and
    gbox / gbox_ref float32 [(nodes - 1) / 8, 6, 8] (lo x/y/z, hi x/y/z planes of each group's 8
    children; group g = export nodes 8g + 1 .. 8g + 8)."""
    L = lib()
    t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 3, 3)
    bp = DrBuildParams(0, split_threshold, 0, box_epsilon, 0)
    h = ctypes.c_void_p()
    check(L.dr_octree_create_host(t.ctypes.data, len(t), ctypes.byref(bp), ctypes.byref(h)))
    try:
        nodes, leaves, refs = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        depth = ctypes.c_int32()
        check(L.dr_octree_stats(h, ctypes.byref(nodes), ctypes.byref(leaves), ctypes.byref(refs), ctypes.byref(depth)))
        box = np.zeros((nodes.value, 6), np.float32)
        child = np.zeros(nodes.value, np.int32)
        leaf = np.zeros((nodes.value, 2), np.int32)
        ref = np.zeros(max(1, refs.value), np.int32)
        check(L.dr_octree_export(h, box.ctypes.data, child.ctypes.data, leaf.ctypes.data, ref.ctypes.data))
        groups = (nodes.value - 1) // 8
        g = np.zeros((max(groups, 1), 6, 8), np.float32)
        r = np.zeros((max(groups, 1), 6, 8), np.float32)
        check(L.dr_octree_group_planes(h, g.ctypes.data, r.ctypes.data))
        return box, child, leaf, g[:groups], r[:groups]
    finally:
        L.dr_octree_destroy(h)


def canonical_tree(box, child, leaf, refs):
    """Depth-first (child order) dump of an exported tree: (boxes [k,6], counts [k] (-1 = inner),
    concatenated leaf triangle ids), comparable across builders regardless of node numbering."""
    out_box, out_cnt, out_tri = [], [], []
    stack = [0]
    while stack:
        i = stack.pop()
        out_box.append(box[i])
        if child[i] < 0:
            f, c = leaf[i]
            out_cnt.append(c)
            out_tri.append(refs[f:f + c])
        else:
            out_cnt.append(-1)
            stack.extend(range(child[i] + 7, child[i] - 1, -1))
    tri = np.concatenate(out_tri) if out_tri else np.zeros(0, np.int32)
    return np.asarray(out_box, np.float32), np.asarray(out_cnt, np.int32), tri.astype(np.int32)


def cast(scene: Scene, origins, directions, ignore=None, cull_backfaces=True, counted=False, stream=None):
    """Closest-hit casts through dr_cast for CUDA tensors origins/directions [n,3] float32.
    Returns (hit_tri int32 [n], hit_t float32 [n]) (+ (box_tests, tri_tests) when counted)."""
    import torch
    n = origins.shape[0]
    dev = origins.device
    tri = torch.empty(n, dtype=torch.int32, device=dev)
    t = torch.empty(n, dtype=torch.float32, device=dev)
    sp = _stream_ptr(stream)
    if counted:
        nb = torch.empty(n, dtype=torch.int32, device=dev)
        nt = torch.empty(n, dtype=torch.int32, device=dev)
        check(lib().dr_cast_counted(scene.handle, _ptr(origins), _ptr(directions), _ptr(ignore), n, 1 if cull_backfaces else 0,
                                    _ptr(tri), _ptr(t), _ptr(nb), _ptr(nt), sp))
        return tri, t, nb, nt
    check(lib().dr_cast(scene.handle, _ptr(origins), _ptr(directions), _ptr(ignore), n, 1 if cull_backfaces else 0,
                        _ptr(tri), _ptr(t), sp))
    return tri, t


class Renderer:
    """Owns the wavefront scratch of one caller (dr_renderer)."""

    def __init__(self, wave_paths: int = 0, lanes: int = 0):
        h = ctypes.c_void_p()
        check(lib().dr_renderer_create(int(wave_paths), ctypes.byref(h)))
        self._h = h
        if lanes:
            self.set_lanes(lanes)

    @property
    def handle(self):
        return self._h

    def launches(self) -> int:
        return int(lib().dr_renderer_launch_count(self._h))

    def set_profiling(self, enable: bool):
        check(lib().dr_renderer_set_profiling(self._h, 1 if enable else 0))

    def kernel_times(self):
        """{class: (ms, launches)} for camera / trace / shade / shadow / resolve."""
        ms = np.zeros(5, np.float64)
        n = np.zeros(5, np.int64)
        check(lib().dr_renderer_kernel_times(self._h, ms.ctypes.data, n.ctypes.data))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(("camera", "trace", "shade", "shadow", "resolve"))}

    def kernel_busy(self):
        """{class: ms}: union of each class's launch intervals over all lanes since profiling began."""
        b = np.zeros(5, np.float64)
        check(lib().dr_renderer_kernel_busy(self._h, b.ctypes.data))
        return {k: float(b[i]) for i, k in enumerate(("camera", "trace", "shade", "shadow", "resolve"))}

    def set_lanes(self, lanes: int):
        """Concurrent wave pipelines of one render (dr_renderer_set_lanes)."""
        check(lib().dr_renderer_set_lanes(self._h, int(lanes)))

    def set_block_shape(self, shape: int):
        """Traversal block shape (dr_renderer_set_block_shape): 0 = 256 x 3, 1 = 128 x 6 per SM."""
        check(lib().dr_renderer_set_block_shape(self._h, int(shape)))

    @property
    def block_shape(self) -> int:
        return int(lib().dr_renderer_block_shape(self._h))

    @property
    def lanes(self) -> int:
        return int(lib().dr_renderer_lanes(self._h))

    def set_counting(self, enable: bool):
        check(lib().dr_renderer_set_counting(self._h, 1 if enable else 0))

    def counters(self):
        c = np.zeros(6, np.int64)
        check(lib().dr_renderer_counters(self._h, c.ctypes.data))
        return dict(trace_rays=int(c[0]), trace_box=int(c[1]), trace_tri=int(c[2]), shadow_casts=int(c[3]),
                    shadow_box=int(c[4]), shadow_tri=int(c[5]))

    def wave_counts(self, n: int = 9):
        """(rays per bounce, shadow records per bounce) of the last wave on the renderer's own scratch
        (dr_renderer_wave_counts), bounces 0 .. n-1."""
        rays = np.zeros(n, np.int32)
        sh = np.zeros(n, np.int32)
        check(lib().dr_renderer_wave_counts(self._h, rays.ctypes.data, sh.ctypes.data, int(n)))
        return rays.tolist(), sh.tolist()

    def render_blocks(self, scene: Scene, cam: DrCamera, fb, start_block: int, end_block: int, params: DrRenderParams,
                      stream=None):
        """dr_render_blocks into ``fb`` (CUDA float32 tensor [blocks*128, 4], block-major)."""
        check(lib().dr_render_blocks(self._h, scene.handle, ctypes.byref(cam), _ptr(fb), int(start_block), int(end_block),
                                     ctypes.byref(params), _stream_ptr(stream)))

    def close(self):
        if self._h is not None:
            lib().dr_renderer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


    def render_adjoint(self, scene: Scene, cam: DrCamera, dl_dfb, start_block: int, end_block: int, params: DrRenderParams,
                       grad_albedo, grad_emission, stream=None):
        """dr_render_adjoint: adds dL/d albedo and dL/d emission (CUDA float32 [n,3]) for dL/dI = dl_dfb."""
        check(lib().dr_render_adjoint(self._h, scene.handle, ctypes.byref(cam), _ptr(dl_dfb), int(start_block), int(end_block),
                                      ctypes.byref(params), _ptr(grad_albedo), _ptr(grad_emission), _stream_ptr(stream)))


class Batch:
    """Many render jobs sharing the same waves (dr_batch); optionally replayed as one CUDA graph."""

    def __init__(self, jobs):
        """jobs: sequence of (scene, camera, params, fb_tensor, start_block, end_block)."""
        self._keep = list(jobs)
        arr = (DrBatchItem * len(self._keep))()
        for i, (scene, cam, params, fb, s0, s1) in enumerate(self._keep):
            arr[i].scene = scene.handle.value
            arr[i].camera = cam
            arr[i].params = params
            arr[i].fb = _ptr(fb)
            arr[i].start_block = s0
            arr[i].end_block = s1
        h = ctypes.c_void_p()
        check(lib().dr_batch_create(ctypes.addressof(arr), len(self._keep), ctypes.byref(h)))
        self._h = h

    def paths(self) -> int:
        return int(lib().dr_batch_paths(self._h))

    def set_iteration(self, iteration: int):
        check(lib().dr_batch_set_iteration(self._h, int(iteration)))

    def render(self, renderer: "Renderer", use_graph: bool = True, stream=None):
        check(lib().dr_batch_render(renderer.handle, self._h, 1 if use_graph else 0, _stream_ptr(stream)))

    def close(self):
        if self._h is not None:
            lib().dr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BlockRenderer:
    """Host mirror of DumbRenderer's block-renderer interface (DumbRenderer.cuh:9-64): the same
    configuration setters and a ``render_blocks_gpu`` that renders a block range of a device frame
    buffer with the progressive blend of iteration ``iteration`` (DumbRenderer.cu:87-113)."""

    def __init__(self, scene: Scene, camera: DrCamera, width: int, height: int, mode=MODE_REFERENCE, boxing=BOXING_HEIGHT,
                 max_bounces=2, samples_per_pixel=(1, 1), ignore_backfaces=True, seed=0, wave_paths=0):
        self.scene, self.camera = scene, camera
        self.width, self.height, self.mode, self.seed = width, height, mode, seed
        self.set_boxing_mode(boxing)
        self.set_max_bounces(max_bounces)
        self.set_samples_per_pixel(*samples_per_pixel)
        self.set_ignore_backfaces(ignore_backfaces)
        self._renderer = Renderer(wave_paths)

    # configuration (DumbRenderer.cu:26-50)
    def set_boxing_mode(self, mode):
        self.boxing = int(mode)

    def set_max_bounces(self, n):
        self.max_bounces = min(int(n), 64)

    def set_samples_per_pixel(self, x, y):
        self.samples_x, self.samples_y = max(1, int(x)), max(1, int(y))

    def set_ignore_backfaces(self, ignore):
        self.ignore_backfaces = bool(ignore)

    def block_count(self) -> int:
        return block_count(self.width, self.height)

    def params(self, iteration: int) -> DrRenderParams:
        return render_params(self.width, self.height, self.mode, (self.samples_x, self.samples_y), self.max_bounces,
                             self.ignore_backfaces, self.boxing, iteration, self.seed)

    def render_blocks_gpu(self, device_fb, start_block: int, end_block: int, iteration: int = 1, stream=None) -> bool:
        self._renderer.render_blocks(self.scene, self.camera, device_fb, start_block, end_block, self.params(iteration), stream)
        return True

    def launches(self) -> int:
        return self._renderer.launches()


def new_frame_buffer(width: int, height: int, device="cuda"):
    import torch
    return torch.zeros((block_count(width, height) * BLOCK_SIZE, 4), dtype=torch.float32, device=device)


def blockmajor_to_image(fb, width: int, height: int) -> np.ndarray:
    """Block-major float4 frame buffer -> row-major [H, W, 4] numpy image."""
    a = fb.detach().cpu().numpy() if hasattr(fb, "detach") else np.asarray(fb)
    bw = (width + BLOCK_W - 1) // BLOCK_W
    bh = (height + BLOCK_H - 1) // BLOCK_H
    a = a.reshape(bh, bw, BLOCK_H, BLOCK_W, 4).transpose(0, 2, 1, 3, 4).reshape(bh * BLOCK_H, bw * BLOCK_W, 4)
    return np.ascontiguousarray(a[:height, :width])


def image_to_blockmajor(img: np.ndarray) -> np.ndarray:
    h, w = img.shape[:2]
    bw = (w + BLOCK_W - 1) // BLOCK_W
    bh = (h + BLOCK_H - 1) // BLOCK_H
    pad = np.zeros((bh * BLOCK_H, bw * BLOCK_W, img.shape[2]), img.dtype)
    pad[:h, :w] = img
    return np.ascontiguousarray(pad.reshape(bh, BLOCK_H, bw, BLOCK_W, -1).transpose(0, 2, 1, 3, 4).reshape(-1, img.shape[2]))


def render_blocks_noalloc(scene: Scene, cam: DrCamera, fb, start_block: int, end_block: int, params: DrRenderParams,
                          stream=None):
    """dr_render_blocks_noalloc: the same render as Renderer.render_blocks for callers that cannot
    allocate device memory while rendering (a foreign memory pool, a thread that must not synchronise
    the device through cudaMalloc); uses the library's
    fixed 16 MiB device scratch array, at most 2048 blocks per call, calls on different streams race."""
    L = lib()
    fn = L.dr_render_blocks_noalloc
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                   ctypes.c_void_p]
    check(fn(scene.handle, ctypes.byref(cam), _ptr(fb), int(start_block), int(end_block), ctypes.byref(params),
             _stream_ptr(stream)))


def render_differentiable(scene: Scene, cam: DrCamera, params: DrRenderParams, albedo, emission, renderer=None):
    """Physical-mode render as a differentiable function of per-triangle albedo and emission
    (CUDA float32 [n,3] tensors): returns the block-major [blocks*128, 4] image; its backward pass is
    the path-replay adjoint (dr_render_adjoint) with the same random numbers.  The parameters are
    copied into the scene's device arrays before rendering; the emissive-triangle sampling table
    keeps the emitter set and powers the scene was created with (sampling pdfs are constants)."""
    import torch

    class _Render(torch.autograd.Function):
        @staticmethod
        def forward(ctx, alb, emi):
            a_ptr, e_ptr = scene.triangle_params_device()
            n = scene.n
            # write the parameters in place (device -> device copies on the current stream)
            at = torch.cuda.current_stream()
            _copy_into(a_ptr, alb.detach().contiguous().float(), n)
            _copy_into(e_ptr, emi.detach().contiguous().float(), n)
            r = renderer if renderer is not None else Renderer(1 << 20)
            fb = new_frame_buffer(params.width, params.height, alb.device)
            r.render_blocks(scene, cam, fb, 0, block_count(params.width, params.height), params, at)
            ctx.r = r
            return fb

        @staticmethod
        def backward(ctx, g):
            g = g.contiguous().float()
            ga = torch.zeros((scene.n, 3), dtype=torch.float32, device=g.device)
            ge = torch.zeros((scene.n, 3), dtype=torch.float32, device=g.device)
            ctx.r.render_adjoint(scene, cam, g, 0, block_count(params.width, params.height), params, ga, ge)
            return ga, ge

    return _Render.apply(albedo, emission)


class _DeviceArray:
    """A raw device allocation exposed through the CUDA array interface (zero-copy torch view)."""

    def __init__(self, ptr: int, shape, typestr="<f4"):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False), "version": 3}


def device_view(ptr: int, shape, device="cuda"):
    """torch view of device memory owned by the library (e.g. a scene's albedo / emission arrays)."""
    import torch
    return torch.as_tensor(_DeviceArray(ptr, shape), device=device)


def _copy_into(dst_ptr: int, src, n: int):
    device_view(dst_ptr, (n, 3), src.device).copy_(src)


# ---- images (host) ---------------------------------------------------------------------------

def _image_arg(rgba):
    a = np.ascontiguousarray(rgba, dtype=np.float32)
    if a.ndim != 3 or a.shape[2] != 4:
        raise ValueError("expected a float32 [height, width, 4] image")
    return a


def to_rgba8(rgba) -> np.ndarray:
    """dr_image_to_rgba8: the reference's 8-bit conversion (v = 255 c, clamped, truncated)."""
    a = _image_arg(rgba)
    out = np.empty(a.shape, np.uint8)
    check(lib().dr_image_to_rgba8(a.ctypes.data, a.shape[1], a.shape[0], out.ctypes.data))
    return out


def image_from_blocks(fb, width: int, height: int) -> np.ndarray:
    """dr_image_from_blocks on a host copy of a block-major frame buffer."""
    f = np.ascontiguousarray(fb.detach().cpu().numpy() if hasattr(fb, "detach") else fb, dtype=np.float32)
    out = np.empty((height, width, 4), np.float32)
    check(lib().dr_image_from_blocks(f.ctypes.data, width, height, out.ctypes.data))
    return out


def write_png(rgba, path) -> None:
    """dr_image_write_png: 8-bit RGBA PNG with the reference's channel conversion."""
    a = _image_arg(rgba)
    check(lib().dr_image_write_png(a.ctypes.data, a.shape[1], a.shape[0], str(path).encode()))


def write_pfm(rgba, path) -> None:
    """dr_image_write_pfm: float RGB portable float map (unclamped radiance)."""
    a = _image_arg(rgba)
    check(lib().dr_image_write_pfm(a.ctypes.data, a.shape[1], a.shape[0], str(path).encode()))


class Progressive:
    """Progressive render process (dr_progressive, the reference's BufferedRenderProcess without its
    window): a native worker thread renders iteration after iteration of one view and publishes each
    finished image.  Callbacks (Python callables without arguments) run on the worker thread."""

    def __init__(self, scene: Scene, cam: DrCamera, params: DrRenderParams, double_buffered: bool = False):
        h = ctypes.c_void_p()
        check(lib().dr_progressive_create(scene.handle, ctypes.byref(cam), ctypes.byref(params),
                                          1 if double_buffered else 0, ctypes.byref(h)))
        self._h, self._scene, self.width, self.height = h, scene, params.width, params.height
        self._cbs = None

    def set_target(self, iterations: int):
        check(lib().dr_progressive_set_target(self._h, int(iterations)))

    def set_view(self, cam: DrCamera = None, params: DrRenderParams = None):
        check(lib().dr_progressive_set_view(self._h, None if cam is None else ctypes.byref(cam),
                                            None if params is None else ctypes.byref(params)))
        if params is not None:
            self.width, self.height = params.width, params.height

    def set_callbacks(self, on_iteration=None, on_complete=None, on_error=None):
        wrap = [PROGRESS_CALLBACK(lambda _a, f=f: f()) if f else PROGRESS_CALLBACK() for f in (on_iteration, on_complete, on_error)]
        self._cbs = wrap   # keep the ctypes thunks alive while the worker may call them
        check(lib().dr_progressive_set_callbacks(self._h, wrap[0], wrap[1], wrap[2], None))

    def start(self):
        check(lib().dr_progressive_start(self._h))

    def stop(self):
        check(lib().dr_progressive_stop(self._h))

    def wait(self, count: int, timeout_ms: int = 60000):
        check(lib().dr_progressive_wait(self._h, int(count), int(timeout_ms)))

    def completed(self) -> int:
        return int(lib().dr_progressive_completed(self._h))

    def read(self):
        """(row-major float32 [H, W, 4] image, its iteration index)."""
        out = np.empty((self.height, self.width, 4), np.float32)
        it = ctypes.c_int32()
        check(lib().dr_progressive_read(self._h, out.ctypes.data, self.width, self.height, ctypes.byref(it)))
        return out, int(it.value)

    def save_png(self, path):
        check(lib().dr_progressive_save_png(self._h, str(path).encode()))

    def render_seconds(self) -> float:
        return float(lib().dr_progressive_render_seconds(self._h))

    def close(self):
        if self._h is not None:
            lib().dr_progressive_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- OBJ meshes (host) -----------------------------------------------------------------------

class SceneFile:
    """A DumbRay scene file (.dumb) read by dr_scene_file_load, like DumbRenderContext::fromFile:
    triangles in push order (``tris``, per-corner ``normals``, ``uv``, ``mat_id``), ``materials``,
    ``lights``, ``textures`` [(rgba, filtering)], the file's ``camera`` and reference-mode ``params``
    (width / height left 0)."""

    def __init__(self, path):
        L = lib()
        h = ctypes.c_void_p()
        check(L.dr_scene_file_load(str(path).encode(), ctypes.byref(h)))
        try:
            counts = np.zeros(3, np.int32)
            check(L.dr_scene_file_counts(h, counts.ctypes.data))
            n, nm, nl = (int(c) for c in counts)
            self.tris = np.zeros((n, 3, 3), np.float32)
            self.normals = np.zeros((n, 3, 3), np.float32)
            self.mat_id = np.zeros(n, np.int32)
            check(L.dr_scene_file_geometry(h, self.tris.ctypes.data, self.normals.ctypes.data, self.mat_id.ctypes.data))
            marr = (DrMaterial * max(1, nm))()
            larr = (DrLight * max(1, nl))()
            if nm:
                check(L.dr_scene_file_materials(h, ctypes.addressof(marr)))
            if nl:
                check(L.dr_scene_file_lights(h, ctypes.addressof(larr)))
            self.materials = [marr[i] for i in range(nm)]
            self.lights = [larr[i] for i in range(nl)]
            self.camera = DrCamera()
            check(L.dr_scene_file_camera(h, ctypes.byref(self.camera)))
            self.params = DrRenderParams()
            check(L.dr_scene_file_render_params(h, ctypes.byref(self.params)))
            self.uv = np.zeros((n, 3, 2), np.float32)
            if n:
                check(L.dr_scene_file_texcoords(h, self.uv.ctypes.data))
            self.textures = []
            for i in range(L.dr_scene_file_textures(h)):
                w, hh, f = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
                check(L.dr_scene_file_texture(h, i, ctypes.byref(w), ctypes.byref(hh), ctypes.byref(f), None))
                img = np.zeros((hh.value, w.value, 4), np.float32)
                check(L.dr_scene_file_texture(h, i, None, None, None, img.ctypes.data))
                self.textures.append((img, f.value))
        finally:
            L.dr_scene_file_destroy(h)

    def render_params(self, width, height, iteration=1, seed=0) -> DrRenderParams:
        p = DrRenderParams.from_buffer_copy(self.params)
        p.width, p.height, p.iteration, p.seed = width, height, iteration, seed
        return p

    def scene(self, **build) -> "Scene":
        """The octree scene over the file's geometry (DumbRenderContext::buildFromFile); ``build``
        takes Scene's build keywords."""
        sc = Scene(self.tris, normals=self.normals, mat_id=self.mat_id, materials=self.materials,
                   lights=self.lights, **build)
        if self.textures:
            sc.set_textures(self.textures, self.uv)
        return sc


def load_scene_file(path) -> SceneFile:
    return SceneFile(path)


def read_png(path) -> np.ndarray:
    """dr_png_read: float RGBA [h, w, 4] = the file's 8-bit channels / 255 (Images::getTexturePNG)."""
    L = lib()
    w, h = ctypes.c_int32(), ctypes.c_int32()
    check(L.dr_png_read(str(path).encode(), ctypes.byref(w), ctypes.byref(h), None))
    px = np.zeros((h.value, w.value, 4), np.uint8)
    check(L.dr_png_read(str(path).encode(), ctypes.byref(w), ctypes.byref(h), px.ctypes.data))
    return px.astype(np.float32) / np.float32(255.0)


def read_obj(path):
    """dr_obj_read: {object name: (xyz [n,3,3], normals [n,3,3], uv [n,3,3])} in file order, read with
    the reference's rules (groups are `g` ranges, x mirrored, generated normals, triangle fans)."""
    L = lib()
    h = ctypes.c_void_p()
    check(L.dr_obj_read(str(path).encode(), ctypes.byref(h)))
    try:
        out = {}
        for i in range(L.dr_mesh_file_objects(h)):
            n = L.dr_mesh_file_object_triangles(h, i)
            xyz, nrm, uv = (np.zeros((n, 3, 3), np.float32) for _ in range(3))
            check(L.dr_mesh_file_object_data(h, i, xyz.ctypes.data, nrm.ctypes.data, uv.ctypes.data))
            out[L.dr_mesh_file_object_name(h, i).decode(errors="replace")] = (xyz, nrm, uv)
        return out
    finally:
        L.dr_mesh_file_destroy(h)
