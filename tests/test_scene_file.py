"""Scene files (.dumb): dr_scene_file_load against the reference's own loader.

The reference side is DumbRenderContext::fromFile compiled from the reference sources
(oracle/_ref/libdumbref.so, dref_dumb_*): the triangles it pushes, and its materials, lights, lens
and camera transform read back field by field.  Our side goes through the same reference
constructors (dref_record_*), so equal dumps mean our loader hands the renderer the constructor
arguments the reference's loader produced.  Comparisons are bit-exact."""
from pathlib import Path
import sys

import numpy as np
import pytest

import dumbray_gb300 as dr
import _oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLD))
from make_golden import _obj_text, write_scene_file, write_scene_file_textured  # noqa: E402

from dumbray_gb300 import scenes  # noqa: E402

need_ref = pytest.mark.skipif(not O.reference_available() or not hasattr(O.reference(), "dref_dumb_load")
                              if O.reference_available() else True, reason="reference library not built")

EXAMPLE = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "example_scenes" / "0" / "0.dumb"


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype == np.float32:
        return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.astype(np.float32).view(np.uint32))
    return np.array_equal(a, b)


def _assert_matches_reference(path):
    ref = O.ref_scene_file_dump(path)
    ours = O.scene_file_dump(dr.load_scene_file(path))
    # A perspective / stochastic lens keeps x = 0.5 / tan(angle / 2).  The reference build folds that
    # at compile time for a default-constructed lens (correctly rounded tan) and evaluates tanf at run
    # time for a lens built from a value, 2 ulp apart at 60 degrees; the renderer evaluates it at run
    # time.  That one field may differ by 2 ulp.
    if ref["camera"][0] in (0, 1):
        a, b = ref["camera"][1:2].view(np.int32), ours["camera"][1:2].view(np.int32)
        assert abs(int(a[0]) - int(b[0])) <= 2
        ref["camera"][1] = ours["camera"][1]
    for k in ("xyz", "nrm", "mat", "materials", "lights", "camera", "uv"):
        assert _same(ref[k], ours[k]), k
    assert len(ref["textures"]) == len(ours["textures"])
    for (ri, rf), (oi, of) in zip(ref["textures"], ours["textures"]):
        assert rf == of and _same(ri, oi)
    sel = [0, 1, 2, 3, 5]  # pixels_per_gpu_thread (4) is a scheduling hint with no counterpart
    assert np.array_equal(ref["settings"][sel], ours["settings"][sel])


def _scene_dir(tmp_path, main, extra=None):
    objects = [("room", scenes.box((2.0, 2.0, 2.0), inward=True)), ("sphere", scenes.icosphere(1, 0.5)),
               ("cube", scenes.box((1.0, 1.0, 1.0)))]
    (tmp_path / "m.obj").write_text(_obj_text(objects))
    for name, text in (extra or {}).items():
        (tmp_path / name).parent.mkdir(parents=True, exist_ok=True)
        (tmp_path / name).write_text(text)
    (tmp_path / "s.dumb").write_text(main)
    return tmp_path / "s.dumb"


@need_ref
def test_fixture_matches_reference_loader():
    _assert_matches_reference(GOLD / "scene_file" / "scene.dumb")


@need_ref
@pytest.mark.skipif(not EXAMPLE.exists(), reason="reference example scene not copied by build_ref.sh")
def test_reference_example_scene_matches_reference_loader():
    """The reference's own example scene (OBJ objects by name, presets with overrides and misspelt
    keys that both loaders ignore, rotated / scaled objects, relative camera position)."""
    _assert_matches_reference(EXAMPLE)


OBJ = '"mesh": { "obj": "m.obj", "object": "%s" }'

VARIANTS = {
    # every dumb_based preset, default constructor state, overrides of each field, metal clamping
    "dumb_based": """{ "materials": [
        { "name": "a", "type": "dumb_based" },
        { "name": "b", "type": "dumb_based", "preset": "rough_gold" },
        { "name": "c", "type": "dumb_based", "preset": "glossy_gold", "diffuse": [ 0.5, 0.4, 0.3 ] },
        { "name": "d", "type": "dumb_based", "preset": "glossy_finish", "metal": 0.6 },
        { "name": "e", "type": "dumb_based", "preset": "matte_finish", "specular": 3.5, "fresnel": [ 0.1, 0.9 ] },
        { "name": "f", "type": "dumb_based", "preset": "glossy", "metal": 1.7, "diffuse": [ 1, 2, 3, 4 ] },
        { "name": "g", "type": "dumb_based", "preset": "matte", "metal": -0.5, "diffuse_texture": null,
          "normal_color": [ 0.5, 0.5, 1 ], "alpha_cutout_threshold": 0.25 },
        { "type": "dumb_based", "preset": "gold", "fresnel": [ 0.3, "x", 0.2, 0.1 ] } ],
      "objects": [ { %s, "material": "g" } ] }""" % (OBJ % "cube"),
    # simple_stochastic defaults (normalised by its constructor) and overrides
    "simple_stochastic": """{ "materials": [
        { "name": "a", "type": "simple_stochastic" },
        { "name": "b", "type": "simple_stochastic", "diffuse": 0.7, "smoothness": 0.9 },
        { "name": "c", "type": "simple_stochastic", "color": [ 0.2, 0.3, 0.4 ], "shininess": 64 } ],
      "objects": [ { %s, "material": "b" }, { %s, "material": { "type": "simple_stochastic", "smoothness": 0.2 } } ] }"""
    % (OBJ % "cube", OBJ % "sphere"),
    # light defaults and overrides
    "lights": """{ "lights": [
        { "type": "simple_soft_directional" },
        { "type": "simple_soft_directional", "distance": 10 },
        { "type": "simple_soft_directional", "direction": [ 0, -2, 0.5 ], "softness": 0.9, "color": [ 2, 1, 0.5 ] },
        { "type": "simple_spherical" },
        { "type": "simple_spherical", "position": [ 1 ], "radius": 0.25, "color": [ 3, 3, 3 ] } ],
      "materials": [ { "name": "m", "type": "dumb_based" } ],
      "objects": [ { %s, "material": "m" } ] }""" % (OBJ % "cube"),
    # transforms: rotation about each axis, non-uniform scale, relative position, whole-file object
    "transforms": """{ "materials": [ { "name": "m", "type": "dumb_based" } ],
      "objects": [
        { %s, "material": "m", "transform": { "rotation": [ 33, 0, 0 ] } },
        { %s, "material": "m", "transform": { "rotation": [ 0, -71, 0 ], "position": [ 1, 2, 3 ] } },
        { %s, "material": "m", "transform": { "rotation": [ 12, 34, 56 ], "scale": [ 0.5, 2, -1.5 ],
                                               "relative_position": [ 0.25, -1, 4 ] } },
        { "mesh": { "obj": "m.obj", "object": "cube" }, "material": "m",
          "transform": { "scale": [ 3, 3, 3 ], "position": [ -1, 0, 0 ], "relative_position": [ 1, 1, 1 ] } } ] }"""
    % (OBJ % "cube", OBJ % "sphere", OBJ % "cube"),
    # groups: named and inline, nested, subgroup references with transforms, fallback / override
    "groups": """{ "materials": [ { "name": "m0", "type": "dumb_based" }, { "name": "m1", "type": "simple_stochastic" },
                                 { "name": "m2", "type": "dumb_based", "preset": "gold" } ],
      "groups": [
        { "name": "g0", "elements": [ { %s, "transform": { "position": [ 0, 1, 0 ] } },
                                      { %s, "material": "m2" } ],
          "fallback_material": "m1", "transform": { "rotation": [ 0, 30, 0 ] } },
        { "name": "g1", "elements": [ "g0",
                                      { "group": "g0", "override_material": "m0", "transform": { "scale": [ 2, 2, 2 ] } },
                                      { "elements": [ { %s } ], "fallback_material": "m2", "name": "inner" } ],
          "transform": { "position": [ 5, 0, 0 ] } } ],
      "objects": [ "g1", { "group": "inner", "transform": { "rotation": [ 90, 0, 0 ] } },
                   { "group": "g0", "fallback_material": "m0", "override_material": { "type": "simple_stochastic" } } ] }"""
    % (OBJ % "cube", OBJ % "sphere", OBJ % "cube"),
    # camera: spherical-segment lens with every field, rotated / scaled / offset transform; renderer
    "camera": """{ "materials": [ { "name": "m", "type": "dumb_based" } ],
      "objects": [ { %s, "material": "m" } ],
      "camera": { "lense": { "type": "spherical_segment", "angle": 120, "distance": 7, "sensor": 0.3, "filter": [ 1, 0.5 ] },
                  "transform": { "position": [ 1, 2, 3 ], "rotation": [ 10, 200, -30 ], "scale": [ 1, 2, 1 ],
                                 "relative_position": [ 0, 0, -5 ] } },
      "renderer": { "resources": { "cpu": 3, "gpu": 1, "gpu_0": 1 }, "blocks": { "cpu_cut": 2, "gpu_cut": 8,
                    "force_host_block_synchronisation": false },
                    "pixel": { "boxing": "max", "bounces": 5, "samples_per_pixel": [ 2, 3 ], "pixels_per_gpu_thread": 4,
                               "ignore_backfaces": false } } }""" % (OBJ % "sphere"),
    # a lens without an angle, no transform; a camera without a lens keeps the default lens
    "lens_defaults": """{ "materials": [ { "name": "m", "type": "dumb_based" } ],
      "objects": [ { %s, "material": "m" } ],
      "camera": { "lense": { "type": "simple_stochastic" } },
      "renderer": { "pixel": { "boxing": "min" } } }""" % (OBJ % "cube"),
    # fresnel_color (engine colours, colour override, an unknown engine colour the reference ignores)
    # and spotlights (defaults, target, folded angles, sphere emitter, no shadows, sample clamping,
    # an unknown emitter shape the reference ignores)
    "fresnel_and_spotlight": """{ "materials": [
        { "name": "f0", "type": "fresnel_color" },
        { "name": "f1", "type": "fresnel_color", "engine_color": "copper" },
        { "name": "f2", "type": "fresnel_color", "engine_color": "silver", "color": [ 0.5, 0.6, 0.7 ] },
        { "name": "f3", "type": "fresnel_color", "engine_color": "unobtainium", "texture": null },
        { "name": "f4", "type": "fresnel_color", "engine_color": "iron" },
        { "name": "f5", "type": "fresnel_color", "engine_color": "gold" },
        { "name": "f6", "type": "fresnel_color", "engine_color": "aluminum" } ],
      "lights": [
        { "type": "spotlight" },
        { "type": "spotlight", "color": [ 1, 0.5, 0.2 ], "luminosity": 300, "position": [ 1, 2, 3 ], "target": [ 0, 0, 0 ],
          "hotspot_angle": 20, "falloff_angle": 10, "falloff_power": 2, "emitter_size": 0.5, "emitter_shape": "sphere",
          "cast_shadows": false, "sample_count": 40 },
        { "type": "spotlight", "direction": [ 0, -1, 0.2 ], "hotspot_angle": -30, "falloff_angle": 200, "emitter_size": 0,
          "emitter_shape": "cone", "sample_count": -2 },
        { "type": "spotlight", "hotspot_angle": 250, "falloff_angle": -5, "direction": [ 3, 0, 0 ], "sample_count": 7 } ],
      "objects": [ { %s, "material": "f1" } ] }""" % (OBJ % "cube"),
    "no_camera": """{ "materials": [ { "name": "m", "type": "dumb_based" } ],
      "objects": [ { %s, "material": "m" } ], "camera": { "transform": { "rotation": [ 0, 90, 0 ] } } }"""
    % (OBJ % "cube"),
}


@need_ref
@pytest.mark.parametrize("name", sorted(VARIANTS))
def test_variants_match_reference_loader(tmp_path, name):
    _assert_matches_reference(_scene_dir(tmp_path, VARIANTS[name]))


@need_ref
def test_include_and_relative_paths(tmp_path):
    """Includes resolve against the including file's directory (then the working directory); the
    included file's OBJ paths against its own directory; materials carry over by name."""
    sub = """{ "materials": [ { "name": "shared", "type": "dumb_based", "preset": "glossy" } ],
              "objects": [ { "mesh": { "obj": "../m.obj", "object": "sphere" }, "material": "shared" } ],
              "camera": { "lense": { "type": "simple_stochastic", "angle": 33 } } }"""
    main = """{ "include": [ "lib/sub.dumb" ],
               "objects": [ { %s, "material": "shared", "transform": { "position": [ 0, 3, 0 ] } } ],
               "renderer": { "pixel": { "bounces": 1 } } }""" % (OBJ % "cube")
    _assert_matches_reference(_scene_dir(tmp_path, main, {"lib/sub.dumb": sub}))


ERRORS = [
    ("[ 1, 2 ]", "dictionary"),
    ('{ "materials": [ { "type": "velvet" } ] }', "unknown material type"),
    ('{ "materials": [ { "name": "x" } ] }', "has to have a type"),
    ('{ "materials": [ { "type": "dumb_based", "preset": "shiny" } ] }', "preset"),
    ('{ "materials": [ { "type": "dumb_based", "specular": "high" } ] }', "number"),
    ('{ "materials": [ { "type": "dumb_based", "diffuse": 0.5 } ] }', "array"),
    ('{ "lights": [ { "type": "laser" } ] }', "unknown light type"),
    ('{ "objects": [ { %s } ] }' % (OBJ % "cube"), "material"),
    ('{ "objects": [ { %s, "material": "nope" } ] }' % (OBJ % "cube"), "not found"),
    ('{ "objects": [ { "mesh": { "obj": "m.obj", "object": "torus" }, "material": { "type": "dumb_based" } } ] }',
     "not found"),
    ('{ "objects": [ { "mesh": { "obj": "missing.obj" }, "material": { "type": "dumb_based" } } ] }', "could not read"),
    ('{ "objects": [ "nogroup" ] }', "not found"),
    ('{ "camera": { "lense": { "type": "fisheye" } } }', "unknown lense type"),
    ('{ "camera": { "lense": { "type": "simple_stochastic", "angle": "wide" } } }', "number"),
    ('{ "renderer": { "pixel": { "boxing": "diagonal" } } }', "boxing"),
    ('{ "renderer": { "pixel": { "samples_per_pixel": [ 2 ] } } }', "samples_per_pixel"),
    ('{ "renderer": { "resources": { "cpu": "most" } } }', "cpu"),
    ('{ "materials": [], "materials": [] }', "duplicate"),
    ('{ "materials": [ 1, ] }', ""),
    ('{ "materials": [ { "type": "dumb_based", "diffuse_texture": { "png": "t.png" } } ] }', "could not read"),
    ('{ "materials": [ { "type": "dumb_based", "fresnel_texture": "named" } ] }', "not found"),
    ('{ "materials": [ { "type": "dumb_based", "diffuse_texture": { "name": "x" } } ] }', "incomplete"),
    ('{ "materials": [ { "type": "dumb_based", "diffuse_texture": [ 1 ] } ] }', "texture"),
    ('{ "a": tru }', "categor"),
]


@pytest.mark.parametrize("text,needle", ERRORS)
def test_errors(tmp_path, text, needle):
    path = _scene_dir(tmp_path, text)
    with pytest.raises(dr.DumbRayError) as e:
        dr.load_scene_file(path)
    assert needle in str(e.value)
    if O.reference_available() and hasattr(O.reference(), "dref_dumb_load"):
        with pytest.raises(O.RefSceneFileError):
            O.ref_scene_file_dump(path)


@pytest.mark.parametrize("text,needle", [
    # the reference leaves primitives unimplemented (and dereferences a missing mesh afterwards)
    ('{ "objects": [ { "mesh": { "primitive": "sphere" }, "material": { "type": "dumb_based" } } ] }', "primitive"),
    # containers nested deeper than 512 (the reference's recursive parser has no bound)
    ('{ "a": ' + '[' * 600 + ']' * 600 + ' }', "nested"),
    # the reference recurses without end on a self-include and crashes on a non-string include
    ('{ "include": [ "s.dumb" ] }', "nested"),
    ('{ "include": [ 3 ] }', "string"),
])
def test_unsupported_fail_clearly(tmp_path, text, needle):
    with pytest.raises(dr.DumbRayError) as e:
        dr.load_scene_file(_scene_dir(tmp_path, text))
    assert needle in str(e.value)


def test_parser_details(tmp_path):
    """Dson quirks: numbers are the decimal prefix of a token, string escapes, empty containers,
    texture entries that are null / bool / number mean "no texture"."""
    text = r"""{ "materials": [ { "name": "q\"\\\/\t", "type": "dumb_based", "specular": 12.5abc, "metal": +0.25,
                                "diffuse_texture": false, "fresnel_texture": 7, "normal_texture": null } ],
                 "lights": [], "groups": [],
                 "objects": [ { "mesh": { "obj": "m.obj", "object": "cube" }, "material": "q\"\\/\t" } ] }"""
    f = dr.load_scene_file(_scene_dir(tmp_path, text))
    assert len(f.materials) == 1 and len(f.lights) == 0 and len(f.tris) == 12
    m = f.materials[0]
    assert m.type == dr.MAT_DUMB_BASED and m.specular == 12.5 and m.metal == 0.25
    assert (f.mat_id == 0).all()


def test_scene_file_arrays_and_scene(tmp_path):
    """Defaults of a minimal file (reference DumbRenderContext constructor: height boxing, 2 bounces,
    1x1 samples, backfaces ignored; SimpleStochasticLense(64) when no lens is given) and the scene
    built from it."""
    f = dr.load_scene_file(_scene_dir(tmp_path, VARIANTS["no_camera"]))
    p = f.params
    assert (p.mode, p.boxing, p.max_bounces, p.samples_x, p.samples_y, p.cull_backfaces) == (
        dr.MODE_REFERENCE, dr.BOXING_HEIGHT, 2, 1, 1, 1)
    assert f.camera.lens == dr.LENS_SIMPLE_STOCHASTIC and f.camera.angle[0] == 64.0 and f.camera.origin_rows == 1
    q = f.render_params(64, 48, iteration=3, seed=7)
    assert (q.width, q.height, q.iteration, q.seed) == (64, 48, 3, 7)
    # rotation by 90 degrees about y: the point transform's rows are the transpose of the direction basis
    R = np.array([list(f.camera.right), list(f.camera.up), list(f.camera.forward)], np.float64).T
    rows = np.array([list(f.camera.row_x), list(f.camera.row_y), list(f.camera.row_z)], np.float64)
    assert np.allclose(rows, R.T, atol=1e-6) and not np.allclose(rows, R, atol=1e-3)


@need_ref
def test_oracle_render_matches_reference_statistically():
    """The CPU oracle renders the scene file our loader read; the reference renders the same file
    read by its own loader (golden fixture: 4 runs x 512 iterations).  Run means agree within the
    Monte Carlo noise."""
    from _stats import compare_runs
    g = np.load(GOLD / "render_scene_file.npz")
    W, H = int(g["width"]), int(g["height"])
    f = dr.load_scene_file(GOLD / "scene_file" / "scene.dumb")
    osc = O.OracleScene(f.tris, normals=f.normals, mat_id=f.mat_id, materials=f.materials, lights=f.lights)
    runs = []
    for seed in range(4):
        p = f.render_params(W, H, seed=seed)
        p.samples_x, p.samples_y = 16, 32
        runs.append(dr.blockmajor_to_image(osc.render_blocks(f.camera, p), W, H))
    compare_runs(runs, g["runs"])


def test_fixture_files_are_current(tmp_path):
    """The committed scene-file fixture is what make_golden.py writes."""
    path = write_scene_file(tmp_path)
    for name in ("scene.dumb", "materials.dumb", "props.obj"):
        assert (path.parent / name).read_text() == (GOLD / "scene_file" / name).read_text(), name


@need_ref
def test_whole_file_item_matches_reference_as_a_set(tmp_path):
    """An item that names no OBJ object takes every object of the file; the reference visits them in
    its hash map's order, the loader in file order, so the triangle sets are compared."""
    text = """{ "materials": [ { "name": "m", "type": "dumb_based" } ],
               "objects": [ { "mesh": { "obj": "m.obj" }, "material": "m", "transform": { "rotation": [ 5, 10, 15 ] } } ] }"""
    path = _scene_dir(tmp_path, text)
    ref = O.ref_scene_file_dump(path)
    ours = O.scene_file_dump(dr.load_scene_file(path))

    def rows(d):
        a = np.concatenate([d["xyz"].view(np.uint32), d["nrm"].view(np.uint32), d["mat"][:, None].view(np.uint32)], 1)
        return a[np.lexsort(a.T[::-1])]

    assert np.array_equal(rows(ref), rows(ours))


@need_ref
def test_textured_fixture_matches_reference_loader():
    """PNG textures by path and by name (and a path looked up as a name), nearest / bilinear
    filtering, tilings, offsets, a normal map, an alpha cutout, a textured fresnel_color; texture
    coordinates from the OBJ: material texture channels, texture coordinates and decoded texels
    equal the reference loader's (lodepng, bytes / 255)."""
    _assert_matches_reference(GOLD / "scene_file_tex" / "scene.dumb")


@need_ref
def test_oracle_renders_textured_scene_file_like_reference():
    from _stats import compare_runs
    g = np.load(GOLD / "render_scene_file_tex.npz")
    W, H = int(g["width"]), int(g["height"])
    f = dr.load_scene_file(GOLD / "scene_file_tex" / "scene.dumb")
    osc = O.OracleScene(f.tris, normals=f.normals, mat_id=f.mat_id, materials=f.materials, lights=f.lights)
    osc.set_textures(f.textures, f.uv)
    runs = []
    for seed in range(4):
        p = f.render_params(W, H, seed=seed)
        p.samples_x, p.samples_y = 16, 32
        runs.append(dr.blockmajor_to_image(osc.render_blocks(f.camera, p), W, H))
    compare_runs(runs, g["runs"])


def test_textured_fixture_files_are_current(tmp_path):
    path = write_scene_file_textured(tmp_path)
    for name in ("scene.dumb", "textured.obj", "checker.png", "noise.png", "bumps.png", "stripes.png"):
        assert (path.parent / name).read_bytes() == (GOLD / "scene_file_tex" / name).read_bytes(), name
