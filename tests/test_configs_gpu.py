"""Parity at the benchmarked configurations' own sizes.

C2 (ray-cast microbenchmark): the level-8 displaced icosphere (1,310,720 triangles, amplitude 0.1,
seed 1) on the reference's octree; dr_cast against the oracle over 1Mi of the benchmark's incoherent
rays plus all 2,073,600 of its 1920x1080 primaries, and against the reference's own Octree::cast on
the golden subset (tests/golden/cast_c2_l8.npz), culling on and off.  The parity rule: hit index
equal to the reference's, except grazing ties (both hit, t within T_EPS relative) counted and capped
at TIE_CAP of the rays; t within T_EPS relative where the index agrees (the kernels are bit-exact,
which the test reports).

C1 (plain path trace, 256x256, 16 spp, depth 4): the physical estimator against the FP64 oracle
(same counter-based random numbers) at 64 spp (four blended iterations of 16 spp); the
reference-expressible twin in reference mode against the oracle per pixel and against four
reference DumbRenderer runs (tests/golden/render_c1_twin.npz) statistically.

C3 (the full path-trace scene): its reference-expressible twin (the level-8 displaced icosphere on a
ground plane, DumbBased diffuse / metal and SimpleStochastic mirror materials, 4 spherical lights,
depth 8), the benchmark's view at 96x54, in reference mode against four reference DumbRenderer runs
(tests/golden/render_c3_twin.npz) statistically."""
from pathlib import Path
import sys

import numpy as np
import pytest
import torch

import dumbray_gb300 as dr
from dumbray_gb300 import scenes
import _oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLD))
from make_golden import C1_DEPTH, C1_SIZE, C3_DEPTH, C3_H, C3_W, c1_twin, c2_rays, c3_twin, mesh_sha256  # noqa: E402

pytestmark = pytest.mark.gpu

T_EPS = 1e-5      # relative t tolerance of a grazing tie and of an agreeing hit
TIE_CAP = 1e-5    # ties allowed, as a fraction of the rays


def _cast(scene, o, d, cuda, cull):
    to = torch.from_numpy(np.ascontiguousarray(o, np.float32)).to(cuda)
    td = torch.from_numpy(np.ascontiguousarray(d, np.float32)).to(cuda)
    idx, t = dr.cast(scene, to, td, cull_backfaces=cull)
    torch.cuda.synchronize()
    return idx.cpu().numpy(), t.cpu().numpy()


def cast_parity(idx, t, ref_idx, ref_t):
    """(ties, other mismatches, bit-exact) of a cast against a reference cast."""
    diff = idx != ref_idx
    both = diff & (idx >= 0) & (ref_idx >= 0)
    rt = ref_t.astype(np.float64)
    close = np.abs(t.astype(np.float64) - rt) <= T_EPS * np.abs(rt)
    ties = both & close
    same = ~diff & (ref_idx >= 0)
    bad = int((diff & ~ties).sum()) + int((same & ~close).sum())
    miss_ok = np.all(t[~diff & (ref_idx < 0)] == np.finfo(np.float32).max)
    exact = not diff.any() and np.array_equal(t[same].view(np.int32), ref_t[same].view(np.int32))
    return int(ties.sum()), bad + (0 if miss_ok else 1), exact


def _check(idx, t, ref_idx, ref_t, what):
    ties, bad, exact = cast_parity(idx, t, ref_idx, ref_t)
    print(f"{what}: {len(idx):,} rays, ties {ties}, mismatches {bad}, bit-exact {exact}")
    assert bad == 0, f"{what}: {bad} mismatches beyond the tie rule"
    assert ties <= TIE_CAP * len(idx), f"{what}: {ties} ties > {TIE_CAP} of {len(idx)} rays"


@pytest.fixture(scope="module")
def c2_mesh():
    return scenes.displaced_icosphere(8, 0.1, 1)


def test_c2_level8_casts_match_reference_golden(cuda, c2_mesh):
    """The reference's own Octree::cast on the level-8 mesh (golden subset: 8,192 incoherent rays and
    8,100 primaries): same node count, same hits."""
    g = np.load(GOLD / "cast_c2_l8.npz")
    assert mesh_sha256(c2_mesh) == str(g["mesh_sha256"]), "level-8 mesh differs from the fixture's"
    o, d = c2_rays()
    assert np.array_equal(o, g["o"]) and np.array_equal(d, g["d"])
    sc = dr.Scene(c2_mesh)
    assert sc.stats()["nodes"] == int(g["nodes"])
    for cull in (1, 0):
        idx, t = _cast(sc, o, d, cuda, bool(cull))
        _check(idx, t, g[f"idx_cull{cull}"], g[f"t_cull{cull}"], f"C2 L8 vs reference, cull {cull}")


def test_c2_level8_casts_match_oracle_full_primary_frame(cuda, c2_mesh):
    """1Mi incoherent rays (the benchmark's distribution, seed 0) and every 1920x1080 primary ray."""
    sc = dr.Scene(c2_mesh)
    osc = O.OracleScene(c2_mesh, threads=16)
    assert sc.stats()["nodes"] == osc.node_count()
    oi, di = scenes.incoherent_rays(1 << 20, -1.1, 1.1, seed=0)
    op, dp = scenes.primary_rays(1920, 1080, 60.0, (0.0, 0.3, -3.0), (0.0, 0.0, 0.0))
    o, d = np.concatenate([oi, op]), np.concatenate([di, dp])
    for cull in (True, False):
        idx, t = _cast(sc, o, d, cuda, cull)
        ri, rt, _, _ = osc.cast(o, d, cull=cull, threads=16)
        _check(idx, t, ri, rt, f"C2 L8 vs oracle, cull {int(cull)}")
        assert (ri >= 0).mean() > 0.1


def _c1_physical():
    c = scenes.box_and_icosphere(5)
    mats = [dr.lambert((0.7, 0.7, 0.7)), dr.lambert((0.7, 0.1, 0.1)),
            dr.lambert((0.0, 0.0, 0.0), emission=(10.0, 10.0, 10.0))]
    return c["tris"], c["mat_id"], mats


def c1_physical_vs_fp64(cuda, box_eps, iterations=4):
    """(relative RMSE, mean relative difference) of the GPU against the FP64 oracle after 1 and after
    `iterations` blended iterations of 16 spp, 256x256, depth 4, pinhole 60 degrees, seed 0."""
    tris, mat, mats = _c1_physical()
    sc = dr.Scene(tris, mat_id=mat, materials=mats, box_epsilon=box_eps)
    osc = O.OracleScene(tris, mat_id=mat, materials=mats, threads=16)
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.99), angle=60.0)
    W = H = C1_SIZE
    nb = dr.block_count(W, H)
    fb = dr.new_frame_buffer(W, H, cuda)
    ofb = np.zeros((nb * 128, 4), np.float32)
    r = dr.Renderer(1 << 20)
    out = []
    for it in range(1, iterations + 1):
        p = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(4, 4), max_bounces=C1_DEPTH, iteration=it, seed=0)
        r.render_blocks(sc, cam, fb, 0, nb, p)
        osc.render_blocks(cam, p, fb=ofb, threads=16)
        torch.cuda.synchronize()
        if it in (1, iterations):
            g = fb.cpu().numpy()[:, :3].astype(np.float64)
            o = ofb[:, :3].astype(np.float64)
            m = max(o.mean(), 1e-9)
            out.append((16 * it, float(np.sqrt(np.mean((g - o) ** 2)) / m), float((g.mean() - o.mean()) / m)))
    r.close()
    return out


@pytest.mark.parametrize("box_eps", [0.0, dr.PHYSICAL_TREE])
def test_c1_physical_matches_fp64_oracle(cuda, box_eps):
    """Per-pixel relative RMSE (RMSE over the image / its mean) within 1% at 64 spp; image means within
    0.2%.  The same random numbers drive both sides, so the RMSE measures float-vs-double divergence
    of individual paths, which averages out as 1/sqrt(spp)."""
    res = c1_physical_vs_fp64(cuda, box_eps)
    for spp, rmse, dm in res:
        print(f"C1 physical vs FP64 oracle ({'physical' if box_eps else 'reference'} tree): {spp} spp, "
              f"relative RMSE {rmse:.4%}, mean difference {dm:+.4%}")
    spp, rmse, dm = res[-1]
    assert rmse <= 0.01, rmse
    assert abs(dm) <= 2e-3, dm


def test_c1_twin_reference_mode_matches_oracle(cuda):
    """Reference semantics at the C1 size: the GPU and the oracle follow the same paths (same random
    numbers); per pixel equal up to float rounding of transcendentals."""
    tris, mat, mats, lights, cam = c1_twin()
    sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights)
    osc = O.OracleScene(tris, mat_id=mat, materials=mats, lights=lights, threads=16)
    W = H = C1_SIZE
    p = dr.render_params(W, H, dr.MODE_REFERENCE, samples=(4, 4), max_bounces=C1_DEPTH, seed=5)
    fb = dr.new_frame_buffer(W, H, cuda)
    r = dr.Renderer(1 << 20)
    r.render_blocks(sc, cam, fb, 0, dr.block_count(W, H), p)
    torch.cuda.synchronize()
    g = fb.cpu().numpy()[:, :3].astype(np.float64)
    o = osc.render_blocks(cam, p, threads=16)[:, :3].astype(np.float64)
    bad = np.abs(g - o) > 2e-3 * np.maximum(np.abs(o), 0.01)
    print(f"C1 twin reference mode vs oracle: {bad.mean():.5f} of channels differ by > 2e-3 relative")
    assert np.isfinite(g).all()
    assert bad.mean() <= 0.02
    assert abs(g.mean() - o.mean()) / max(o.mean(), 1e-9) <= 5e-3
    r.close()


def test_c1_twin_matches_reference_renderer_statistically(cuda):
    """8 GPU runs of 64 spp (8x8 sub-pixels) against four reference DumbRenderer runs of 64 iterations
    (golden fixture) over all 65,536 pixels: MSE of the run means within 1.5x of the variance the runs
    predict, image means within 4 standard errors."""
    from _stats import compare_runs
    g = np.load(GOLD / "render_c1_twin.npz")
    assert int(g["size"]) == C1_SIZE and int(g["bounces"]) == C1_DEPTH
    tris, mat, mats, lights, cam = c1_twin()
    sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights)
    W = H = C1_SIZE
    r = dr.Renderer(1 << 22)
    runs = []
    for seed in range(200, 208):
        p = dr.render_params(W, H, dr.MODE_REFERENCE, samples=(8, 8), max_bounces=C1_DEPTH, seed=seed)
        fb = dr.new_frame_buffer(W, H, cuda)
        r.render_blocks(sc, cam, fb, 0, dr.block_count(W, H), p)
        torch.cuda.synchronize()
        runs.append(dr.blockmajor_to_image(fb, W, H)[..., :3])
    r.close()
    ratio, dm_se = compare_runs(runs, g["runs"].astype(np.float32))
    print(f"C1 twin vs reference DumbRenderer: MSE / expected {ratio:.3f}, mean difference {dm_se:+.2f} SE")


def test_c3_twin_matches_reference_renderer_statistically(cuda):
    """8 GPU runs of 256 spp (16x16 sub-pixels) against four reference DumbRenderer runs of 256
    iterations of the full path-trace scene's twin (1,310,722 triangles, depth 8): MSE of the run
    means within 1.5x of the variance the runs predict, image means within 4 standard errors."""
    from _stats import compare_runs
    g = np.load(GOLD / "render_c3_twin.npz")
    assert int(g["width"]) == C3_W and int(g["height"]) == C3_H and int(g["bounces"]) == C3_DEPTH
    tris, mat, mats, lights, cam = c3_twin()
    sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights, device_build=True)
    r = dr.Renderer(1 << 22)
    runs = []
    for seed in range(300, 308):
        p = dr.render_params(C3_W, C3_H, dr.MODE_REFERENCE, samples=(16, 16), max_bounces=C3_DEPTH, seed=seed)
        fb = dr.new_frame_buffer(C3_W, C3_H, cuda)
        r.render_blocks(sc, cam, fb, 0, dr.block_count(C3_W, C3_H), p)
        torch.cuda.synchronize()
        runs.append(dr.blockmajor_to_image(fb, C3_W, C3_H)[..., :3])
    r.close()
    sc.close()
    ratio, dm_se = compare_runs(runs, g["runs"].astype(np.float32))
    print(f"C3 twin vs reference DumbRenderer: MSE / expected {ratio:.3f}, mean difference {dm_se:+.2f} SE")
