"""Path-replay adjoint (dr_render_adjoint): gradients of an L2 image loss with respect to
per-triangle albedo and emission, checked against central finite differences with common random
numbers on the GPU (same seeds, parameters written in place so the sampling tables stay fixed:
the forward estimator is then a smooth function of the parameters) and against finite differences
of the FP64 CPU oracle.  Tolerance: 1e-2 relative on the checked components."""
import numpy as np
import pytest
import torch

import dumbray_gb300 as dr
from dumbray_gb300 import scenes
import _oracle as O

pytestmark = pytest.mark.gpu

W = H = 32
SPP = (2, 2)
DEPTH = 3


def _setup(cuda):
    c = scenes.box_and_icosphere(2)
    tris = c["tris"]
    n = len(tris)
    mats = [dr.lambert((0.7, 0.7, 0.7)), dr.glossy((0.8, 0.6, 0.4), 0.3), dr.mirror((0.9, 0.9, 0.9))]
    h = scenes.tri_hash_u32(np.arange(n), 2) % 100
    mat = np.where(h < 70, 0, np.where(h < 90, 1, 2)).astype(np.int32)
    lo = c["n_room"] + c["n_sphere"]
    mat[lo:] = 0
    rng = np.random.default_rng(7)
    albedo = rng.uniform(0.2, 0.8, (n, 3)).astype(np.float32)
    emission = np.zeros((n, 3), np.float32)
    emission[lo:] = 10.0
    rough = np.full(n, 0.3, np.float32)
    sc = dr.Scene(tris, mat_id=mat, materials=mats)
    sc.set_triangle_params(albedo, emission, rough)
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.99), angle=60.0)
    p = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=SPP, max_bounces=DEPTH, seed=3)
    target_alb = np.clip(albedo + rng.normal(0, 0.15, albedo.shape), 0.05, 0.95).astype(np.float32)
    return sc, cam, p, tris, mat, mats, albedo, emission, rough, target_alb


def _render(sc, cam, p, cuda):
    fb = dr.new_frame_buffer(W, H, cuda)
    dr.Renderer(1 << 14).render_blocks(sc, cam, fb, 0, dr.block_count(W, H), p)
    torch.cuda.synchronize()
    return fb


def _loss(fb, target):
    d = (fb[:, :3].double() - target[:, :3].double())
    return float((d * d).sum())


def test_adjoint_matches_central_differences_with_common_random_numbers(cuda):
    sc, cam, p, tris, mat, mats, albedo, emission, rough, target_alb = _setup(cuda)
    n = len(tris)
    a_ptr, e_ptr = sc.triangle_params_device()
    alb_dev = dr.device_view(a_ptr, (n, 3), cuda)
    emi_dev = dr.device_view(e_ptr, (n, 3), cuda)
    alb_dev.copy_(torch.from_numpy(target_alb).to(cuda))
    target = _render(sc, cam, p, cuda)
    alb_dev.copy_(torch.from_numpy(albedo).to(cuda))
    img = _render(sc, cam, p, cuda)
    dl = torch.zeros_like(img)
    dl[:, :3] = 2.0 * (img[:, :3] - target[:, :3])
    ga = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    ge = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    dr.Renderer(1 << 14).render_adjoint(sc, cam, dl, 0, dr.block_count(W, H), p, ga, ge)
    torch.cuda.synchronize()
    ga_h, ge_h = ga.cpu().numpy(), ge.cpu().numpy()
    # albedo: the 8 largest-gradient components
    flat = np.argsort(-np.abs(ga_h).ravel())[:8]
    for f in flat:
        k, ch = divmod(int(f), 3)
        hstep = 1e-3
        vals = []
        for sgn in (1, -1):
            alb_dev[k, ch] = float(albedo[k, ch]) + sgn * hstep
            vals.append(_loss(_render(sc, cam, p, cuda), target))
        alb_dev[k, ch] = float(albedo[k, ch])
        fd = (vals[0] - vals[1]) / (2 * hstep)
        assert abs(ga_h[k, ch] - fd) <= 1e-2 * abs(fd) + 1e-6, (k, ch, ga_h[k, ch], fd)
    # emission: both emitter triangles, every channel
    for k in range(n - 2, n):
        for ch in range(3):
            hstep = 1e-2
            vals = []
            for sgn in (1, -1):
                emi_dev[k, ch] = float(emission[k, ch]) + sgn * hstep
                vals.append(_loss(_render(sc, cam, p, cuda), target))
            emi_dev[k, ch] = float(emission[k, ch])
            fd = (vals[0] - vals[1]) / (2 * hstep)
            assert abs(ge_h[k, ch] - fd) <= 1e-2 * abs(fd) + 1e-6, (k, ch, ge_h[k, ch], fd)


def _fd_report(what, rows):
    for name, k, ch, adj, fd in rows:
        print(f"{what}: {name}[{k},{ch}] adjoint {adj:+.6e} fd {fd:+.6e} rel {abs(adj - fd) / max(abs(fd), 1e-12):.2e}")


def test_adjoint_matches_fp64_oracle_finite_differences(cuda):
    """Reference gradient: central differences of the FP64 CPU oracle's loss (same estimator, same
    random numbers, double precision, light-selection table held fixed as on the device) for the 8
    largest albedo components and every channel of the two emitter triangles, within 1e-2 relative.  64 spp: paths whose float and double versions
    diverge (a hit decided differently near an edge) add noise that falls as 1/sqrt(paths)."""
    sc, cam, p, tris, mat, mats, albedo, emission, rough, target_alb = _setup(cuda)
    p = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(8, 8), max_bounces=DEPTH, seed=3)
    n = len(tris)
    osc = O.OracleScene(tris, mat_id=mat, materials=mats, threads=16)
    osc.set_triangle_params(target_alb, emission, rough)
    t_or = osc.render_blocks(cam, p, threads=16).astype(np.float64)
    osc.set_triangle_params(albedo, emission, rough)
    # the device's light-selection table stays as built at scene creation while parameters are
    # written in place; the oracle keeps its own fixed from here, so both differentiate one estimator
    osc.freeze_sampling()
    img_or = osc.render_blocks(cam, p, threads=16).astype(np.float64)
    img = _render(sc, cam, p, cuda)
    # the adjoint weights come from the oracle's image: both sides differentiate the same loss
    dl = torch.zeros_like(img)
    dl[:, :3] = torch.from_numpy(2.0 * (img_or[:, :3] - t_or[:, :3])).float().to(cuda)
    ga = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    ge = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    dr.Renderer(1 << 16).render_adjoint(sc, cam, dl, 0, dr.block_count(W, H), p, ga, ge)
    torch.cuda.synchronize()
    ga_h, ge_h = ga.cpu().numpy(), ge.cpu().numpy()

    def oracle_loss(alb, emi):
        osc.set_triangle_params(alb, emi, rough)
        im = osc.render_blocks(cam, p, threads=16).astype(np.float64)
        return float(((im[:, :3] - t_or[:, :3]) ** 2).sum())

    rows = []
    for f in np.argsort(-np.abs(ga_h).ravel())[:8]:
        k, ch = divmod(int(f), 3)
        vals = []
        for sgn in (1, -1):
            a2 = albedo.copy()
            a2[k, ch] += sgn * 1e-3
            vals.append(oracle_loss(a2, emission))
        rows.append(("albedo", k, ch, float(ga_h[k, ch]), (vals[0] - vals[1]) / 2e-3))
    for k in range(n - 2, n):
        for ch in range(3):
            vals = []
            for sgn in (1, -1):
                e2 = emission.copy()
                e2[k, ch] += sgn * 1e-2
                vals.append(oracle_loss(albedo, e2))
            rows.append(("emission", k, ch, float(ge_h[k, ch]), (vals[0] - vals[1]) / 2e-2))
    _fd_report("32x32 vs FP64 FD", rows)
    for name, k, ch, adj, fd in rows:
        assert abs(adj - fd) <= 1e-2 * abs(fd) + 1e-6, (name, k, ch, adj, fd)


def test_c5_workload_gradient_vs_fp64_oracle_fd(cuda):
    """The differentiable workload itself (icosphere L7 + box room, 327,692 triangles, per-triangle albedo
    U[0.1, 0.9], emission 10 on 64 triangles, 512x512, 16 spp, depth 5) on a 64-block range at the image
    centre (8,192 pixels): adjoint gradients of the L2 loss against central differences (h = 1e-3) of
    the FP64 oracle's loss for the 8 largest albedo components, within 1e-2 relative."""
    S = scenes.differentiable_scene(7)
    tris, n = S["tris"], len(S["tris"])
    mats = [dr.lambert()]
    sc = dr.Scene(tris, mat_id=S["mat_id"], materials=mats, box_epsilon=dr.PHYSICAL_TREE)
    sc.set_triangle_params(S["albedo"], S["emission"], S["roughness"])
    osc = O.OracleScene(tris, mat_id=S["mat_id"], materials=mats, threads=16)
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.99), angle=60.0)
    p = dr.render_params(512, 512, dr.MODE_PHYSICAL, samples=(4, 4), max_bounces=5, seed=7)
    bw = dr.block_count(512, 512) // 32            # blocks per block row (64)
    ranges = [((14 + r) * bw + 16, (14 + r) * bw + 32) for r in range(4)]     # 4 rows x 16 blocks

    def oracle_image():
        fb = np.zeros((dr.block_count(512, 512) * 128, 4), np.float32)
        for s0, s1 in ranges:
            osc.render_blocks(cam, p, fb=fb, start=s0, end=s1, threads=16)
        return fb.astype(np.float64)

    mask = np.zeros(dr.block_count(512, 512) * 128, bool)
    for s0, s1 in ranges:
        mask[s0 * 128:s1 * 128] = True
    osc.set_triangle_params(S["albedo_target"], S["emission"], S["roughness"])
    t_or = oracle_image()
    osc.set_triangle_params(S["albedo"], S["emission"], S["roughness"])
    i_or = oracle_image()
    dl_h = np.zeros((len(mask), 4), np.float32)
    dl_h[mask, :3] = 2.0 * (i_or[mask, :3] - t_or[mask, :3])
    dl = torch.from_numpy(dl_h).to(cuda)
    ga = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    ge = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    rend = dr.Renderer(1 << 18)
    for s0, s1 in ranges:
        rend.render_adjoint(sc, cam, dl, s0, s1, p, ga, ge)
    torch.cuda.synchronize()
    ga_h = ga.cpu().numpy()
    assert float(np.abs(ga_h).sum()) > 0 and float(ge.abs().sum()) > 0
    rows = []
    for f in np.argsort(-np.abs(ga_h).ravel())[:8]:
        k, ch = divmod(int(f), 3)
        vals = []
        for sgn in (1, -1):
            a2 = S["albedo"].copy()
            a2[k, ch] += sgn * 1e-3
            osc.set_triangle_params(a2, S["emission"], S["roughness"])
            im = oracle_image()
            vals.append(float(((im[mask, :3] - t_or[mask, :3]) ** 2).sum()))
        rows.append(("albedo", k, ch, float(ga_h[k, ch]), (vals[0] - vals[1]) / 2e-3))
    _fd_report("C5 workload vs FP64 FD", rows)
    for name, k, ch, adj, fd in rows:
        assert abs(adj - fd) <= 1e-2 * abs(fd) + 1e-6, (name, k, ch, adj, fd)


def test_autograd_harness(cuda):
    """torch.autograd.Function over the C ABI: backward equals a direct dr_render_adjoint call."""
    sc, cam, p, tris, mat, mats, albedo, emission, rough, target_alb = _setup(cuda)
    n = len(tris)
    alb = torch.from_numpy(albedo).to(cuda).requires_grad_(True)
    emi = torch.from_numpy(emission).to(cuda).requires_grad_(True)
    target = torch.zeros((dr.block_count(W, H) * 128, 4), device=cuda)
    img = dr.render_differentiable(sc, cam, p, alb, emi)
    loss = ((img[:, :3] - target[:, :3]) ** 2).sum()
    loss.backward()
    dl = torch.zeros_like(img)
    dl[:, :3] = 2.0 * img.detach()[:, :3]
    ga = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    ge = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    dr.Renderer(1 << 14).render_adjoint(sc, cam, dl, 0, dr.block_count(W, H), p, ga, ge)
    torch.cuda.synchronize()
    assert torch.allclose(alb.grad, ga, rtol=1e-4, atol=1e-7)
    assert torch.allclose(emi.grad, ge, rtol=1e-4, atol=1e-7)
    assert float(alb.grad.abs().sum()) > 0 and float(emi.grad.abs().sum()) > 0


def test_adjoint_rejects_reference_mode(cuda):
    room = scenes.box((2, 2, 2), inward=True)
    sc = dr.Scene(room, materials=[dr.dumb_based()], lights=[dr.spherical_light((1, 1, 1), (0, 0.5, 0), 0.1)])
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.9))
    p = dr.render_params(16, 16, dr.MODE_REFERENCE)
    fb = dr.new_frame_buffer(16, 16, cuda)
    g = torch.zeros((len(room), 3), device=cuda)
    with pytest.raises(dr.DumbRayError):
        dr.Renderer(1 << 12).render_adjoint(sc, cam, fb, 0, 2, p, g, g)


def test_adjoint_over_concurrent_lanes_equals_one_lane(cuda):
    """The adjoint pass runs its waves on the renderer's concurrent lanes, each with its own prefix
    buffer.  The C5 workload's full frame (4.2M paths: four 1Mi-path waves) with 4 lanes gives the
    gradients of one lane, up to the order of the float atomic additions."""
    S = scenes.differentiable_scene(7)
    tris, n = S["tris"], len(S["tris"])
    sc = dr.Scene(tris, mat_id=S["mat_id"], materials=[dr.lambert()], box_epsilon=dr.PHYSICAL_TREE)
    sc.set_triangle_params(S["albedo"], S["emission"], S["roughness"])
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.99), angle=60.0)
    p = dr.render_params(512, 512, dr.MODE_PHYSICAL, samples=(4, 4), max_bounces=5, seed=7)
    nb = dr.block_count(512, 512)
    dl = torch.zeros((nb * 128, 4), dtype=torch.float32, device=cuda)
    dl[:, :3] = 1.0
    grads = {}
    for run, lanes in (("one", 1), ("one_again", 1), ("four", 4)):
        rend = dr.Renderer(1 << 20)
        rend.set_lanes(lanes)
        ga = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
        ge = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
        rend.render_adjoint(sc, cam, dl, 0, nb, p, ga, ge)
        torch.cuda.synchronize()
        grads[run] = (ga.cpu().numpy().astype(np.float64), ge.cpu().numpy().astype(np.float64))
        rend.close()
    # The gradients are float32 atomic sums of millions of small terms: the largest components (the
    # walls' albedo, ~10) take terms far below their ulp's worth of precision, so another order of
    # the additions moves them by parts in 1e4 (two one-lane runs, whose order stays the same in
    # practice, agree closely; four lanes interleave the waves: measured 1.7e-3 relative L2).  A lane
    # that lost or doubled its wave would move the gradient by ~25%.
    def rel_l2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))
    for k in range(2):
        one, again, four = grads["one"][k], grads["one_again"][k], grads["four"][k]
        assert np.abs(one).sum() > 0
        assert rel_l2(again, one) <= 5e-3, rel_l2(again, one)
        assert rel_l2(four, one) <= 5e-3, rel_l2(four, one)
        big = np.abs(one) > 1e-3 * np.abs(one).max()
        worst = float((np.abs(four - one)[big] / np.abs(one)[big]).max())
        assert worst <= 2e-2, worst
