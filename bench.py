"""Benchmark: Mpaths/s of the full path trace at 1920x1080, 64 spp, depth 8 on one GB300.

Workload (synthetic, seeded; no dataset): icosphere level 8 (1,310,720 triangles) radially displaced
by 3-octave value noise (amplitude 0.1, seed 1) on a 2-triangle ground plane, lit by 4 emissive
quads; materials by triangle-index hash (60% Lambert albedo U[0.2,0.8]^3, 25% mirror, 15% GGX
glossy roughness U[0.05,0.4]); pinhole 60 degrees.  One step = one full frame (132,710,400 paths)
rendered through dr_render_blocks into the block-major float4 frame buffer.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` = paths of all ranks / max-over-ranks device time of the K
timed steps (inputs resident in HBM).  `e2e` = the same through the public API with the frame buffer
copied host->device before and device->host after every step (pinned host memory).  `roofline`
describes the dominant kernel (k_trace): algorithmic bytes per launch = rays x (40 + 32 C_box +
36 C_tri) with C_box / C_tri the reference traversal's mean child-box / triangle tests per ray
(counted in an untimed pass), divided by its CUDA-event launch time measured over the timed region.
N > 1: every rank renders its own frame of distinct samples (weak scaling, no collective on the data
path).  `--impl reference` times the reference DumbRenderer on host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpaths/s 1080p 64spp on 1 GB300: plain vs batched, fwd vs fwd+adjoint, at RMSE"
# DRAM bytes (read + write) per extension ray of k_trace: ncu dram__bytes_read.sum + dram__bytes_write.sum
# of the bounce-1 launch of a 960x544, 4 spp frame of the same scene, camera and octree rendered as one
# wave (458.9 MB over its 1,375,097 rays, caches flushed before the launch); the `traffic` of an average
# full-size launch is this times its ray count.
TRACE_DRAM_BYTES_PER_RAY = 333.7
UNIT = "Mpaths/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--depth", type=int, default=8)
    ap.add_argument("--level", type=int, default=8)
    ap.add_argument("--lens", default="pinhole", choices=["pinhole", "fisheye", "spherical"])
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--wave", type=int, default=1 << 24,
                    help="paths per wave (renderer capacity); 16Mi: about 5 GB of scratch per lane")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer e2e pass (profiling cases)")
    ap.add_argument("--no-count", action="store_true", help="skip the traversal-counting pass (profiling cases)")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-scene batched leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable (adjoint) leg")
    ap.add_argument("--no-raycast", action="store_true", help="skip the ray-cast microbenchmark leg")
    ap.add_argument("--no-twin", action="store_true", help="skip the reference-mode twin leg")
    ap.add_argument("--no-c1", action="store_true", help="skip the 256x256 plain path-trace leg")
    ap.add_argument("--raycast-only", action="store_true",
                    help="profiling case: run only the ray-cast microbenchmark leg and print it")
    ap.add_argument("--twin-only", action="store_true",
                    help="profiling case: run only the reference-mode twin leg (at --twin-size / --twin-spp) and print it")
    ap.add_argument("--twin-size", default="1920x1080", help="reference-mode twin resolution WxH")
    ap.add_argument("--twin-spp", type=int, default=64, help="reference-mode twin samples per pixel (a square)")
    ap.add_argument("--twin-tree", default="reference", choices=["reference", "physical"],
                    help="octree padding of the reference-mode twin scene")
    ap.add_argument("--lanes", type=int, default=8,
                    help="concurrent wave pipelines per renderer (0 = the library default, 4; path trace at 16Mi-path "
                         "waves: 4 lanes 788.5, 6 791.6, 8 798.3 Mpaths/s)")
    ap.add_argument("--split", type=int, default=4,
                    help="octree leaf split threshold of the path-trace scene (4: with 3 the best of 2-24 on this "
                         "workload with the physical-mode padding and the refitted group-test planes; the "
                         "reference uses 8)")
    ap.add_argument("--ref-tree", action="store_true",
                    help="build the path-trace scene with the reference's octree padding (1.28e-3) instead of the "
                         "physical-mode padding scaled to the coordinates")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=5, help="timed steps of each batched arm")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def samples_xy(spp):
    sx = int(round(spp ** 0.5))
    while spp % sx:
        sx -= 1
    return sx, spp // sx


def build_scene(dr, level, split=0, ref_tree=False):
    from dumbray_gb300 import scenes
    S = scenes.full_scene(level=level, seed=1)
    mats = [dr.lambert(), dr.mirror(), dr.glossy()]
    t0 = time.time()
    S["box_epsilon"] = 0.0 if ref_tree else dr.tight_box_epsilon(S["tris"])
    S["split"] = 8 if ref_tree else (split if split > 0 else 8)   # the reference's tree: its split rule and 8
    scene = dr.Scene(S["tris"], mat_id=S["mat_id"], materials=mats, split_threshold=S["split"],
                     box_epsilon=0.0 if ref_tree else dr.PHYSICAL_TREE, device_build=True)
    scene.set_triangle_params(S["albedo"], S["emission"], S["roughness"])
    return S, scene, time.time() - t0


def make_camera(dr, lens):
    pos, target = (0.0, 0.6, -3.4), (0.0, -0.15, 0.0)
    if lens == "fisheye":
        return dr.camera(dr.LENS_FISHEYE, position=pos, target=target, angle=(180.0, 180.0))
    if lens == "spherical":
        return dr.camera(dr.LENS_SPHERICAL, position=pos, target=target, angle=(200.0, 180.0))
    return dr.camera(dr.LENS_PINHOLE, position=pos, target=target, angle=(60.0, 60.0))


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def octree_build_times(dr, S):
    """Wall time of the octree build alone (dr_octree_create_host + export) on the host threads and on
    the GPU (device_build, same tree), for the path-trace scene's parameters."""
    out = {}
    for name, dev in (("host_threads", False), ("device", True)):
        dr.build_octree_host(S["tris"][:1000], device_build=dev)   # warm-up (allocator, first launch)
        t0 = time.time()
        st = dr.build_octree_host(S["tris"], split_threshold=S["split"], box_epsilon=S["box_epsilon"],
                                  device_build=dev)[0]
        out[name] = round(time.time() - t0, 3)
    out.update(cores=os.cpu_count() or 1, nodes=st["nodes"], leaf_refs=st["refs"])
    return out


def cpu_sample_ranges(W, H, rows=8, cols=12):
    """Block ranges of a rows x cols patch of blocks at the image centre (the bounded CPU sample)."""
    bw = (W + 7) // 8
    bh = (H + 15) // 16
    r0, c0 = bh // 2 - rows // 2, bw // 2 - cols // 2
    return [((r0 + r) * bw + c0, (r0 + r) * bw + c0 + cols) for r in range(rows)]


def cpu_baseline_ours(S, cam, W, H, depth, seed, spp=(8, 8)):
    """FP64 oracle (physical mode) on a bounded sample: an 8x12-block patch (12,288 pixels) at the
    image centre, 64 spp, same depth (about 10 s on 16 cores)."""
    sys.path.insert(0, str(ROOT / "tests"))
    import dumbray_gb300 as dr
    import _oracle as O
    threads = os.cpu_count() or 1
    osc = O.OracleScene(S["tris"], mat_id=S["mat_id"], materials=[dr.lambert(), dr.mirror(), dr.glossy()], threads=threads)
    osc.set_triangle_params(S["albedo"], S["emission"], S["roughness"])
    p = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=spp, max_bounces=depth, seed=seed)
    fb = np.zeros((dr.block_count(W, H) * 128, 4), np.float32)
    ranges = cpu_sample_ranges(W, H)
    t0 = time.time()
    for a, b in ranges:
        osc.render_blocks(cam, p, fb=fb, start=a, end=b, threads=threads)
    dt = time.time() - t0
    px = sum(b - a for a, b in ranges) * 128
    paths = px * spp[0] * spp[1]
    return dict(value=paths / dt / 1e6, unit=UNIT, cores=threads, kind="port",
                sample=f"FP64 oracle, centre patch of 8x12 blocks of {W}x{H} ({px:,} px) x {spp[0] * spp[1]} spp, "
                       f"depth {depth}, {dt:.1f} s"), (ranges, fb, p, osc)


def fp64_error(g, o):
    """Relative RMSE (RMSE over the compared pixels / the oracle's mean), relative difference of the
    means, and that difference in units of its Monte Carlo standard error (per-pixel differences)."""
    g = np.asarray(g, np.float64)[..., :3]
    o = np.asarray(o, np.float64)[..., :3]
    m = max(float(o.mean()), 1e-12)
    diff = (g - o).reshape(-1, 3).mean(1)
    se = max(float(diff.std(ddof=1) / np.sqrt(len(diff))), 1e-15)
    return {"rmse_rel": round(float(np.sqrt(np.mean((g - o) ** 2)) / m), 6),
            "mean_rel_diff": round(float((g.mean() - o.mean()) / m), 7),
            "mean_diff_in_se": round(float(diff.mean() / se), 3)}


def run_ours(a):
    import torch
    import dumbray_gb300 as dr

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    S, scene, build_s = build_scene(dr, a.level, a.split, a.ref_tree)
    cam = make_camera(dr, a.lens)
    W, H = a.width, a.height
    sx, sy = samples_xy(a.spp)
    nb = dr.block_count(W, H)
    paths_per_frame = W * H * a.spp
    fb = dr.new_frame_buffer(W, H, dev)
    rend = dr.Renderer(a.wave, a.lanes)
    stream = torch.cuda.current_stream()

    def params(it):
        # each rank renders distinct samples: iteration index offset by rank
        return dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(sx, sy), max_bounces=a.depth,
                                iteration=1 + rank * 100000 + it, seed=1234)

    first_ms = None
    for i in range(a.warmup):
        w0 = time.time()
        rend.render_blocks(scene, cam, fb, 0, nb, params(i), stream)
        if i == 0:
            torch.cuda.synchronize()
            first_ms = (time.time() - w0) * 1e3
    torch.cuda.synchronize()
    # timed region: device-resident inputs
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    rend.set_profiling(True)
    launches0 = rend.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(a.steps):
        rend.render_blocks(scene, cam, fb, 0, nb, params(a.warmup + i), stream)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = rend.launches() - launches0
    wave_rays, wave_shadows = rend.wave_counts(a.depth + 1)
    ktimes = rend.kernel_times()
    kbusy = rend.kernel_busy()
    rend.set_profiling(False)
    ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.barrier()
        ms = float(t.item())
    value = world * paths_per_frame * a.steps / (ms / 1e3) / 1e6

    # e2e through the public API with host buffers (pinned), copies inside the timed region
    if a.no_e2e:
        a.steps_e2e = 0
    host_fb = torch.zeros(fb.shape, dtype=torch.float32).pin_memory()
    host_out = torch.zeros(fb.shape, dtype=torch.float32).pin_memory()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for i in range(0 if a.no_e2e else a.steps):
        fb.copy_(host_fb, non_blocking=True)
        rend.render_blocks(scene, cam, fb, 0, nb, params(a.warmup + a.steps + i), stream)
        host_out.copy_(fb, non_blocking=True)
    f1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = f0.elapsed_time(f1)
    if world > 1:
        t = torch.tensor([ms_e2e], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_e2e = float(t.item())
    e2e = world * paths_per_frame * a.steps / (ms_e2e / 1e3) / 1e6 if not a.no_e2e else None
    fb_bytes = fb.numel() * 4

    # counting pass (untimed): reference traversal counts of the extension rays of one frame
    if a.no_count:
        cnt = dict(trace_rays=0, trace_box=0, trace_tri=0, shadow_casts=0, shadow_box=0, shadow_tri=0)
    else:
        rend.set_counting(True)
        rend.render_blocks(scene, cam, fb, 0, nb, params(0), stream)
        cnt = rend.counters()
        rend.set_counting(False)
    c_box = cnt["trace_box"] / max(1, cnt["trace_rays"])
    c_tri = cnt["trace_tri"] / max(1, cnt["trace_rays"])
    bytes_per_ray = 40.0 + 32.0 * c_box + 36.0 * c_tri
    # k_trace time = its busy time: the union of its launch intervals over the renderer's lanes
    # (launches of concurrent lanes overlap; with one lane this is the summed launch durations)
    trace_sum_ms, trace_launches = ktimes["trace"]
    trace_ms = kbusy["trace"]
    rays_per_launch = cnt["trace_rays"] * a.steps / max(1, trace_launches)
    frames = a.steps
    trace_bytes_per_frame = cnt["trace_rays"] * bytes_per_ray
    achieved = (trace_bytes_per_frame * frames) / (trace_ms / 1e3) / 1e9 if trace_ms > 0 else 0.0
    peak, peak_src = measured_peak()

    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": round(ms / a.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"full path trace: {len(S['tris']):,}-tri displaced icosphere L{a.level} + ground + 4 emissive "
                               f"quads, {W}x{H}, {a.spp} spp, depth {a.depth}, {a.lens}",
                   "triangles": int(len(S["tris"])), "width": W, "height": H, "spp": a.spp, "depth": a.depth,
                   "lens": a.lens, "mode": "physical", "wave_paths": a.wave, "lanes": rend.lanes,
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (scene ~0.3 GB, wavefront queues ~2 GB), no flush",
                   "scene_build_s": round(build_s, 2),
                   "octree_build_s": octree_build_times(dr, S),
                   "octree": {"split_threshold": S["split"], "box_epsilon": S["box_epsilon"] or 1.28e-3,
                              "rule": "reference split rule; " + ("reference padding" if a.ref_tree else
                                      "physical-mode padding 2^-18 x max |coordinate|")}},
        "e2e": {"value": None if e2e is None else round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": fb_bytes, "d2h_bytes_per_step": fb_bytes},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": round(TRACE_DRAM_BYTES_PER_RAY * rays_per_launch) if cnt["trace_rays"] else None,
                     "traffic_unit": "bytes per launch (ncu dram__bytes_read+write, scaled by rays per launch)",
                     "algorithmic_bytes_per_launch": round(bytes_per_ray * rays_per_launch), "kernel": "k_trace",
                     "peak_source": f"{peak_src} hbm_gbs", "bytes_per_ray": round(bytes_per_ray, 1),
                     "c_box": round(c_box, 2), "c_tri": round(c_tri, 2),
                     "launch_ms_avg": round(trace_ms / max(1, trace_launches), 4),
                     "launch_ms_avg_basis": "k_trace busy time (union of its launch intervals over all lanes) per launch",
                     "launch_ms_avg_own_duration": round(trace_sum_ms / max(1, trace_launches), 4)},
        "kernel_ms_per_step": {k: round(v / a.steps, 2) for k, v in kbusy.items()},
        "kernel_ms_per_step_basis": "busy time per kernel class (union of launch intervals over lanes)",
        "kernel_launch_ms_sum_per_step": {k: round(v[0] / a.steps, 2) for k, v in ktimes.items()},
        "first_frame_ms": None if first_ms is None else round(first_ms, 1),
        "rays_per_frame": {"extension": cnt["trace_rays"], "shadow": cnt["shadow_casts"]},
        "last_wave_rays_per_bounce": {"extension": wave_rays, "shadow": wave_shadows,
                                      "basis": "queue sizes of the last wave on the renderer's first lane"},
        "mrays_per_s": round((cnt["trace_rays"] + cnt["shadow_casts"]) * a.steps / (ms / 1e3) / 1e6, 1),
    }
    if clocks:
        out["clocks"] = clocks
    if rank == 0 and world == 1 and not a.no_variants:
        variants = {}
        for lens in ("fisheye", "spherical"):
            c2 = make_camera(dr, lens)
            rend.render_blocks(scene, c2, fb, 0, nb, params(0), stream)
            torch.cuda.synchronize()
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            rend.render_blocks(scene, c2, fb, 0, nb, params(1), stream)
            g1.record(stream)
            torch.cuda.synchronize()
            variants[lens] = round(paths_per_frame / (g0.elapsed_time(g1) / 1e3) / 1e6, 3)
        out["lens_variants_mpaths_s"] = variants
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        base, (ranges, ofb, p, osc) = cpu_baseline_ours(S, cam, W, H, a.depth, 4321)
        out["cpu_baseline"] = base
        # accuracy on the same sample: GPU at the same samples vs the FP64 oracle
        gfb = dr.new_frame_buffer(W, H, dev)
        for s0, s1 in ranges:
            rend.render_blocks(scene, cam, gfb, s0, s1, p, stream)
        torch.cuda.synchronize()
        gall = gfb.cpu().numpy()
        g = np.concatenate([gall[s0 * 128:s1 * 128, :3] for s0, s1 in ranges]).astype(np.float64)
        o = np.concatenate([ofb[s0 * 128:s1 * 128, :3] for s0, s1 in ranges]).astype(np.float64)
        # same counter-based random numbers on both sides: most paths coincide; float-vs-double shading
        # makes some deep paths diverge, which shows up as noise, so report the relative RMSE and the
        # patch-mean difference in units of its Monte Carlo standard error (64 spp per pixel)
        diff = (g - o).mean(1)
        out["accuracy_vs_fp64_oracle"] = {
            "rmse_rel": float(np.sqrt(np.mean((g - o) ** 2)) / max(o.mean(), 1e-9)),
            "mean_rel_diff": float((g.mean() - o.mean()) / max(o.mean(), 1e-9)),
            "mean_diff_in_se": float(diff.mean() / max(diff.std(ddof=1) / np.sqrt(len(diff)), 1e-12)),
            "sample": "centre patch 12,288 px x 64 spp, same seeds"}
        # converged: 12 blocks (1,536 px) at the centre, 16 progressive iterations of 64 spp (1,024 spp)
        # on both sides; per-pixel differences from diverging paths average out as 1/sqrt(spp)
        crng = cpu_sample_ranges(W, H, rows=1, cols=12)
        ofb2 = np.zeros((nb * 128, 4), np.float32)
        gfb2 = dr.new_frame_buffer(W, H, dev)
        threads = os.cpu_count() or 1
        for it in range(1, 17):
            pit = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(8, 8), max_bounces=a.depth, iteration=it, seed=4321)
            for s0, s1 in crng:
                osc.render_blocks(cam, pit, fb=ofb2, start=s0, end=s1, threads=threads)
                rend.render_blocks(scene, cam, gfb2, s0, s1, pit, stream)
        torch.cuda.synchronize()
        g2 = np.concatenate([gfb2.cpu().numpy()[s0 * 128:s1 * 128, :3] for s0, s1 in crng]).astype(np.float64)
        o2 = np.concatenate([ofb2[s0 * 128:s1 * 128, :3] for s0, s1 in crng]).astype(np.float64)
        out["accuracy_vs_fp64_oracle_converged"] = {
            "rmse_rel": float(np.sqrt(np.mean((g2 - o2) ** 2)) / max(o2.mean(), 1e-9)),
            "mean_rel_diff": float((g2.mean() - o2.mean()) / max(o2.mean(), 1e-9)),
            "sample": "centre row of 12 blocks (1,536 px), 16 iterations x 64 spp = 1,024 spp, same seeds"}
        # the fisheye and spherical lens variants of the same frame, on the same samples
        lens_acc = {}
        for lens in ("fisheye", "spherical"):
            c2 = make_camera(dr, lens)
            ofb3 = np.zeros((nb * 128, 4), np.float32)
            gfb3 = dr.new_frame_buffer(W, H, dev)
            for s0, s1 in ranges:
                osc.render_blocks(c2, p, fb=ofb3, start=s0, end=s1, threads=threads)
                rend.render_blocks(scene, c2, gfb3, s0, s1, p, stream)
            ofb4 = np.zeros((nb * 128, 4), np.float32)
            gfb4 = dr.new_frame_buffer(W, H, dev)
            for it in range(1, 17):
                pit = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(8, 8), max_bounces=a.depth, iteration=it, seed=4321)
                for s0, s1 in crng:
                    osc.render_blocks(c2, pit, fb=ofb4, start=s0, end=s1, threads=threads)
                    rend.render_blocks(scene, c2, gfb4, s0, s1, pit, stream)
            torch.cuda.synchronize()
            g3, g4 = gfb3.cpu().numpy(), gfb4.cpu().numpy()
            lens_acc[lens] = {
                "patch_64spp": fp64_error(np.concatenate([g3[s0 * 128:s1 * 128] for s0, s1 in ranges]),
                                          np.concatenate([ofb3[s0 * 128:s1 * 128] for s0, s1 in ranges])),
                "converged_1024spp": fp64_error(np.concatenate([g4[s0 * 128:s1 * 128] for s0, s1 in crng]),
                                                np.concatenate([ofb4[s0 * 128:s1 * 128] for s0, s1 in crng]))}
        lens_acc["sample"] = ("as for the pinhole: centre patch 12,288 px x 64 spp and centre row of 12 blocks x "
                              "1,024 spp, same seeds on both sides")
        out["lens_variants_accuracy_vs_fp64_oracle"] = lens_acc
    del rend
    if rank == 0 and world == 1 and not a.no_raycast:
        out["raycast"] = run_raycast(dr, torch, dev, a, peak, peak_src)
    if rank == 0 and world == 1 and not a.no_c1:
        out["c1_plain"] = run_c1(dr, torch, dev, a)
    if rank == 0 and world == 1 and not a.no_twin:
        out["reference_mode_twin"] = run_reference_twin_gpu(dr, torch, dev, a, S, peak, peak_src)
    if rank == 0 and world == 1 and not a.no_batched:
        out["batched"] = run_batched(dr, torch, dev, a)
    if rank == 0 and world == 1 and not a.no_adjoint:
        out["differentiable"] = run_differentiable(dr, torch, dev, a)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_c1(dr, torch, dev, a):
    """The CPU-runnable plain path trace (2x2x2 room with a red wall, icosphere level 5 of radius 0.6,
    0.5x0.5 emissive quad of radiance 10; pinhole 60 degrees; 256x256, 16 spp, depth 4, seed 0,
    reference leaf size 8): GPU Mpaths/s (physical mode), its error against the FP64 oracle on the
    whole image at the same samples, and the reference-expressible twin (the quad as a spherical
    light of the same power) rendered in reference mode on the GPU and by the reference
    DumbRenderer on host cores."""
    from dumbray_gb300 import scenes
    sys.path.insert(0, str(ROOT / "tests"))
    import _oracle as O
    c = scenes.box_and_icosphere(5)
    mats = [dr.lambert((0.7, 0.7, 0.7)), dr.lambert((0.7, 0.1, 0.1)), dr.lambert((0.0, 0.0, 0.0), emission=(10.0, 10.0, 10.0))]
    W = H = 256
    nb = dr.block_count(W, H)
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.99), angle=60.0)
    sc = dr.Scene(c["tris"], mat_id=c["mat_id"], materials=mats)
    rend = dr.Renderer(1 << 22)
    fb = dr.new_frame_buffer(W, H, dev)

    def params(it):
        return dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(4, 4), max_bounces=4, iteration=it, seed=0)

    for i in range(3):
        rend.render_blocks(sc, cam, fb, 0, nb, params(2 + i))
    K = 20
    ms = _events_ms(torch, lambda i: rend.render_blocks(sc, cam, fb, 0, nb, params(2 + i)), K) / K
    # the same frames as a one-job batch: the whole launch sequence replayed from one CUDA graph
    # (dr_batch_render), the iteration rewritten in the job table between replays
    batch = dr.Batch([(sc, cam, params(2), fb, 0, nb)])
    batch.render(rend, use_graph=True)

    def graph_step(i):
        batch.set_iteration(3 + i)
        batch.render(rend, use_graph=True)

    graph_ms = _events_ms(torch, graph_step, K) / K
    batch.close()
    rend.render_blocks(sc, cam, fb, 0, nb, params(1))
    torch.cuda.synchronize()
    g = fb.cpu().numpy()
    threads = os.cpu_count() or 1
    osc = O.OracleScene(c["tris"], mat_id=c["mat_id"], materials=mats, threads=threads)
    t0 = time.time()
    o = osc.render_blocks(cam, params(1), threads=threads)
    osec = time.time() - t0
    paths = W * H * 16
    out = {"workload": f"room + icosphere L5 + emissive quad ({len(c['tris']):,} tris), 256x256, 16 spp, depth 4, pinhole, "
                       "physical mode",
           "mpaths_s": round(paths / (ms / 1e3) / 1e6, 2), "ms_per_frame": round(ms, 3),
           "one_job_graph_mpaths_s": round(paths / (graph_ms / 1e3) / 1e6, 2),
           "one_job_graph_ms_per_frame": round(graph_ms, 3),
           "accuracy_vs_fp64_oracle": dict(fp64_error(g, o), sample="whole image, 16 spp, same seeds"),
           "fp64_oracle_mpaths_s": round(paths / osec / 1e6, 4), "fp64_oracle_cores": threads}
    rend.close()
    sc.close()
    # reference-expressible twin: reference mode on the GPU vs the reference DumbRenderer on host cores
    gold = ROOT / "tests" / "golden"
    sys.path.insert(0, str(gold))
    from make_golden import c1_twin
    tris, mat, tmats, lights, tcam = c1_twin()
    tsc = dr.Scene(tris, mat_id=mat, materials=tmats, lights=lights)
    trend = dr.Renderer(1 << 22)
    tfb = dr.new_frame_buffer(W, H, dev)

    def tparams(it):
        return dr.render_params(W, H, dr.MODE_REFERENCE, samples=(4, 4), max_bounces=4, iteration=it, seed=0)

    for i in range(3):
        trend.render_blocks(tsc, tcam, tfb, 0, nb, tparams(1 + i))
    tms = _events_ms(torch, lambda i: trend.render_blocks(tsc, tcam, tfb, 0, nb, tparams(4 + i)), K) / K
    trend.close()
    tsc.close()
    twin = {"workload": "reference-expressible twin (the quad as a spherical light of equal power at y = 0.8), "
                        "reference mode, 256x256, 16 spp, depth 4",
            "gpu_mpaths_s": round(paths / (tms / 1e3) / 1e6, 2),
            "parity": "tests/test_configs_gpu.py: per pixel vs the oracle, statistically vs the reference DumbRenderer"}
    ref = time_reference_renderer(tris, mat, tmats, lights, tcam, 4, steps=3, warmup=1, sw=W, sh=H)
    if ref is not None:
        sec, rbuild, rthreads, rpaths = ref
        twin["reference_cpu_mpaths_s"] = round(rpaths / sec / 1e6, 4)
        twin["reference_cpu_cores"] = rthreads
        twin["vs_reference_cpu"] = round(twin["gpu_mpaths_s"] / twin["reference_cpu_mpaths_s"], 1)
    out["reference_mode_twin"] = twin
    return out


def _batch_scene(dr, job, split=0):
    sc = dr.Scene(job["tris"], mat_id=job["mat_id"], materials=[dr.lambert(), dr.mirror(), dr.glossy()],
                  split_threshold=split, box_epsilon=dr.PHYSICAL_TREE, device_build=True)
    sc.set_triangle_params(job["albedo"], job["emission"], job["roughness"])
    return sc


def _events_ms(torch, fn, steps):
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(steps):
        fn(i)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def time_reference_renderer(tris, mat, mats, lights, cam, depth, steps, warmup, sw=240, sh=136):
    """The reference DumbRenderer (compiled from the reference sources into oracle/_ref) on all host
    threads: mean seconds per sw x sh x 1 spp render after `warmup` untimed ones, plus the octree
    build time and the thread count.  None when the reference library is absent."""
    sys.path.insert(0, str(ROOT / "tests"))
    import _oracle as O
    if not O.reference_available():
        return None
    L = O.reference()
    threads = os.cpu_count() or 1
    t_ = np.ascontiguousarray(tris, np.float32)
    m_ = np.ascontiguousarray(mat, np.int32)
    mrec = np.ascontiguousarray(np.stack([O.ref_material_record(m) for m in mats]))
    lrec = np.ascontiguousarray(np.stack([O.ref_light_record(l) for l in lights]))
    crec = O.ref_camera_record(cam)
    t0 = time.time()
    h = L.dref_scene_create(t_.ctypes.data, None, m_.ctypes.data, len(t_), mrec.ctypes.data, len(mrec),
                            lrec.ctypes.data, len(lrec), crec.ctypes.data)
    build_s = time.time() - t0
    img = np.zeros((sh, sw, 4), np.float32)
    try:
        for _ in range(warmup):
            L.dref_render(h, sw, sh, 1, 1, depth, 1, 1, threads, img.ctypes.data)
        secs = [L.dref_render(h, sw, sh, 1, 1, depth, 1, 1, threads, img.ctypes.data) for _ in range(steps)]
    finally:
        L.dref_scene_destroy(h)
    return float(np.mean(secs)), build_s, threads, sw * sh


def run_reference_twin_gpu(dr, torch, dev, a, S, peak, peak_src):
    """The drop-in path at the headline size: the reference-expressible twin of the path-trace scene
    (DumbBased / SimpleStochastic materials, 4 spherical lights, SimpleStochasticLense 60 degrees from
    (0, 0.6, -3.4)) rendered in reference mode (DumbRenderer's estimator) on the reference's octree,
    1920x1080, 64 spp (8x8 sub-pixels), depth a.depth, i.e. the workload the reference arm times on
    host cores.  value: CUDA events over the timed frames, scene resident; e2e: the same through the
    public API with the frame buffer copied host->device and device->host every frame (pinned);
    roofline: the photon casts (k_shadow_ref first casts + k_photon_chain transparency chains, the
    dominant kernel class), algorithmic bytes = casts x (40 + 32 C_box + 36 C_tri) from the counting pass, over
    their busy time; last_wave_counts: extension rays and photon records per bounce of the counting
    pass's last wave (the whole frame when it is one wave), so casts / records is the photons' mean
    cast count; cpu_baseline: the reference DumbRenderer itself on a 240x136 x 1 spp sample."""
    tris, mat, mats, lights = reference_twin(S, dr)
    t0 = time.time()
    sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights, device_build=True,
                  box_epsilon=dr.PHYSICAL_TREE if a.twin_tree == "physical" else 0.0)
    build_s = time.time() - t0
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.6, -3.4), angle=60.0)
    W, H = (int(v) for v in a.twin_size.split("x"))
    sx, sy = samples_xy(a.twin_spp)
    spp = sx * sy
    nb = dr.block_count(W, H)
    fb = dr.new_frame_buffer(W, H, dev)
    rend = dr.Renderer(a.wave, a.lanes)
    stream = torch.cuda.current_stream()

    def params(i):
        return dr.render_params(W, H, dr.MODE_REFERENCE, samples=(sx, sy), max_bounces=a.depth, iteration=1 + i, seed=77)

    rend.render_blocks(sc, cam, fb, 0, nb, params(0), stream)
    K = max(2, min(3, a.steps))
    torch.cuda.synchronize()
    rend.set_profiling(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(K):
        rend.render_blocks(sc, cam, fb, 0, nb, params(1 + i), stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / K
    kt = rend.kernel_times()
    kbusy = rend.kernel_busy()
    rend.set_profiling(False)
    host_fb = torch.zeros(fb.shape, dtype=torch.float32).pin_memory()
    host_out = torch.zeros(fb.shape, dtype=torch.float32).pin_memory()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for i in range(K):
        fb.copy_(host_fb, non_blocking=True)
        rend.render_blocks(sc, cam, fb, 0, nb, params(1 + K + i), stream)
        host_out.copy_(fb, non_blocking=True)
    f1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = f0.elapsed_time(f1) / K
    rend.set_counting(True)
    rend.render_blocks(sc, cam, fb, 0, nb, params(0), stream)
    cnt = rend.counters()
    wave_rays, wave_photons = rend.wave_counts(a.depth + 1)
    rend.set_counting(False)
    rend.close()
    sc.close()
    paths = W * H * spp
    value = paths / (ms / 1e3) / 1e6
    e2e = paths / (ms_e2e / 1e3) / 1e6
    casts = cnt["shadow_casts"]
    c_box = cnt["shadow_box"] / max(1, casts)
    c_tri = cnt["shadow_tri"] / max(1, casts)
    bpr = 40.0 + 32.0 * c_box + 36.0 * c_tri
    shadow_ms = kbusy["shadow"] / K
    achieved = casts * bpr / (shadow_ms / 1e3) / 1e9 if shadow_ms > 0 else 0.0
    out = {"workload": f"reference-expressible twin ({len(tris):,} tris, {len(lights)} spherical lights), reference mode "
                       f"(DumbRenderer's estimator), {W}x{H} x {spp} spp, depth {a.depth}, {a.twin_tree} octree",
           "mpaths_s": round(value, 3), "ms_per_frame": round(ms, 2), "frames": K,
           "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": int(fb.numel() * 4),
                   "d2h_bytes_per_step": int(fb.numel() * 4)},
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "peak_source": f"{peak_src} hbm_gbs",
                        "kernel": "k_shadow_ref + k_photon_chain (photon casts, chains included)", "casts_per_frame": int(casts),
                        "c_box": round(c_box, 2), "c_tri": round(c_tri, 2), "bytes_per_cast": round(bpr, 1),
                        "busy_ms_per_frame": round(shadow_ms, 2),
                        "basis": "photon-cast busy time (union of launch intervals over lanes) per frame"},
           "extension_rays_per_frame": int(cnt["trace_rays"]),
           "last_wave_counts": {"extension": wave_rays, "photon_records": wave_photons,
                                "single_wave": paths <= a.wave},
           "kernel_busy_ms_per_frame": {k: round(v / K, 2) for k, v in kbusy.items()},
           "kernel_launch_ms_sum_per_frame": {k: round(v[0] / K, 2) for k, v in kt.items()},
           "scene_build_s": round(build_s, 2)}
    ref = None if a.twin_only else time_reference_renderer(tris, mat, mats, lights, cam, a.depth, steps=3, warmup=1)
    if ref is not None:
        sec, rbuild, threads, rpaths = ref
        rv = rpaths / sec / 1e6
        out["cpu_baseline"] = {"value": round(rv, 5), "unit": UNIT, "cores": threads, "kind": "reference",
                               "sample": f"reference DumbRenderer (CPU threads) compiled from the reference sources; "
                                         f"240x136 px x 1 spp per step ({rpaths:,} paths), 3 steps, octree build "
                                         f"{rbuild:.1f} s excluded"}
        out["vs_reference_cpu"] = {"device": round(value / rv, 1), "e2e": round(e2e / rv, 1)}
    return out


def run_raycast(dr, torch, dev, a, peak, peak_src):
    """Closest-hit ray casting through dr_cast on the displaced icosphere alone (level 8, 1,310,720
    triangles, amplitude 0.1, seed 1): 1920x1080 coherent pinhole primary rays (60 degrees, from
    (0, 0.3, -3) toward the origin) and 8M incoherent rays (origins uniform in [-1.1, 1.1]^3,
    directions uniform on the sphere, seed 0), each timed over K casts of the whole set with CUDA
    events, on the reference's octree and on the physical-mode one.  Roofline: algorithmic bytes =
    rays x (40 + 32 C_box + 36 C_tri) with the mean box and triangle tests per ray counted by
    dr_cast_counted, divided by the kernel time."""
    from dumbray_gb300 import scenes

    mesh = scenes.displaced_icosphere(a.level, 0.1, 1)
    out = {"workload": f"displaced icosphere L{a.level} alone ({len(mesh):,} tris), closest hit, backface culling "
                       "(the renderer default; *_no_cull: the same rays without); "
                       "reference_tree = the reference's octree (casts bit-exact to Octree::cast), physical_tree = "
                       "padding 2^-18 x max |coordinate| (same closest hits up to float32 near-ties)",
           "counts": "c_box / c_tri from dr_cast_counted: on the reference tree the reference's own traversal (it "
                     "also tests boxes lying behind the ray origin, which dr_cast skips without changing any hit), "
                     "so the reference-tree roofline is an effective figure; on the physical tree the traversal "
                     "dr_cast runs"}
    sets = {"primary_1080p": scenes.primary_rays(1920, 1080, 60.0, (0.0, 0.3, -3.0), (0.0, 0.0, 0.0)),
            "incoherent_8M": scenes.incoherent_rays(8 * 1024 * 1024, -1.1, 1.1, seed=0)}
    K = max(3, a.steps)
    hits = {}
    for tree, eps in (("reference_tree", 0.0), ("physical_tree", dr.PHYSICAL_TREE)):
        sc = dr.Scene(mesh, materials=[dr.lambert()], box_epsilon=eps)
        st = sc.stats()
        res = {"octree": {"nodes": st["nodes"], "leaf_refs": st["refs"], "refs_per_tri": round(st["refs"] / len(mesh), 2)}}
        hits[tree] = {}
        for name, (o, d) in sets.items():
            ot = torch.from_numpy(o).to(dev)
            dt = torch.from_numpy(d).to(dev)
            n = len(o)
            for _ in range(3):
                dr.cast(sc, ot, dt)
            ms = _events_ms(torch, lambda i: dr.cast(sc, ot, dt), K) / K
            tri, t, nb, nt = dr.cast(sc, ot, dt, counted=True)
            c_box = float(nb.double().mean())
            c_tri = float(nt.double().mean())
            bpr = 40.0 + 32.0 * c_box + 36.0 * c_tri
            achieved = n * bpr / (ms / 1e3) / 1e9
            res[name] = {"rays": n, "ms": round(ms, 3), "mrays_s": round(n / (ms / 1e3) / 1e6, 1),
                         "hit_fraction": round(float((tri >= 0).float().mean()), 4), "c_box": round(c_box, 2),
                         "c_tri": round(c_tri, 2), "bytes_per_ray": round(bpr, 1),
                         "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                                      "frac": round(achieved / peak, 4), "peak_source": f"{peak_src} hbm_gbs",
                                      "kernel": "k_cast"}}
            hits[tree][name] = tri.cpu().numpy()
            # the same rays with backface culling off (dr_cast clip_backfaces = 0)
            for _ in range(2):
                dr.cast(sc, ot, dt, cull_backfaces=False)
            ms0 = _events_ms(torch, lambda i: dr.cast(sc, ot, dt, cull_backfaces=False), K) / K
            tri0, _, nb0, nt0 = dr.cast(sc, ot, dt, cull_backfaces=False, counted=True)
            c_box0, c_tri0 = float(nb0.double().mean()), float(nt0.double().mean())
            bpr0 = 40.0 + 32.0 * c_box0 + 36.0 * c_tri0
            achieved0 = n * bpr0 / (ms0 / 1e3) / 1e9
            res[name + "_no_cull"] = {"rays": n, "ms": round(ms0, 3), "mrays_s": round(n / (ms0 / 1e3) / 1e6, 1),
                                      "hit_fraction": round(float((tri0 >= 0).float().mean()), 4),
                                      "c_box": round(c_box0, 2), "c_tri": round(c_tri0, 2), "bytes_per_ray": round(bpr0, 1),
                                      "roofline": {"bound": "hbm", "achieved": round(achieved0, 1), "peak": peak,
                                                   "unit": "GB/s", "frac": round(achieved0 / peak, 4),
                                                   "peak_source": f"{peak_src} hbm_gbs", "kernel": "k_cast"}}
            del ot, dt, tri0, nb0, nt0
        out[tree] = res
        sc.close()
    # parity on a subset: 65,536 incoherent rays and every 32nd primary, reference tree, culling on,
    # against the oracle (the reference's Octree::cast restated; pinned to the reference's own casts)
    sys.path.insert(0, str(ROOT / "tests"))
    import _oracle as O
    osc = O.OracleScene(mesh, threads=os.cpu_count() or 1)
    so = np.concatenate([sets["incoherent_8M"][0][:65536], sets["primary_1080p"][0][::32]])
    sd = np.concatenate([sets["incoherent_8M"][1][:65536], sets["primary_1080p"][1][::32]])
    sc = dr.Scene(mesh, materials=[dr.lambert()])
    gi, gt = dr.cast(sc, torch.from_numpy(so).to(dev), torch.from_numpy(sd).to(dev))
    gi, gt = gi.cpu().numpy(), gt.cpu().numpy()
    oi, ot, _, _ = osc.cast(so, sd, cull=True, threads=os.cpu_count() or 1)
    hit = oi >= 0
    out["parity_vs_oracle"] = {"rays": int(len(so)), "index_mismatches": int((gi != oi).sum()),
                               "t_bit_mismatches": int((gt[hit].view(np.int32) != ot[hit].view(np.int32)).sum()),
                               "tree": "reference", "cull": True}
    sc.close()
    del osc
    out["physical_vs_reference_tree_hit_mismatch"] = {
        k: float(np.mean(hits["reference_tree"][k] != hits["physical_tree"][k])) for k in sets}
    return out


def run_batched(dr, torch, dev, a):
    """64 independent scenes rendered scene by scene (plain dr_render_blocks launches, library default
    leaf split 8) and as one batch (shared waves, one CUDA graph, autotuned leaf split and wave
    size); both with the physical-mode octree padding.  Both arms render progressive iterations 1..K+1 of every job into the same frame buffers;
    Mpaths/s = all paths of the K timed iterations / CUDA-event time."""
    from dumbray_gb300 import autotune, scenes

    t0 = time.time()
    jobs = scenes.batch_workload(a.batch_scenes)
    gen_s = time.time() - t0
    n_tris = [len(j["tris"]) for j in jobs]
    cams = [dr.camera(dr.LENS_PINHOLE, position=j["cam_pos"], target=j["cam_target"], angle=60.0) for j in jobs]
    nbs = [dr.block_count(j["width"], j["height"]) for j in jobs]
    fbs = [dr.new_frame_buffer(j["width"], j["height"], dev) for j in jobs]
    paths = sum(j["width"] * j["height"] * j["spp"] for j in jobs)

    def params(j, it):
        return dr.render_params(j["width"], j["height"], dr.MODE_PHYSICAL, samples=samples_xy(j["spp"]),
                                max_bounces=j["depth"], iteration=it, seed=j["seed"])

    t0 = time.time()
    plain = [_batch_scene(dr, j) for j in jobs]
    build_s = time.time() - t0
    K = a.batch_steps

    # scene-by-scene plain launches
    rend = dr.Renderer(a.wave, a.lanes)

    def plain_step(i):
        for j, sc, cam, fb, nb in zip(jobs, plain, cams, fbs, nbs):
            rend.render_blocks(sc, cam, fb, 0, nb, params(j, 2 + i))

    for j, sc, cam, fb, nb in zip(jobs, plain, cams, fbs, nbs):
        rend.render_blocks(sc, cam, fb, 0, nb, params(j, 1))
    plain_ms = _events_ms(torch, plain_step, K)
    plain_launches = rend.launches()
    plain_means = np.array([fb[:, :3].double().mean().item() for fb in fbs])
    rend.close()

    # autotuning: leaf split threshold per size class, then wave size on a quarter of the jobs
    t0 = time.time()
    reps = autotune.representatives(jobs, n_tris)
    best_split, split_table = autotune.tune_leaf_threshold(lambda i, c: _batch_scene(dr, jobs[i], c), reps,
                                                           lambda i: cams[i], depth=jobs[0]["depth"], device=dev)
    tuned = []
    for i, j in enumerate(jobs):
        c = best_split[autotune.size_class(n_tris[i])]
        if c == 8:
            tuned.append(plain[i])
        else:
            tuned.append(_batch_scene(dr, j, c))
            plain[i].close()
    plain = None
    items = [(tuned[i], cams[i], params(j, 1), fbs[i], 0, nbs[i]) for i, j in enumerate(jobs)]
    sub = dr.Batch(items[::4])
    best_wave, wave_table, brend = autotune.tune_wave(sub, lanes=a.lanes)
    best_shape, shape_table = autotune.tune_block_shape(sub, brend)
    sub.close()
    tune_s = time.time() - t0

    batch = dr.Batch(items)
    batch.render(brend, use_graph=True)            # capture + warm-up (iteration 1)
    l0 = brend.launches()

    def batch_step(i):
        batch.set_iteration(2 + i)
        batch.render(brend, use_graph=True)

    batch_ms = _events_ms(torch, batch_step, K)
    batch_launches = brend.launches() - l0
    classes = batch_classes(dr, torch, jobs, tuned, cams, fbs, nbs, params, brend, K)
    batch_means = np.array([fb[:, :3].double().mean().item() for fb in fbs])
    rel = np.abs(batch_means - plain_means) / np.maximum(np.abs(plain_means), 1e-9)
    # FP64 oracle error of a sample of jobs: the 4 cheapest for the oracle (paths x depth plus tree
    # build), one per resolution, rendered by the batch at iteration 1 and by the oracle alike
    sys.path.insert(0, str(ROOT / "tests"))
    import _oracle as O
    threads = os.cpu_count() or 1
    batch.set_iteration(1)
    batch.render(brend, use_graph=True)
    torch.cuda.synchronize()
    cost = [j["width"] * j["height"] * j["spp"] + 4 * n for j, n in zip(jobs, n_tris)]
    picked, seen = [], set()
    for i in np.argsort(cost):
        if jobs[i]["width"] not in seen:
            picked.append(int(i))
            seen.add(jobs[i]["width"])
        if len(picked) == 4:
            break
    acc = {}
    for i in picked:
        j = jobs[i]
        osc = O.OracleScene(j["tris"], mat_id=j["mat_id"], materials=[dr.lambert(), dr.mirror(), dr.glossy()], threads=threads)
        osc.set_triangle_params(j["albedo"], j["emission"], j["roughness"])
        ofb = osc.render_blocks(cams[i], params(j, 1), threads=threads)
        acc[f"job{i}"] = dict(fp64_error(fbs[i].cpu().numpy(), ofb), triangles=int(n_tris[i]),
                              resolution=int(j["width"]), spp=int(j["spp"]))
        del osc
    v_plain = paths * K / (plain_ms / 1e3) / 1e6
    v_batch = paths * K / (batch_ms / 1e3) / 1e6
    res = sorted({(j["width"], j["spp"]) for j in jobs})
    out = {
        "workload": f"{len(jobs)} scenes, {sum(n_tris):,} triangles (per scene {min(n_tris):,}-{max(n_tris):,}, "
                    "displaced icosphere + random boxes + ground + emissive quad), square resolutions "
                    "128-1024, spp 4/16/64, depth 6, seeds 0-63, pinhole",
        "paths_per_step": int(paths), "steps": K,
        "scene_by_scene_mpaths_s": round(v_plain, 3), "batched_mpaths_s": round(v_batch, 3),
        "speedup": round(v_batch / v_plain, 3),
        "scene_by_scene_ms_per_step": round(plain_ms / K, 1), "batched_ms_per_step": round(batch_ms / K, 1),
        "batched_gpu_launches_per_step": int(batch_launches // max(1, K)), "graph": True,
        "autotune": {"leaf_split_by_class": {str(autotune.SIZE_CLASSES[k]) if k < len(autotune.SIZE_CLASSES)
                                             else "inf": v for k, v in sorted(best_split.items())},
                     "leaf_probe_ms": {str(k): v for k, v in split_table.items()},
                     "wave": best_wave, "wave_probe_ms": {str(k): v for k, v in wave_table.items()},
                     "block_shape": ["256x3", "128x6"][best_shape],
                     "block_shape_probe_ms": {["256x3", "128x6"][k]: v for k, v in shape_table.items()}},
        "job_mean_max_rel_diff_batched_vs_plain": float(rel.max()),
        "by_size_class": classes,
        "accuracy_vs_fp64_oracle": dict(acc, sample="4 jobs (the cheapest for the oracle of each resolution), "
                                                    "whole image, iteration 1 at the job's spp, same seeds"),
        "host_s": {"generate": round(gen_s, 1), "build": round(build_s, 1), "autotune": round(tune_s, 1)},
        "resolution_spp_mix": [list(r) for r in res],
    }
    batch.close()
    brend.close()
    for sc in tuned:
        sc.close()
    return out


BATCH_CLASSES = ((0, 1 << 20, "<=1M paths"), (1 << 20, 1 << 24, "1M-16M paths"), (1 << 24, 1 << 62, ">16M paths"))


def batch_classes(dr, torch, jobs, scenes, cams, fbs, nbs, params, rend, K):
    """Where the batch's time goes, by job size (paths per frame): for each class the jobs' share of
    the paths, their scene-by-scene time (plain dr_render_blocks launches, the same renderer and
    scenes as the batch) and the same jobs as a batch of their own, K timed iterations each; and the
    bound this puts on the whole batch's speed-up (only the time a class loses to plain launches can
    be recovered)."""
    out = {}
    t_plain_total = 0.0
    t_batch_total = 0.0
    for lo, hi, name in BATCH_CLASSES:
        idx = [i for i, j in enumerate(jobs) if lo < j["width"] * j["height"] * j["spp"] <= hi]
        if not idx:
            continue
        paths = sum(jobs[i]["width"] * jobs[i]["height"] * jobs[i]["spp"] for i in idx)

        def plain_step(k):
            for i in idx:
                rend.render_blocks(scenes[i], cams[i], fbs[i], 0, nbs[i], params(jobs[i], 2 + k))

        plain_step(0)
        t_plain = _events_ms(torch, plain_step, K) / K
        sub = dr.Batch([(scenes[i], cams[i], params(jobs[i], 1), fbs[i], 0, nbs[i]) for i in idx])
        sub.render(rend, use_graph=True)

        def sub_step(k):
            sub.set_iteration(2 + k)
            sub.render(rend, use_graph=True)

        t_batch = _events_ms(torch, sub_step, K) / K
        sub.close()
        t_plain_total += t_plain
        t_batch_total += t_batch
        out[name] = {"jobs": len(idx), "paths": int(paths), "plain_ms": round(t_plain, 2), "batched_ms": round(t_batch, 2),
                     "plain_mpaths_s": round(paths / (t_plain / 1e3) / 1e6, 2),
                     "batched_mpaths_s": round(paths / (t_batch / 1e3) / 1e6, 2),
                     "speedup": round(t_plain / t_batch, 3)}
    for v in out.values():
        v["share_of_plain_time"] = round(v["plain_ms"] / max(t_plain_total, 1e-9), 4)
    # upper bound of the whole batch's speed-up if every class ran at the fastest per-path rate any
    # class reaches, batched or not
    total_paths = sum(v["paths"] for v in out.values())
    best_rate = max(max(v["plain_mpaths_s"], v["batched_mpaths_s"]) for v in out.values())
    out["bound"] = {"plain_ms_sum": round(t_plain_total, 2), "class_batches_ms_sum": round(t_batch_total, 2),
                    "speedup_if_every_class_ran_at_best_rate": round(t_plain_total / (total_paths / best_rate / 1e3), 3)}
    return out


def run_differentiable(dr, torch, dev, a):
    """Forward render and path-replay adjoint of an L2 image loss w.r.t. per-triangle albedo and
    emission: icosphere level 7 + box room (327,692 triangles), 512x512, 16 spp, depth 5; target
    rendered from hidden albedo (seed 7).  Times forward and forward+adjoint steps and checks the
    largest gradient components against central finite differences with common random numbers."""
    from dumbray_gb300 import scenes

    S = scenes.differentiable_scene(7)
    n = len(S["tris"])
    sc = dr.Scene(S["tris"], mat_id=S["mat_id"], materials=[dr.lambert()], box_epsilon=dr.PHYSICAL_TREE)
    sc.set_triangle_params(S["albedo_target"], S["emission"], S["roughness"])
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.99), angle=60.0)
    W = H = 512
    p = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(4, 4), max_bounces=5, seed=7)
    nb = dr.block_count(W, H)
    rend = dr.Renderer(1 << 22)
    target = dr.new_frame_buffer(W, H, dev)
    rend.render_blocks(sc, cam, target, 0, nb, p)
    a_ptr, e_ptr = sc.triangle_params_device()
    alb = dr.device_view(a_ptr, (n, 3), dev)
    emi = dr.device_view(e_ptr, (n, 3), dev)
    alb.copy_(torch.from_numpy(S["albedo"]).to(dev))
    img = dr.new_frame_buffer(W, H, dev)
    dl = torch.zeros_like(img)
    ga = torch.zeros((n, 3), dtype=torch.float32, device=dev)
    ge = torch.zeros((n, 3), dtype=torch.float32, device=dev)

    def fwd(i):
        rend.render_blocks(sc, cam, img, 0, nb, p)

    def fwd_adj(i):
        rend.render_blocks(sc, cam, img, 0, nb, p)
        torch.sub(img[:, :3], target[:, :3], out=dl[:, :3]).mul_(2.0)
        ga.zero_()
        ge.zero_()
        rend.render_adjoint(sc, cam, dl, 0, nb, p, ga, ge)

    K = max(3, a.steps)
    for i in range(3):
        fwd_adj(i)
    fwd_ms = _events_ms(torch, fwd, K) / K
    fa_ms = _events_ms(torch, fwd_adj, K) / K
    paths = W * H * 16

    def loss():
        rend.render_blocks(sc, cam, img, 0, nb, p)
        d = img[:, :3].double() - target[:, :3].double()
        return float((d * d).sum())

    ga_h, ge_h = ga.cpu().numpy(), ge.cpu().numpy()
    errs = []
    for f in np.argsort(-np.abs(ga_h).ravel())[:8]:
        k, ch = divmod(int(f), 3)
        x = float(S["albedo"][k, ch])
        alb[k, ch] = x + 1e-3
        lp = loss()
        alb[k, ch] = x - 1e-3
        lm = loss()
        alb[k, ch] = x
        fd = (lp - lm) / 2e-3
        errs.append(("albedo", k, ch, float(ga_h[k, ch]), fd, abs(ga_h[k, ch] - fd) / max(abs(fd), 1e-12)))
    em_ids = S["emissive_ids"]
    for k in em_ids[np.argsort(-np.abs(ge_h[em_ids]).sum(1))[:4]]:
        ch = int(np.argmax(np.abs(ge_h[k])))
        x = float(S["emission"][k, ch])
        emi[k, ch] = x + 1e-2
        lp = loss()
        emi[k, ch] = x - 1e-2
        lm = loss()
        emi[k, ch] = x
        fd = (lp - lm) / 2e-2
        errs.append(("emission", int(k), ch, float(ge_h[k, ch]), fd, abs(ge_h[k, ch] - fd) / max(abs(fd), 1e-12)))
    # forward image against the FP64 oracle: 4 rows x 16 blocks at the image centre (8,192 px), 16 spp
    sys.path.insert(0, str(ROOT / "tests"))
    import _oracle as O
    threads = os.cpu_count() or 1
    osc = O.OracleScene(S["tris"], mat_id=S["mat_id"], materials=[dr.lambert()], threads=threads)
    osc.set_triangle_params(S["albedo"], S["emission"], S["roughness"])
    bw = nb // 32
    ranges = [((14 + r) * bw + 16, (14 + r) * bw + 32) for r in range(4)]
    ofb = np.zeros((nb * 128, 4), np.float32)
    for s0, s1 in ranges:
        osc.render_blocks(cam, p, fb=ofb, start=s0, end=s1, threads=threads)
    rend.render_blocks(sc, cam, img, 0, nb, p)
    torch.cuda.synchronize()
    gimg = img.cpu().numpy()
    fwd_acc = dict(fp64_error(np.concatenate([gimg[s0 * 128:s1 * 128] for s0, s1 in ranges]),
                              np.concatenate([ofb[s0 * 128:s1 * 128] for s0, s1 in ranges])),
                   sample="4 rows x 16 blocks at the centre (8,192 px), 16 spp, same seeds")
    del osc
    rend.close()
    sc.close()
    worst = max(errs, key=lambda e: e[5])
    return {
        "workload": f"icosphere L7 + box room ({n:,} tris), per-triangle albedo U[0.1,0.9], emission 10 on 64 tris, "
                    "512x512, 16 spp, depth 5, L2 loss vs target from hidden albedo (seed 7)",
        "fwd_ms": round(fwd_ms, 3), "fwd_adj_ms": round(fa_ms, 3), "ratio": round(fa_ms / fwd_ms, 3),
        "fwd_mpaths_s": round(paths / (fwd_ms / 1e3) / 1e6, 3),
        "fwd_adj_mpaths_s": round(paths / (fa_ms / 1e3) / 1e6, 3),
        "forward_accuracy_vs_fp64_oracle": fwd_acc,
        "fd_check": {"method": "central differences, common random numbers, parameters written in place; "
                               "h = 1e-3 (albedo), 1e-2 (emission 10)",
                     "components": len(errs), "max_rel_err": float(max(e[5] for e in errs)),
                     "worst": {"param": worst[0], "tri": worst[1], "channel": worst[2], "adjoint": worst[3],
                               "fd": worst[4]}},
    }


def reference_twin(S, dr):
    """Reference-expressible twin of the workload: emissive quads -> SphericalLightEmitter at the
    quad centres (colour = radiance x area x pi so the power matches), Lambert -> DumbBasedShader
    (metal 0), mirror -> SimpleStochasticShader(diffuse 0, smoothness 1), glossy -> DumbBasedShader
    (metal 1, Phong exponent 2/r^2 - 2), lens -> SimpleStochasticLense(60)."""
    tris = S["tris"]
    n_geo = S["n_mesh"] + S["n_ground"]
    mat = S["mat_id"][:n_geo].copy()
    mats = [dr.dumb_based(diffuse=(0.5, 0.5, 0.5), metal=0.0), dr.simple_stochastic((0.9, 0.9, 0.9), 0.0, 1.0, 64.0),
            dr.dumb_based(fresnel=(0.6, 0.6, 0.6), specular=2.0 / 0.2 ** 2 - 2.0, diffuse=(1, 1, 1), metal=1.0)]
    lights = []
    lt = tris[n_geo:].reshape(-1, 2, 3, 3)
    for q in lt:
        c = q.reshape(-1, 3).mean(0)
        lights.append(dr.spherical_light((10.0 * np.pi,) * 3, tuple(c - np.array([0, 0.05, 0])), 0.3))
    return tris[:n_geo], mat, mats, lights


def run_reference(a):
    world, rank, local = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "tests"))
    import dumbray_gb300 as dr
    import _oracle as O
    from dumbray_gb300 import scenes
    S = scenes.full_scene(level=a.level, seed=1)
    tris, mat, mats, lights = reference_twin(S, dr)
    threads = os.cpu_count() or 1
    cam_pos = (0.0, 0.6, -3.4)
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=cam_pos, angle=60.0)
    # bounded sample of the 1080p frame: a 240x136 image (1/64 of the pixels) at 1 spp per step
    sw, sh = 240, 136
    paths = sw * sh
    ref = time_reference_renderer(tris, mat, mats, lights, cam, a.depth, a.steps, a.warmup, sw, sh)
    if ref is not None:
        sec, build_s, threads, _ = ref
        secs = [sec]
        kind = "reference"
        what = "reference DumbRenderer (CPU threads) compiled from the reference sources"
    else:
        osc = O.OracleScene(tris, mat_id=mat, materials=mats, lights=lights, threads=threads)
        build_s = 0.0
        p = dr.render_params(sw, sh, dr.MODE_REFERENCE, samples=(1, 1), max_bounces=a.depth)
        for _ in range(a.warmup):
            osc.render_blocks(cam, p, threads=threads)
        secs = []
        for _ in range(a.steps):
            t0 = time.time()
            osc.render_blocks(cam, p, threads=threads)
            secs.append(time.time() - t0)
        kind = "port"
        what = "oracle restatement of DumbRenderer (reference library unavailable on this machine)"
    sec = float(np.mean(secs))
    value = paths / sec / 1e6
    out = {"metric": METRIC, "value": round(value, 5), "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": round(sec * 1e3, 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic", "impl": "reference",
           "config": {"workload": f"reference-expressible twin of the full path trace ({len(tris):,} tris, 4 spherical lights), "
                                  f"{sw}x{sh} sample of 1920x1080, 1 spp per step, depth {a.depth}",
                      "octree_build_s": round(build_s, 1)},
           "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": threads, "kind": kind,
                            "sample": f"{what}; {sw}x{sh} px x 1 spp per step ({paths:,} paths)"},
           "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.raycast_only:
        import torch
        import dumbray_gb300 as dr
        torch.cuda.set_device(0)
        peak, peak_src = measured_peak()
        print(json.dumps(run_raycast(dr, torch, torch.device("cuda", 0), a, peak, peak_src)), flush=True)
    elif a.twin_only:
        import torch
        import dumbray_gb300 as dr
        from dumbray_gb300 import scenes
        torch.cuda.set_device(0)
        peak, peak_src = measured_peak()
        out = run_reference_twin_gpu(dr, torch, torch.device("cuda", 0), a, scenes.full_scene(level=a.level, seed=1),
                                     peak, peak_src)
        print(json.dumps(out), flush=True)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
