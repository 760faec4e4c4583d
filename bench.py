"""Benchmark: Mrays/s of the octree raymarch hot path on GB300.

Workload (default, the plain-traversal configuration): a 2048^3 octree
(depth 11) of a 5-octave value-noise terrain (amplitude 0.3*N, 2-voxel shell)
plus 200 solid spheres with radii U[10, 120], built on the GPU from the dense
grid; 32 seeded cameras at 1920x1080 FP32 primary rays plus one shadow ray per
primary hit towards a fixed directional light.  One step traces all primary
rays and all shadow rays.  Primary rays return what the reference computes
per pixel: raymarch's t and leaf word (its `normal`) and the viewer's 8-bit
colour (renderTile's RGBA8 packing of shade()), 12 B per ray.  Shadow rays
return the hit flag.  The step with the earlier 20-byte output set (t, leaf
index, shade as 3 floats) is timed beside it.
Inputs are synthetic (seeded generators in scenes.py) and resident in HBM
before timing; the octree (~1.8 GB) and ray arrays (~1.6 GB + shadow) are far
larger than L2, so no explicit flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's raymarch restated in C (the oracle,
the reference's own code cannot run on the GPU host) over all host threads on
the same octree and rays; rank 0 only.
Multi-GPU (torchrun): every rank traces its own 32 cameras over a replica of
the octree (weak scaling, no collective on the data path).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIDE = 2048
N_SPHERES = 200
SCENE_SEED = 1
N_CAMS = 32
W_PIX, H_PIX = 1920, 1080
MEM_BUDGET = 8 << 30
LIGHT = np.array([0.3, 0.8, 0.52], np.float32)
LIGHT = (LIGHT / np.linalg.norm(LIGHT)).astype(np.float32)


def shadow_offset(side):
    """Shadow-ray origin offset: 1.5 voxels along the light, float32."""
    return (np.float32(1.5 / side) * LIGHT).astype(np.float32)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--side", type=int, default=SIDE)
    p.add_argument("--cams", type=int, default=N_CAMS)
    p.add_argument("--width", type=int, default=W_PIX)
    p.add_argument("--height", type=int, default=H_PIX)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--config", type=int, default=1, choices=[0, 1, 2, 3, 4],
                   help="workload of the main line: 0 the 256^3 sphere union, 12 views at 1024x768; 1 plain "
                        "traversal of the 2048^3 terrain (default); 2 the 327,680-triangle mesh build at 1024^3; "
                        "3 batched vs plain over 96 octrees and views; 4 differentiable leaf shading fwd+bwd on "
                        "the 512^3 sphere union")
    p.add_argument("--sweeps", action="store_true",
                   help="batched workload: also time the table-cache depths and register budgets")
    p.add_argument("--no-extra", action="store_true",
                   help="skip the other workloads' legs (batched, shading, mesh build, frames) in the default run")
    p.add_argument("--views", type=int, default=96)
    p.add_argument("--max-side", type=int, default=0,
                   help="batched workload: clamp each octree's side to this (a smaller case for profiling)")
    p.add_argument("--train-steps", type=int, default=200, help="Adam steps of the leaf-shading leg")
    return p.parse_args()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "10"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a while to start; the timed region (about 0.1 s at the default
            # step count) begins once it is sampling, and only samples from then on count
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.005)
        except Exception:
            self.proc = None
        self.first = len(self.lines)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[self.first:] or self.lines[-1:]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "interval_ms": 10}


def smi_index(local):
    """nvidia-smi's index of this process's GPU."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    return vis.split(",")[local] if vis else local


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def rank_cameras(scenes, n, rank, center):
    """The n orbit cameras rank `rank` traces: every rank draws its own views
    (seed 1000 + rank) over its replica of the octree, so no rays are shared
    and nothing is exchanged on the data path."""
    return scenes.orbit_cameras(n, 1000 + rank, center, radius=1.25, radius_hi=2.0, pitch=45.0)


def reduce_over_ranks(torch, units, seconds, device):
    """The job's units (summed over ranks; ranks trace different views, so
    their shadow-ray counts differ) and its time (the slowest rank's)."""
    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return units, seconds
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return int(u.item()), float(t.item())


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def pack_rgba8(grey, hit):
    """The viewer's packed colour of a traced pixel (renderTile,
    Main.cpp:126-131), from the oracle's shade and hit flag."""
    g = np.where(hit == 1, grey, np.float32(0.0)).astype(np.float32)
    g = np.where(np.float32(1.0) < g, np.float32(1.0), g)
    c = (g.astype(np.float64) * 255.0).astype(np.uint32)
    return c | (c << 8) | (c << 16) | np.uint32(0xFF000000)


def cpu_trace_sample(oracle, words, prim_rays, shadow_rays, cam_slices, shadow_slices, gpu=None, budget_s=12.0):
    """Time the oracle's raymarch over whole cameras (primary + their shadow
    rays) on all host threads until about `budget_s` seconds have elapsed.
    With `gpu` (the GPU's t, word and rgba8 of the primary rays and hit of
    the shadow rays, as numpy arrays) every sampled camera is also compared
    with it bit for bit, outside the timed calls."""
    threads = cpu_threads()
    rays_done, elapsed, cams, exact = 0, 0.0, 0, True
    for (a, b), (sa, sb) in zip(cam_slices, shadow_slices):
        t0 = time.perf_counter()
        rp = oracle.raymarch(words, prim_rays[a:b], light=LIGHT, threads=threads)
        rs = oracle.raymarch(words, shadow_rays[sa:sb], threads=threads)
        elapsed += time.perf_counter() - t0
        if gpu is not None:
            exact = exact and np.array_equal(gpu["t"][a:b].view(np.uint32), rp["t"].view(np.uint32)) and \
                np.array_equal(gpu["word"][a:b].view(np.uint32), rp["word"]) and \
                np.array_equal(gpu["rgba8"][a:b].view(np.uint32), pack_rgba8(rp["grey"], rp["hit"])) and \
                np.array_equal(gpu["hit"][sa:sb], rs["hit"])
        rays_done += (b - a) + (sb - sa)
        cams += 1
        if elapsed >= budget_s:
            break
    return rays_done, elapsed, cams, threads, (exact if gpu is not None else None)


def setup_scene(args, rank, torch, svo, scenes):
    """Builds the octree on the GPU and the primary/shadow ray arrays."""
    side = args.side
    heights, centers, radii = scenes.terrain_scene_params(side, N_SPHERES, SCENE_SEED)
    t0 = time.perf_counter()
    bm = scenes.gpu_occupancy(side, heights, centers, radii)
    grid = scenes.gpu_payload_grid(bm, side)
    del bm
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    tree = svo.VoxelOctree(svo.VoxelData(grid, MEM_BUDGET))
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    # the same build again: its scratch now comes from the library's pool
    # instead of first-touch device allocations
    t0 = time.perf_counter()
    tree2 = svo.VoxelOctree(svo.VoxelData(grid, MEM_BUDGET))
    torch.cuda.synchronize()
    t_build_warm = time.perf_counter() - t0
    warm_same = bool(np.array_equal(tree2.words(), tree.words()))
    tree2.close()
    del tree2
    n_vox = int((grid != 0).sum().item())
    del grid
    torch.cuda.empty_cache()
    # the traversal's descriptor table (built by the first trace call anyway)
    t0 = time.perf_counter()
    n_tab = tree.table_size()
    t_table = time.perf_counter() - t0
    center = tree.center()
    cams = rank_cameras(scenes, args.cams, rank, center)
    npix = args.width * args.height
    prim = torch.empty((len(cams) * npix, 6), dtype=torch.float32, device="cuda")
    for i, cam in enumerate(cams):
        scenes.gpu_camera_rays(cam, args.width, args.height, out=prim[i * npix:(i + 1) * npix])
    # primary pass once to derive the shadow rays (setup, not timed)
    R = prim.shape[0]
    t = torch.empty(R, dtype=torch.float32, device="cuda")
    hit = torch.empty(R, dtype=torch.uint8, device="cuda")
    tree.trace(prim, out={"t": t, "hit": hit})
    torch.cuda.synchronize()
    # one shadow ray per hit, ordered by 8x4 pixel tile within each camera so
    # that a warp's 32 consecutive shadow rays start at neighbouring pixels
    pix = torch.arange(npix, device="cuda")
    px, py = pix % args.width, pix // args.width
    tiles_x = (args.width + 7) // 8
    tile_key = ((py // 4) * tiles_x + px // 8) * 32 + (py % 4) * 8 + px % 8
    order = torch.argsort(tile_key)
    perm = (torch.arange(len(cams), device="cuda")[:, None] * npix + order[None, :]).reshape(-1)
    idx = perm[hit[perm] == 1]
    del pix, px, py, tile_key, order, perm
    o = prim[idx, :3]
    d = prim[idx, 3:]
    p = o + t[idx, None] * d
    L = torch.from_numpy(LIGHT).cuda()
    so = p + torch.from_numpy(shadow_offset(side)).cuda()
    shadow = torch.cat([so, L.expand_as(so)], dim=1).contiguous()
    # per-camera slices of the shadow array (hits are in camera order)
    cam_of_hit = (idx // npix).cpu().numpy()
    counts = np.bincount(cam_of_hit, minlength=len(cams))
    starts = np.concatenate([[0], np.cumsum(counts)])
    shadow_slices = [(int(starts[i]), int(starts[i + 1])) for i in range(len(cams))]
    cam_slices = [(i * npix, (i + 1) * npix) for i in range(len(cams))]
    del t, hit, idx, o, d, p, so
    info = {"gen_s": t_gen, "build_s": t_build, "build_warm_s": t_build_warm, "warm_same": warm_same, "voxels": n_vox, "words": tree.num_words(), "table_s": t_table,
            "table_entries": n_tab}
    return tree, prim, shadow, cam_slices, shadow_slices, info


def host_link_rates(torch, host):
    """This machine's host link: one pinned copy of `host` (a numpy array in
    page-locked memory) to the device and back, GB/s each way.  It sets the
    e2e figure, which moves the rays in and the results out; the rate differs
    between boxes."""
    src = torch.from_numpy(host.reshape(-1).view(np.uint8))
    dev = torch.empty(src.numel(), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dev.copy_(src, non_blocking=True)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    src.copy_(dev, non_blocking=True)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    n = src.numel()
    del dev
    return {"h2d": round(n / (t1 - t0) / 1e9, 1), "d2h": round(n / (t2 - t1) / 1e9, 1), "bytes": int(n)}


def workload_config(args, n_words, n_vox, Rp, Rs, world):
    """The plain-traversal workload's `config`, identical in both arms."""
    return {"workload": "plain traversal: %d^3 octree (terrain + %d spheres), %d cams %dx%d primary rays "
                        "+ 1 shadow ray per hit" % (args.side, N_SPHERES, args.cams, args.width, args.height),
            "outputs": {"primary": "t, leaf word (raymarch's normal), RGBA8 colour (renderTile's packing of "
                                   "shade()): 12 B/ray", "shadow": "hit flag: 1 B/ray"},
            "octree_words": int(n_words), "voxels": int(n_vox), "primary_rays": int(Rp), "shadow_rays": int(Rs),
            "rays_per_step": int(Rp + Rs),
            "l2": "no flush: octree %.2f GB and rays %.2f GB exceed L2" % (n_words * 4 / 1e9, (Rp + Rs) * 24 / 1e9),
            "parallelism": "replicas x%d" % world}


def _timed(torch, fn, steps, warmup, stream, events=None):
    for _ in range(warmup):
        fn(None)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(steps):
        fn(events[k] if events else None)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def run_ours(args):
    rank, world, local = dist_setup(args)
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__ as ge
    ge.build()
    svo = ge._package()
    import svo_gb300.scenes as scenes

    if args.config == 4:
        r4 = run_leaf_shading(args, torch, svo, scenes, n_steps=args.train_steps)
        if rank == 0:
            print(json.dumps({"metric": "fwd+bwd Mrays/s", "value": r4["fwd_bwd_mrays_s"], "unit": "Mrays/s",
                              "n_gpus": world, "steps": r4["steps"], "warmup": 0,
                              "ms_per_step": r4["step_ms_with_adam"], "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                              "config": {"workload": "differentiable: " + r4["workload"]}, "fwd_bwd": r4,
                              "gpu_launches": 4 * r4["steps"]}))
        return

    if args.config == 2:
        r2 = run_mesh_build(args, torch, svo, scenes, check=not args.no_cpu)
        if rank == 0:
            print(json.dumps({"metric": "voxels/s", "value": r2["voxels_per_s"], "unit": "voxels/s",
                              "n_gpus": world, "steps": r2["steps"], "warmup": r2["warmup"],
                              "ms_per_step": r2["build_ms"], "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                              "config": {"workload": "mesh build: " + r2["workload"]},
                              "e2e": {"value": r2["e2e_voxels_per_s"], "unit": "voxels/s",
                                      "h2d_bytes_per_step": r2["ply_bytes"], "d2h_bytes_per_step": 0},
                              "mesh_build": r2, "cpu_baseline": r2["cpu_baseline"],
                              "gpu_launches": r2["launches_per_build"] * r2["steps"]}))
        return

    if args.config == 0:
        r0 = run_sphere_views(args, torch, svo, scenes)
        if rank == 0:
            print(json.dumps({"metric": "Mrays/s", "value": r0["mrays_s"], "unit": "Mrays/s", "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": r0["ms_per_step"],
                              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                              "data": "synthetic (seeded sphere union, seeded orbit cameras)",
                              "config": {"workload": r0["workload"], "l2": r0["l2"]}, "e2e": r0["e2e"],
                              "roofline": r0["roofline"], "cpu_baseline": r0["cpu_baseline"],
                              "sphere_views": r0, "gpu_launches": r0["launches_per_step"] * args.steps}))
        return

    if args.config == 3:
        r3 = run_batched(args, torch, svo, scenes)
        if rank == 0:
            print(json.dumps({"metric": "Mrays/s", "value": r3["batched_mrays_s"], "unit": "Mrays/s",
                              "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": r3["batched_ms"], "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                              "config": {"workload": "batched: " + r3["workload"]}, "batched_vs_plain": r3,
                              "gpu_launches": args.steps}))
        return

    tree, prim, shadow, cam_slices, shadow_slices, info = setup_scene(args, rank, torch, svo, scenes)
    Rp, Rs = prim.shape[0], shadow.shape[0]
    W, H = args.width, args.height * args.cams  # the cameras' images stacked row-major
    rays_per_step = Rp + Rs
    # primary rays: t, leaf word, RGBA8 colour (12 B); shadow rays: hit (1 B)
    mk = lambda: ({"t": torch.empty(Rp, dtype=torch.float32, device="cuda"),
                   "word": torch.empty(Rp, dtype=torch.int32, device="cuda"),
                   "rgba8": torch.empty(Rp, dtype=torch.int32, device="cuda")},
                  {"hit": torch.empty(Rs, dtype=torch.uint8, device="cuda")})
    out_p, out_s = mk()
    stream = torch.cuda.current_stream()

    # loads per ray (the reference's word reads), for the algorithmic bytes
    loads = torch.empty(max(Rp, Rs), dtype=torch.int32, device="cuda")
    tree.count_loads(prim, loads=loads[:Rp])
    lp = int(loads[:Rp].sum().item())
    tree.count_loads(shadow, loads=loads[:Rs])
    ls = int(loads[:Rs].sum().item())
    del loads
    bytes_prim = 4 * lp + Rp * (24 + 12)
    bytes_shadow = 4 * ls + Rs * (24 + 1)

    # 1. the drop-in path: svo_trace_image (primary rays) + svo_trace (shadow rays)
    def image_step(ev):
        if ev is not None:
            ev[0].record(stream)
        tree.trace_image(prim, W, H, out=out_p, light=LIGHT, stream=stream)
        if ev is not None:
            ev[1].record(stream)
        tree.trace(shadow, out=out_s, stream=stream)
        if ev is not None:
            ev[2].record(stream)

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler(smi_index(local)) as clk:
        ms = _timed(torch, image_step, args.steps, args.warmup, stream, evs)
    if world > 1:
        torch.distributed.barrier()
    t_prim = [e[0].elapsed_time(e[1]) for e in evs]
    t_shadow = [e[1].elapsed_time(e[2]) for e in evs]
    if tree.device_status() != 0:
        raise RuntimeError("traversal error flag raised")
    ref_p = {k: v.clone() for k, v in out_p.items()}
    ref_s = out_s["hit"].clone()
    total_rays, ms_max = reduce_over_ranks(torch, rays_per_step * args.steps, ms, "cuda")
    value = total_rays / (ms_max / 1e3) / 1e6

    # 2. the plain per-ray kernel on the same rays (svo_trace for both sets)
    out_p2, out_s2 = mk()

    def plain_step(ev):
        tree.trace(prim, out=out_p2, light=LIGHT, stream=stream)
        tree.trace(shadow, out=out_s2, stream=stream)

    ms_plain = _timed(torch, plain_step, args.steps, args.warmup, stream) / args.steps
    exact_plain = all(torch.equal(out_p2[k], ref_p[k]) for k in ref_p) and torch.equal(out_s2["hit"], ref_s)
    del out_p2, out_s2

    # the same step with the 20-byte primary output set: t, leaf index, shade as 3 floats
    out_f = {"t": torch.empty(Rp, dtype=torch.float32, device="cuda"),
             "leaf": torch.empty(Rp, dtype=torch.int32, device="cuda"),
             "rgb": torch.empty((Rp, 3), dtype=torch.float32, device="cuda")}
    out_sf = {"hit": torch.empty(Rs, dtype=torch.uint8, device="cuda")}
    ev_f = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]

    def f32_step(ev):
        if ev is not None:
            ev[0].record(stream)
        tree.trace_image(prim, W, H, out=out_f, light=LIGHT, stream=stream)
        if ev is not None:
            ev[1].record(stream)
        tree.trace(shadow, out=out_sf, stream=stream)
        if ev is not None:
            ev[2].record(stream)

    ms_f32 = _timed(torch, f32_step, args.steps, args.warmup, stream, ev_f) / args.steps
    t_prim_f32 = sum(e[0].elapsed_time(e[1]) for e in ev_f) / len(ev_f)
    rgba_f = torch.where(out_f["leaf"] != -1, out_f["rgb"][:, 0], torch.zeros_like(out_f["t"]))
    c8 = (torch.clamp(rgba_f, max=1.0).double() * 255.0).to(torch.int64)
    rgba_f = (c8 | (c8 << 8) | (c8 << 16) | 0xFF000000).to(torch.int64)
    exact_f32 = torch.equal(out_f["t"], ref_p["t"]) and \
        torch.equal(rgba_f, ref_p["rgba8"].to(torch.int64) & 0xFFFFFFFF) and torch.equal(out_sf["hit"], ref_s)
    alt_outputs = {"primary_outputs": "t, leaf index, shade as 3 floats (20 B/ray)",
                   "ms_per_step": round(ms_f32, 3), "mrays_s": round(rays_per_step / ms_f32 / 1e3, 1),
                   "primary_launch_ms": round(t_prim_f32, 3), "same_t_and_colour": bool(exact_f32)}
    del out_f, out_sf, rgba_f, c8

    # 3. one autotuned, graph-captured persistent launch over the 32 images + the shadow rays
    npix = args.width * args.height
    out_p3, out_s3 = mk()
    views = [{"octree": tree, "rays": prim[i * npix:(i + 1) * npix], "width": args.width, "height": args.height,
              "light": LIGHT, "out": {k: v[i * npix:(i + 1) * npix] for k, v in out_p3.items()}}
             for i in range(args.cams)]
    views.append({"octree": tree, "rays": shadow, "out": out_s3})
    batch = svo.Batch(views)
    cfg, _ = batch.autotune()
    batch.capture_graph(cfg)
    ms_batched = _timed(torch, lambda ev: batch.launch_graph(stream), args.steps, args.warmup, stream) / args.steps
    exact_batched = all(torch.equal(out_p3[k], ref_p[k]) for k in ref_p) and torch.equal(out_s3["hit"], ref_s)
    del batch, views, out_p3, out_s3

    # end to end through the C ABI with host buffers (copies inside the timed region)
    e2e = None
    if not args.no_e2e:
        hp_pin = prim.cpu().pin_memory().numpy()
        hs_pin = shadow.cpu().pin_memory().numpy()
        op = {"t": torch.empty(Rp, dtype=torch.float32).pin_memory().numpy(),
              "word": torch.empty(Rp, dtype=torch.int32).pin_memory().numpy(),
              "rgba8": torch.empty(Rp, dtype=torch.int32).pin_memory().numpy()}
        os_ = {"hit": torch.empty(Rs, dtype=torch.uint8).pin_memory().numpy()}
        def host_step():
            # both calls queued on the handle's host pipeline.  The shadow call
            # (trace-bound) goes first, so its traces run while the primary
            # call's rays (copy-bound) cross the link: 12.2 ms per step against
            # 12.6-13.3 ms in the other order, alternated in one run
            tree.trace_host(hs_pin, out=os_, wait=False)
            tree.trace_image_host(hp_pin, W, H, light=LIGHT, out=op, wait=False)
            tree.synchronize()

        for _ in range(max(1, args.warmup)):
            host_step()
        if world > 1:
            torch.distributed.barrier()
        # Every step is timed on its own: a single step now and then stalls
        # for 5-70 ms on the host side (the same calls made one at a time in
        # the same run are unaffected), and one such stall moves a 10-step
        # mean by up to 50%.  The figure is the median step; the mean and
        # every step's time are reported with it.
        step_s = []
        for _ in range(args.steps):
            ta = time.perf_counter()
            host_step()
            step_s.append(time.perf_counter() - ta)
        e2e_median_s = statistics.median(step_s)
        _, e2e_s = reduce_over_ranks(torch, 0, e2e_median_s * args.steps, "cuda")
        _, e2e_mean_s = reduce_over_ranks(torch, 0, sum(step_s), "cuda")
        exact_e2e = all(np.array_equal(op[k].view(np.uint32), ref_p[k].cpu().numpy().view(np.uint32))
                        for k in op) and np.array_equal(os_["hit"], ref_s.cpu().numpy())
        # the same two calls, each waiting for its results (not the e2e figure)
        t_calls = [0.0, 0.0]
        n_sync = max(1, min(args.steps, 5))
        for _ in range(n_sync):
            ta = time.perf_counter()
            tree.trace_image_host(hp_pin, W, H, light=LIGHT, out=op)
            tb = time.perf_counter()
            tree.trace_host(hs_pin, out=os_)
            t_calls[0] += tb - ta
            t_calls[1] += time.perf_counter() - tb
        e2e = {"value": round(total_rays / e2e_s / 1e6, 2), "unit": "Mrays/s",
               "h2d_bytes_per_step": (Rp + Rs) * 24, "d2h_bytes_per_step": Rp * 12 + Rs * 1,
               "api": "svo_trace_host_async (shadow) + svo_trace_image_host_async (primary) + "
                      "svo_octree_synchronize: pinned host rays in, t/word/rgba8 and shadow hit out",
               "exact": bool(exact_e2e), "step_ms": round(e2e_s / args.steps * 1e3, 3),
               "statistic": "median step (slowest rank)",
               "mean_value": round(total_rays / e2e_mean_s / 1e6, 2),
               "step_ms_all": [round(t * 1e3, 2) for t in step_s],
               "waiting_calls_ms": {"primary": round(t_calls[0] / n_sync * 1e3, 3),
                                    "shadow": round(t_calls[1] / n_sync * 1e3, 3)},
               "link_gbs": host_link_rates(torch, hp_pin)}
        del hp_pin, hs_pin, op, os_

    peaks, peak_kind = load_peaks()
    t_prim_avg = sum(t_prim) / len(t_prim)
    achieved = bytes_prim / (t_prim_avg / 1e3) / 1e9
    traffic, traffic_source = profiled_traffic(Rp)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": traffic, "traffic_source": traffic_source,
                "kernel": "k_trace_single (svo_trace_image, primary rays)", "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": bytes_prim, "bytes_per_ray": round(bytes_prim / Rp, 2),
                "launch_ms": round(t_prim_avg, 3), "issue_bound": profiled_issue()}

    cpu = None
    oracle_parity = None
    frames = None
    oracle = words = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        pyoracle.build_oracle(with_reference=False)
        oracle = pyoracle.Oracle()
        words = tree.words()
        gpu = {k: v.cpu().numpy() for k, v in ref_p.items()}
        gpu["hit"] = ref_s.cpu().numpy()
        n, secs, ncam, thr, exact_cpu = cpu_trace_sample(oracle, words, prim.cpu().numpy(), shadow.cpu().numpy(),
                                                         cam_slices, shadow_slices, gpu=gpu)
        del gpu
        cpu = {"value": round(n / secs / 1e6, 3), "unit": "Mrays/s", "cores": thr, "kind": "port",
               "sample": "%d of %d cameras: %d primary+shadow rays in %.1f s (oracle C restatement of "
                         "VoxelOctree::raymarch, %d threads)" % (ncam, len(cam_slices), n, secs, thr)}
        # the octree's words against the oracle's build of the same scene
        # (CPU scene generator + sorted-voxel build, oracle/scene_build.c)
        t0 = time.perf_counter()
        heights, centers, radii = scenes.terrain_scene_params(args.side, N_SPHERES, SCENE_SEED)
        keys, pay = oracle.scene_voxels(args.side, heights, scenes.sphere_boxes((args.side,) * 3, centers, radii),
                                        np.concatenate([centers, radii[:, None]], 1), threads=cpu_threads())
        o_words = oracle.build_sorted(keys, pay, args.side.bit_length() - 1)
        del keys, pay
        words_exact = bool(o_words.size == words.size and np.array_equal(o_words, words))
        del o_words
        oracle_parity = {"cameras": ncam, "rays": n, "exact": bool(exact_cpu), "words_exact": words_exact,
                         "words": int(words.size), "oracle_build_s": round(time.perf_counter() - t0, 1),
                         "what": "the timed step's primary t, leaf word and RGBA8 and shadow hit flags against "
                                 "the oracle's raymarch + shade on the same rays, bit for bit; words_exact: the GPU "
                                 "build's octree words against the oracle's build of the same scene"}
    if not args.no_extra and world == 1:
        center = tree.center()
        cams = rank_cameras(scenes, args.cams, rank, center)
        frames = {"scene": run_frames(args, torch, svo, tree, cams, oracle, words),
                  "dragon": run_dragon_frames(args, torch, svo, scenes, oracle)}
    del words

    extra = extra0 = extra2 = extra4 = extra_vf = None
    if not args.no_extra and world == 1:
        del prim, shadow, out_p, out_s, ref_p, ref_s, tree
        torch.cuda.empty_cache()
        extra0 = run_sphere_views(args, torch, svo, scenes)
        torch.cuda.empty_cache()
        extra = run_batched(args, torch, svo, scenes)
        torch.cuda.empty_cache()
        extra4 = run_leaf_shading(args, torch, svo, scenes)
        torch.cuda.empty_cache()
        extra2 = run_mesh_build(args, torch, svo, scenes, steps=3, warmup=1, check=not args.no_cpu)
        torch.cuda.empty_cache()
        extra_vf = run_voxel_file(args, torch, svo, scenes)

    if rank == 0:
        mr = lambda ms: round(rays_per_step / ms / 1e3, 1)
        line = {
            "metric": "Mrays/s", "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded terrain + spheres, seeded orbit cameras)",
            "config": workload_config(args, info["words"], info["voxels"], Rp, Rs, world),
            "api": "svo_trace_image (primary, 8x4-pixel tiles, persistent) + svo_trace (shadow rays, ordered "
                   "per camera by 8x4 pixel tile)",
            "e2e": e2e, "gpu_launches": 2 * args.steps, "roofline": roofline, "cpu_baseline": cpu,
            "oracle_parity": oracle_parity,
            "clocks": clk.summary(),
            "kernel_ms": {"primary": round(t_prim_avg, 3), "shadow": round(sum(t_shadow) / len(t_shadow), 3)},
            "plain": {"api": "svo_trace for primary (row order) and shadow rays", "ms_per_step": round(ms_plain, 3),
                      "mrays_s": mr(ms_plain), "exact_vs_value_path": bool(exact_plain)},
            "alt_outputs": alt_outputs,
            "batched": {"api": "svo_batch: 32 image views + shadow view, autotuned, CUDA graph",
                        "ms_per_step": round(ms_batched, 3), "mrays_s": mr(ms_batched),
                        "config": cfg.as_dict(), "exact_vs_value_path": bool(exact_batched)},
            "build": {"build_s": round(info["build_s"], 3), "build_warm_s": round(info["build_warm_s"], 4),
                      "voxels_per_s": round(info["voxels"] / info["build_s"], 1),
                      "warm_voxels_per_s": round(info["voxels"] / info["build_warm_s"], 1),
                      "warm_words_equal": info["warm_same"], "scene_gen_s": round(info["gen_s"], 3),
                      "descriptor_table_s": round(info["table_s"], 4),
                      "descriptor_table_entries": info["table_entries"]},
            "sphere_views": extra0,
            "batched_vs_plain": extra,
            "fwd_bwd": extra4,
            "mesh_build": extra2,
            "viewer_frames": frames,
            "voxel_file_build": extra_vf,
        }
        line["summary"] = summary_of(line)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def summary_of(line):
    """The legs' headline figures, printed last on the line."""
    g = lambda d, *ks: None if d is None else (g(d.get(ks[0]), *ks[1:]) if len(ks) > 1 else d.get(ks[0]))
    s = {"plain_traversal_mrays_s": line["value"], "plain_traversal_e2e_mrays_s": g(line, "e2e", "value"),
         "plain_traversal_exact": g(line, "oracle_parity", "exact"),
         "plain_traversal_words_exact": g(line, "oracle_parity", "words_exact"),
         "primary_roofline_frac": g(line, "roofline", "frac"),
         "cpu_baseline_mrays_s": g(line, "cpu_baseline", "value"),
         "sphere_views_mrays_s": g(line, "sphere_views", "mrays_s"),
         "sphere_views_exact": g(line, "sphere_views", "exact_vs_oracle"),
         "batched_mrays_s": g(line, "batched_vs_plain", "batched_mrays_s"),
         "plain_image_mrays_s": g(line, "batched_vs_plain", "plain_image_mrays_s"),
         "plain_queue_mrays_s": g(line, "batched_vs_plain", "plain_mrays_s"),
         "batched_speedup_vs_best_plain": g(line, "batched_vs_plain", "speedup_vs_best_plain"),
         "batched_exact_hit_parity": g(line, "batched_vs_plain", "exact_hit_parity"),
         "fwd_bwd_mrays_s": g(line, "fwd_bwd", "fwd_bwd_mrays_s"),
         "fwd_bwd_step_ms_with_adam": g(line, "fwd_bwd", "step_ms_with_adam"),
         "fwd_bwd_step_ms_dense_adam": g(line, "fwd_bwd", "dense_path", "step_ms_with_adam"),
         "fwd_bwd_hit_leaves_exact": g(line, "fwd_bwd", "check", "hit_leaves_exact"),
         "fwd_bwd_fd_max_rel": g(line, "fwd_bwd", "check", "fd_max_rel"),
         "fwd_bwd_fd_own_truncation_max_rel": g(line, "fwd_bwd", "check", "fp64_analytic_vs_fd_max_rel"),
         "fwd_bwd_richardson_fd_max_rel": g(line, "fwd_bwd", "check", "richardson_fd_max_rel"),
         "mesh_build_ms": g(line, "mesh_build", "build_ms"),
         "mesh_build_exact": g(line, "mesh_build", "exact_vs_oracle"),
         "octree_build_warm_ms": None if g(line, "build", "build_warm_s") is None
         else round(g(line, "build", "build_warm_s") * 1e3, 2)}
    return s


def run_sphere_views(args, torch, svo, scenes, n_views=12, W=1024, H=768):
    """The 256^3 sphere union (48 solid spheres, seed 0), 12 orbit views
    (radius 2, seeded yaw/pitch) at 1024x768, FP32 primary rays, each view
    shaded with its own headlight.  A step traces the 12 views with
    svo_trace_image, one launch per view, returning t, leaf word and RGBA8
    (12 B/ray).  e2e: svo_trace_image_host per view from pinned host rays.
    CPU baseline and parity: the oracle's raymarch + shade over all 12 views
    on all host threads, compared bit for bit."""
    side = 256
    grid = scenes.gpu_sphere_scene(side, 48, 0)
    tree = svo.VoxelOctree(svo.VoxelData(grid))
    del grid
    center = tree.center()
    cams = scenes.orbit_cameras(n_views, 0, center, radius=2.0)
    lights = [scenes.headlight(c) for c in cams]
    npix = W * H
    R = n_views * npix
    rays = torch.empty((R, 6), dtype=torch.float32, device="cuda")
    for i, c in enumerate(cams):
        scenes.gpu_camera_rays(c, W, H, out=rays[i * npix:(i + 1) * npix])
    out = {"t": torch.empty(R, dtype=torch.float32, device="cuda"),
           "word": torch.empty(R, dtype=torch.int32, device="cuda"),
           "rgba8": torch.empty(R, dtype=torch.int32, device="cuda")}
    views = [(rays[i * npix:(i + 1) * npix], {k: v[i * npix:(i + 1) * npix] for k, v in out.items()}, lights[i])
             for i in range(n_views)]
    stream = torch.cuda.current_stream()
    loads = torch.empty(R, dtype=torch.int32, device="cuda")
    tree.count_loads(rays, loads=loads)
    n_loads = int(loads.sum().item())
    del loads
    bytes_step = 4 * n_loads + R * (24 + 12)

    def step(ev):
        for r, o, l in views:
            tree.trace_image(r, W, H, out=o, light=l, stream=stream)

    with ClockSampler(smi_index(int(os.environ.get("LOCAL_RANK", "0")))) as clk:
        ms = _timed(torch, step, args.steps, args.warmup, stream) / args.steps
    assert tree.device_status() == 0
    gpu = {k: v.cpu().numpy().view(np.uint32) for k, v in out.items()}
    peaks, peak_kind = load_peaks()
    achieved = bytes_step / (ms / 1e3) / 1e9
    res = {"workload": "256^3 sphere union (48 spheres, seed 0), %d orbit views %dx%d, headlight shade" % (
               n_views, W, H),
           "api": "svo_trace_image, one launch per view", "rays_per_step": R, "octree_words": tree.num_words(),
           "ms_per_step": round(ms, 4), "mrays_s": round(R / ms / 1e3, 1), "launches_per_step": n_views,
           "l2": "no flush: rays %.0f MB + outputs %.0f MB per step exceed L2; the %.1f MB octree stays "
                 "L2-resident, as it does for the reference's CPU caches" % (R * 24 / 1e6, R * 12 / 1e6,
                                                                            tree.num_words() * 4 / 1e6),
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                        "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": None,
                        "traffic_source": "not captured for this workload",
                        "kernel": "k_trace_single (svo_trace_image)", "peak_kind": peak_kind,
                        "algorithmic_bytes_per_step": bytes_step, "bytes_per_ray": round(bytes_step / R, 2)},
           "clocks": clk.summary(), "e2e": None, "cpu_baseline": None, "exact_vs_oracle": None}
    if not args.no_e2e:
        h_rays = rays.cpu().pin_memory().numpy()
        h_out = {k: torch.empty(R, dtype=torch.int32 if k != "t" else torch.float32).pin_memory().numpy()
                 for k in out}
        hv = [(h_rays[i * npix:(i + 1) * npix], {k: v[i * npix:(i + 1) * npix] for k, v in h_out.items()},
               lights[i]) for i in range(n_views)]

        def host_step():
            for r, o, l in hv:
                tree.trace_image_host(r, W, H, light=l, out=o, wait=False)
            tree.synchronize()

        for _ in range(max(1, args.warmup)):
            host_step()
        step_s = []  # the median step, as for the headline e2e figure
        for _ in range(args.steps):
            ta = time.perf_counter()
            host_step()
            step_s.append(time.perf_counter() - ta)
        e2e_s = statistics.median(step_s)
        exact = all(np.array_equal(h_out[k].view(np.uint32), gpu[k]) for k in out)
        res["e2e"] = {"value": round(R / e2e_s / 1e6, 1), "unit": "Mrays/s", "h2d_bytes_per_step": R * 24,
                      "d2h_bytes_per_step": R * 12,
                      "api": "svo_trace_image_host_async per view + svo_octree_synchronize, pinned host buffers",
                      "statistic": "median step", "mean_value": round(R * len(step_s) / sum(step_s) / 1e6, 1),
                      "exact": bool(exact)}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        pyoracle.build_oracle(with_reference=False)
        oracle = pyoracle.Oracle()
        words = tree.words()
        h = rays.cpu().numpy()
        threads = cpu_threads()
        exact, secs = True, 0.0
        for i in range(n_views):
            sl = slice(i * npix, (i + 1) * npix)
            t0 = time.perf_counter()
            ref = oracle.raymarch(words, h[sl], light=lights[i], threads=threads)
            secs += time.perf_counter() - t0
            exact = exact and np.array_equal(gpu["t"][sl], ref["t"].view(np.uint32)) and \
                np.array_equal(gpu["word"][sl], ref["word"]) and \
                np.array_equal(gpu["rgba8"][sl], pack_rgba8(ref["grey"], ref["hit"]))
        res["exact_vs_oracle"] = bool(exact)
        res["cpu_baseline"] = {"value": round(R / secs / 1e6, 3), "unit": "Mrays/s", "cores": threads,
                               "kind": "port", "sample": "all %d views (%d rays) once, oracle C restatement of "
                                                         "VoxelOctree::raymarch + shade" % (n_views, R)}
    tree.close()
    return res


def run_batched(args, torch, svo, scenes, tune_cache=None):
    """Batched persistent launch (graph-captured, autotuned) against the plain
    per-view kernel over the 96 views of scenes.batched_views; checks exact parity."""
    t0 = time.perf_counter()
    views, plain_out, rays_list = [], [], []
    trees = []
    total_rays = 0
    for (i, side, gen, W, H) in scenes.batched_views(args.views):
        if args.max_side:
            side = min(side, args.max_side)
        grid = scenes.gpu_sphere_scene(side, 48, i) if gen == "sphere" else scenes.gpu_terrain_scene(side, 200, i)
        tree = svo.VoxelOctree(svo.VoxelData(grid))
        del grid
        trees.append(tree)
        cam = scenes.orbit_cameras(1, 5000 + i, tree.center(), radius=2.0)[0]
        rays = scenes.gpu_camera_rays(cam, W, H)
        light = scenes.headlight(cam)
        n = W * H
        mk = lambda: {"t": torch.empty(n, dtype=torch.float32, device="cuda"),
                      "leaf": torch.empty(n, dtype=torch.int32, device="cuda"),
                      "rgb": torch.empty((n, 3), dtype=torch.float32, device="cuda")}
        out_b, out_p, out_i = mk(), mk(), mk()
        views.append({"octree": tree, "rays": rays, "width": W, "height": H, "light": light, "out": out_b})
        plain_out.append((tree, rays, light, out_p, W, H, out_i))
        total_rays += n
    torch.cuda.empty_cache()
    setup_s = time.perf_counter() - t0
    batch = svo.Batch(views)
    if tune_cache:
        os.environ.setdefault("SVO_AUTOTUNE_CACHE", tune_cache)
    t0 = time.perf_counter()
    cfg, tune_ms = batch.autotune()
    tune_s = time.perf_counter() - t0
    batch.capture_graph(cfg)
    stream = torch.cuda.current_stream()

    def plain_step():
        for tree, rays, light, out, _, _, _ in plain_out:
            tree.trace(rays, out=out, light=light, stream=stream)

    def image_step():
        for tree, rays, light, _, W, H, out in plain_out:
            tree.trace_image(rays, W, H, out=out, light=light, stream=stream)

    def batched_step():
        batch.launch_graph(stream)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms_plain = timed(plain_step)
    ms_image = timed(image_step)
    ms_batched = timed(batched_step)
    same = lambda: all(torch.equal(v["out"][k], po[3][k]) for v, po in zip(views, plain_out)
                       for k in ("t", "leaf", "rgb"))
    exact = same()
    exact_image = all(torch.equal(po[6][k], po[3][k]) for po in plain_out for k in ("t", "leaf", "rgb"))
    ms_best_plain = min(ms_plain, ms_image)
    res = {"workload": None, "rays_per_step": total_rays, "octree_words": int(sum(t.num_words() for t in trees)),
           "plain_ms": round(ms_plain, 3), "plain_image_ms": round(ms_image, 3), "batched_ms": round(ms_batched, 3),
           "plain_mrays_s": round(total_rays / ms_plain / 1e3, 1),
           "plain_image_mrays_s": round(total_rays / ms_image / 1e3, 1),
           "batched_mrays_s": round(total_rays / ms_batched / 1e3, 1),
           "speedup": round(ms_plain / ms_batched, 3),
           "speedup_vs_best_plain": round(ms_best_plain / ms_batched, 3),
           "best_plain": "svo_trace_image" if ms_image <= ms_plain else "svo_trace",
           "exact_hit_parity": bool(exact and exact_image),
           "plain_apis": {"plain": "96 svo_trace launches (persistent, 32 rays per queue access, row order)",
                          "plain_image": "96 svo_trace_image launches (persistent, 8x4-pixel tiles)"},
           "config": cfg.as_dict(), "autotune_s": round(tune_s, 1), "setup_s": round(setup_s, 1),
           "launches": {"plain": len(views), "plain_image": len(views), "batched": 1}}
    depth_hi = min(11, args.max_side.bit_length() - 1) if args.max_side else 11
    res["workload"] = ("%d octrees (depth 7-%d, sphere/terrain generators, seeds 1..%d), one view each, "
                       "256x256..1920x1080 log-uniform pixels" % (len(views), depth_hi, len(views)))
    if not getattr(args, "sweeps", False):
        return res
    # the chosen plain-tile shape (or the default tile shape, when lane refill
    # won) at each per-warp table cache depth the autotuner tries
    base = cfg.as_dict()
    if base["refill_idle"] != 0:
        base.update(refill_idle=0, steps_per_round=1, chunk=32)
    cache_sweep = {}
    for ce in (0, 64, 256):
        if (base["block_threads"] // 32) * ce * 16 > 65536:
            continue
        c = svo.default_config(**dict(base, cache_entries=ce, reg_cap=0))
        ms = timed(lambda: batch.trace(c, stream))
        cache_sweep[str(ce)] = {"ms": round(ms, 3), "exact_hit_parity": bool(same())}
    # the chosen lane-refill shape (or the default one) with each register budget
    rbase = cfg.as_dict()
    if rbase["refill_idle"] == 0:
        rbase = svo.default_config().as_dict()
    reg_sweep = {}
    for cap in (0, 48):
        c = svo.default_config(**dict(rbase, reg_cap=cap))
        ms = timed(lambda: batch.trace(c, stream))
        reg_sweep[str(cap)] = {"ms": round(ms, 3), "exact_hit_parity": bool(same())}
    res["table_cache_sweep"] = {"shape": {k: v for k, v in base.items() if k not in ("cache_entries", "reg_cap")},
                                "ms_by_cache_entries": cache_sweep}
    res["register_budget_sweep"] = {"shape": {k: v for k, v in rbase.items() if k != "reg_cap"},
                                    "ms_by_reg_cap": reg_sweep}
    return res


FRAME_W, FRAME_H, FRAME_STRIPS = 1280, 720, 16  # the viewer's GWidth, GHeight, NumThreads (Main.cpp:47-59)


def run_frames(args, torch, svo, tree, cams, oracle=None, words=None, steps=None, label=None):
    """The viewer's frame loop (svo_render_frame: beam prepass + per-pixel
    trace + RGBA8, 1280x720 in 16 strips) over the cameras; device time per
    frame from CUDA events, parity and a CPU time from the oracle's
    restatement of renderBatch (all host threads)."""
    steps = steps or args.steps
    out = torch.empty((FRAME_H, FRAME_W), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    for cam in cams[:max(1, args.warmup)]:
        tree.render_frame(cam[:9], cam[9:12], FRAME_W, FRAME_H, FRAME_STRIPS, 1, out=out, stream=stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        for cam in cams:
            tree.render_frame(cam[:9], cam[9:12], FRAME_W, FRAME_H, FRAME_STRIPS, 1, out=out, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / (steps * len(cams))
    res = {"workload": label or "%d camera views" % len(cams), "frame": "%dx%d, %d strips" % (FRAME_W, FRAME_H,
                                                                                           FRAME_STRIPS),
           "frame_ms": round(ms, 4), "fps": round(1e3 / ms, 1), "mpix_s": round(FRAME_W * FRAME_H / ms / 1e3, 1)}
    assert tree.device_status() == 0
    if oracle is not None and words is not None:
        exact = True
        t_cpu, n_cpu = 0.0, 0
        for cam in (cams[0], cams[-1]):
            tree.render_frame(cam[:9], cam[9:12], FRAME_W, FRAME_H, FRAME_STRIPS, 1, out=out, stream=stream)
            gpu = out.cpu().numpy().view(np.uint32)
            t0 = time.perf_counter()
            ref = oracle.render_frame(words, cam[:9], cam[9:12], FRAME_W, FRAME_H, FRAME_STRIPS, 1,
                                      threads=cpu_threads())
            t_cpu += time.perf_counter() - t0
            n_cpu += 1
            exact = exact and bool(np.array_equal(gpu, ref))
        res["exact_vs_oracle"] = exact
        res["cpu_baseline"] = {"fps": round(n_cpu / t_cpu, 2), "cores": cpu_threads(), "kind": "port",
                               "sample": "%d frames of the oracle's renderBatch restatement" % n_cpu}
    return res


def run_dragon_frames(args, torch, svo, scenes, oracle=None):
    """The viewer's own model: the shipped XYZRGB dragon octree (words from
    the committed fixture) at 1280x720 from 16 orbit cameras."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "dragon.npz"))
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    cams = scenes.orbit_cameras(16, 77, g["center"], radius=1.0, radius_hi=2.0, pitch=45.0)
    return run_frames(args, torch, svo, tree, cams, oracle, g["words"] if oracle is not None else None,
                      steps=max(args.steps, 20), label="XYZRGB dragon (119,887 words), 16 camera views")


MESH_LEVEL, MESH_SEED, MESH_SIDE, MESH_THREADS, MESH_MEM = 7, 3, 1024, 16, 1 << 30
MESH_SLAB_MEM = 1 << 28  # 270 of the volume's 1023 slices per slab: four slabs


def profiled_launches_per_build():
    """Kernel launches of one mesh build, from the committed ncu launch list
    (profiles/mesh_build_icosphere1024.md)."""
    try:
        for line in open(os.path.join(ROOT, "profiles", "mesh_build_icosphere1024.md")):
            if line.startswith("launches per build:"):
                return int(line.split(":")[1])
    except OSError:
        pass
    return None


def profile_kernels(torch, fn):
    """Kernel launches of one untimed call of fn, from the CUDA activity
    trace: (launch count, {kernel: [launches, device ms]}) for the ten
    longest kernels; memcpy and memset records are not kernels."""
    try:
        from torch.profiler import ProfilerActivity, profile
        torch.cuda.synchronize()
        with profile(activities=[ProfilerActivity.CUDA]) as prof:
            r = fn()
            torch.cuda.synchronize()
        del r
        from torch.autograd import DeviceType
        rows = {}
        for ev in prof.key_averages():
            name = ev.key
            if ev.device_type != DeviceType.CUDA or name.startswith(("Memcpy", "Memset")):
                continue
            t = getattr(ev, "device_time_total", None)
            if t is None:
                t = getattr(ev, "cuda_time_total", 0.0)
            rows[name] = [int(ev.count), round(t / 1e3, 4)]
        total = sum(v[0] for v in rows.values())
        top = dict(sorted(rows.items(), key=lambda kv: -kv[1][1])[:10])
        return total, {(k[:60] + ".." if len(k) > 62 else k): v for k, v in top.items()}
    except Exception as e:  # the profiler is optional here
        return None, {"unavailable": repr(e)[:120]}


def run_mesh_build(args, torch, svo, scenes, steps=None, warmup=None, check=True):
    """Mesh build: a level-7 icosphere (327,680 triangles) radially displaced
    by 4-octave seeded noise (15% of the radius), per-vertex RGB ~U[0,255],
    written as a binary little-endian PLY (float xyz, uchar rgb); voxelized at
    1024^3 with the reference's triangle/box rule and built into an octree,
    with the reference's result parameters pinned: 16 worker threads (16
    sub-blocks per cache block) and a 1 GiB budget (512^3 cache blocks).
    Each step is one VoxelOctree(VoxelData(PlyLoader, side, mem, threads))
    from the device-resident mesh; e2e adds reading, parsing and uploading
    the PLY file (svo_octree_build_ply)."""
    import tempfile
    steps = steps or args.steps
    warmup = args.warmup if warmup is None else warmup
    pos, faces, col = scenes.displaced_icosphere(MESH_LEVEL, MESH_SEED)
    tmp = tempfile.mkdtemp(prefix="svo_mesh_")
    path = os.path.join(tmp, "icosphere7.ply")
    scenes.write_ply(path, pos, faces, colors=col)
    ply_bytes = os.path.getsize(path)
    t0 = time.perf_counter()
    loader = svo.PlyLoader(path)
    load_s = time.perf_counter() - t0
    data = svo.VoxelData(loader, MESH_SIDE, MESH_MEM, MESH_THREADS)
    times, tree = [], None
    for k in range(warmup + steps):
        tree = None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tree = svo.VoxelOctree(data)
        torch.cuda.synchronize()
        if k >= warmup:
            times.append(time.perf_counter() - t0)
    n_desc, n_leaves = tree.validate()
    words = tree.words()
    e2e = []
    for k in range(warmup + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t2 = svo.VoxelOctree(svo.VoxelData(svo.PlyLoader(path), MESH_SIDE, MESH_MEM, MESH_THREADS))
        torch.cuda.synchronize()
        if k >= warmup:
            e2e.append(time.perf_counter() - t0)
        del t2
    build_s = sorted(times)[len(times) // 2]
    e2e_s = sorted(e2e)[len(e2e) // 2]
    launches, kernels = profile_kernels(torch, lambda: svo.VoxelOctree(data))
    if not launches:  # no CUDA activity trace in this process: the count from the committed launch list
        launches = profiled_launches_per_build()
    out = {"workload": "level-7 displaced icosphere (327,680 triangles, seed %d) as binary PLY, %d^3, %d threads, "
                       "1 GiB budget" % (MESH_SEED, MESH_SIDE, MESH_THREADS),
           "triangles": loader.num_triangles, "voxels": int(n_leaves), "octree_words": int(words.size),
           "descriptors": int(n_desc), "steps": steps, "warmup": warmup,
           "build_ms": round(build_s * 1e3, 3), "build_ms_all": [round(t * 1e3, 3) for t in times],
           "voxels_per_s": round(n_leaves / build_s, 1), "e2e_ms": round(e2e_s * 1e3, 3),
           "e2e_voxels_per_s": round(n_leaves / e2e_s, 1), "ply_load_ms": round(load_s * 1e3, 3),
           "ply_bytes": ply_bytes, "launches_per_build": launches, "kernels": kernels, "cpu_baseline": None,
           "exact_vs_oracle": None}
    # the same mesh written out as a volume (PlyLoader::convertToVolume, the
    # builder's --mode 1): device time of svo_mesh_to_volume into one buffer
    w3, h3, d3 = loader.suggested_dimensions(MESH_SIDE)
    vol = torch.empty((d3, h3, w3), dtype=torch.int32, device="cuda")

    def time_volume(mem):
        vol_ms = []
        for k in range(warmup + steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            loader.to_volume(MESH_SIDE, MESH_THREADS, mem, out=vol)
            torch.cuda.synchronize()
            if k >= warmup:
                vol_ms.append((time.perf_counter() - t0) * 1e3)
        med = sorted(vol_ms)[len(vol_ms) // 2]
        slab = min(mem // (w3 * h3), d3)
        return {"cells": w3 * h3 * d3, "dims": [w3, h3, d3], "mem": mem, "slabs": -(-d3 // slab),
                "voxels": int(torch.count_nonzero(vol).item()), "ms": round(med, 3),
                "cells_per_s": round(w3 * h3 * d3 / (med / 1e3), 1), "exact_vs_oracle": None}

    # z-slabs of a budget below the volume: the reference's slab loop through
    # one buffer it never clears
    out["to_volume_slabs"] = time_volume(MESH_SLAB_MEM)
    slab_vol = vol.cpu().numpy().view(np.uint32).copy() if check else None
    out["to_volume"] = time_volume(MESH_MEM)
    out["to_volume"]["cpu_baseline"] = None
    if check:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        pyoracle.build_oracle(with_reference=False)
        oracle = pyoracle.Oracle()
        t0 = time.perf_counter()
        ow, oc = oracle.build_mesh(pos, faces, MESH_SIDE, MESH_THREADS, MESH_MEM, colors=col.astype(np.float32))
        cpu_s = time.perf_counter() - t0
        out["exact_vs_oracle"] = bool(np.array_equal(ow, words) and np.array_equal(oc, tree.center()))
        out["cpu_baseline"] = {"value": round(n_leaves / cpu_s, 1), "unit": "voxels/s", "cores": 1, "kind": "port",
                               "sample": "the full build (oracle/ply_oracle.c, single-threaded restatement of "
                                         "PlyLoader + VoxelData + VoxelOctree) on the same mesh",
                               "build_s": round(cpu_s, 3)}
        t0 = time.perf_counter()
        ov = oracle.mesh_to_volume(pos, faces, MESH_SIDE, MESH_THREADS, MESH_MEM, colors=col.astype(np.float32))
        cpu_v = time.perf_counter() - t0
        out["to_volume"]["exact_vs_oracle"] = bool(np.array_equal(ov, vol.cpu().numpy().view(np.uint32)))
        out["to_volume"]["cpu_baseline"] = {"s": round(cpu_v, 3), "cores": 1, "kind": "port",
                                            "sample": "oracle/ply_oracle.c's convertToVolume restatement, "
                                                      "single-threaded, same mesh and parameters"}
        del ov
        ov = oracle.mesh_to_volume(pos, faces, MESH_SIDE, MESH_THREADS, MESH_SLAB_MEM, colors=col.astype(np.float32))
        out["to_volume_slabs"]["exact_vs_oracle"] = bool(np.array_equal(ov, slab_vol))
        del ov, slab_vol
    del vol
    os.unlink(path)
    os.rmdir(tmp)
    return out


def run_voxel_file(args, torch, svo, scenes, side=512, slab_mib=64):
    """VoxelData(path, mem) + VoxelOctree from a .voxel file: the whole grid
    on the device versus the streamed form (slabs of about slab_mib MiB),
    both timed from the file (page cache warm) to the resident octree."""
    import tempfile
    grid = scenes.gpu_terrain_scene(side, 60, 5)
    d, h, w = grid.shape
    tmp = tempfile.mkdtemp(prefix="svo_vox_")
    path = os.path.join(tmp, "scene.voxel")
    with open(path, "wb") as f:
        f.write(np.array([w, h, d], np.int32).tobytes())
        f.write(grid.cpu().numpy().tobytes())
    del grid
    torch.cuda.empty_cache()

    def timed(data):
        best, tree = None, None
        for _ in range(3):
            tree = None
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            tree = svo.VoxelOctree(data)
            torch.cuda.synchronize()
            s = time.perf_counter() - t0
            best = s if best is None else min(best, s)
        return best, tree

    mem = 1 << 30
    t_whole, a = timed(svo.VoxelData(path, mem))
    t_stream, b = timed(svo.VoxelData(path, mem, slab_bytes=slab_mib << 20))
    nd, nl = a.validate()
    exact = bool(np.array_equal(a.words(), b.words()))
    os.unlink(path)
    os.rmdir(tmp)
    return {"workload": "%d^3 terrain + 60 spheres as a .voxel file (%.1f GiB), 1 GiB budget" % (side, w * h * d * 4 / 2 ** 30),
            "voxels": int(nl), "whole_grid_ms": round(t_whole * 1e3, 1), "streamed_ms": round(t_stream * 1e3, 1),
            "streamed_slab_mib": slab_mib, "streamed_voxels_per_s": round(nl / t_stream, 1),
            "streamed_equals_whole": exact,
            "note": "file read from the page cache inside the timed region; the streamed form keeps one slab and "
                    "the occupied voxels on the device instead of the whole grid"}


def run_leaf_shading(args, torch, svo, scenes, n_steps=200):
    """Differentiable leaf shading: 512^3 sphere union (160 spheres, seed 7),
    per-leaf FP32 rgb and normal parameters ~U[0,1], 24 views 512x512 against
    targets from a seeded 3-octave noise colour field; L2 loss, forward +
    hand-written adjoint, Adam lr 1e-2, 200 steps."""
    side, W, H, V = 512, 512, 512, 24
    t0 = time.perf_counter()
    grid = scenes.gpu_sphere_scene(side, 160, 7)
    tree = svo.VoxelOctree(svo.VoxelData(grid))
    del grid
    center = tree.center()
    cams = scenes.orbit_cameras(V, 7, center, radius=2.0)
    rays = torch.empty((V * W * H, 6), dtype=torch.float32, device="cuda")
    for i, c in enumerate(cams):
        scenes.gpu_camera_rays(c, W, H, out=rays[i * W * H:(i + 1) * W * H])
    lights = torch.from_numpy(np.stack([scenes.headlight(c) for c in cams]).astype(np.float32)).cuda()
    R = rays.shape[0]
    nw = tree.num_words()
    # targets: noise colour at the hit point, lit with the leaf's own normal
    t = torch.empty(R, dtype=torch.float32, device="cuda")
    word = torch.empty(R, dtype=torch.int32, device="cuda")
    hit = torch.empty(R, dtype=torch.uint8, device="cuda")
    for v in range(V):
        sl = slice(v * W * H, (v + 1) * W * H)
        tree.trace(rays[sl], out={"t": t[sl], "word": word[sl], "hit": hit[sl]})
    torch.cuda.synchronize()
    h = hit == 1
    p = rays[h, :3] + t[h, None] * rays[h, 3:]
    gt = torch.stack([scenes.noise3(p, 7 + k) for k in range(3)], 1)
    n = scenes.decompress_normal(word[h].to(torch.int64) & 0xFFFFFFFF)
    d = rays[h, 3:]
    l = lights.repeat_interleave(W * H, 0)[h]
    ln = (l * n).sum(1)
    r = d - 2 * (n * d).sum(1, keepdim=True) * n
    spec = torch.clamp((l * r).sum(1), min=0) ** 2 * 0.2
    target = torch.zeros((R, 3), dtype=torch.float32, device="cuda")
    target[h] = gt * 0.9 * ln.abs()[:, None] + spec[:, None]
    del t, word, p, gt, n, d, l, ln, r, spec
    gen = torch.Generator(device="cuda").manual_seed(7)
    p0_rgb = torch.rand((nw, 3), generator=gen, device="cuda")
    p0_n = torch.rand((nw, 3), generator=gen, device="cuda")
    rgb = torch.empty((R, 3), dtype=torch.float32, device="cuda")
    leaf = torch.empty(R, dtype=torch.int32, device="cuda")
    d_rgb = torch.empty((R, 3), dtype=torch.float32, device="cuda")
    scale = 2.0 / (3 * R)  # L = sum (rgb - target)^2 / (3R): dL/drgb = scale (rgb - target)
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    # one untimed forward + adjoint at the initial parameters, for the checks
    # against the oracle after the timed loops
    check = None
    if not args.no_cpu:
        g_rgb, g_n = torch.zeros_like(p0_rgb), torch.zeros_like(p0_n)
        tree.diff_forward(rays, W, H, V, lights, p0_rgb, p0_n, rgb, hit_leaf=leaf, stream=stream)
        torch.sub(rgb, target, out=d_rgb)
        d_rgb.mul_(scale)
        tree.diff_backward(rays, W, H, V, lights, p0_rgb, p0_n, d_rgb, g_rgb, g_n, hit_leaf=leaf, stream=stream)
        torch.cuda.synchronize()
        check = {"leaf": leaf.cpu().numpy().view(np.uint32), "g_rgb": g_rgb.cpu().numpy(), "g_n": g_n.cpu().numpy(),
                 "p_rgb": p0_rgb.cpu().numpy(), "p_n": p0_n.cpu().numpy(), "target": target.cpu().numpy()}
        del g_rgb, g_n

    def train(steps, fused):
        """`steps` optimisation steps from the initial parameters.  fused:
        the parameters as 8-float leaf records, svo_diff_backward_l2 (loss
        gradient and loss sum in the adjoint, touched leaves recorded) +
        svo_adam_step_leaves; else 3-float arrays, the loss gradient in torch
        + svo_diff_backward + dense svo_adam_step."""
        if fused:
            # one 32-byte record per leaf (rgb, normal, 2 unused floats):
            # each gather and each leaf's gradient atomics touch one sector,
            # and one Adam launch updates whole records
            rec = torch.zeros((nw, 8), dtype=torch.float32, device="cuda")
            rec[:, 0:3] = p0_rgb
            rec[:, 3:6] = p0_n
            grec = torch.zeros_like(rec)
            rec.grad = grec
            p_rgb, p_n, g_rgb, g_n = rec[:, 0:3], rec[:, 3:6], grec[:, 0:3], grec[:, 3:6]
            stride = 8
            leaves = svo.LeafSet(nw)
            opt = svo.LeafAdam([rec], lr=1e-2, leaves=leaves, width=8)  # zeroes the gradients it reads
        else:
            p_rgb, p_n = p0_rgb.clone(), p0_n.clone()
            g_rgb, g_n = torch.zeros_like(p_rgb), torch.zeros_like(p_n)
            p_rgb.grad, p_n.grad = g_rgb, g_n
            stride = 3
            leaves = None
            opt = svo.LeafAdam([p_rgb, p_n], lr=1e-2)
        loss_sum = torch.zeros(steps, dtype=torch.float64, device="cuda")
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(steps)]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for k in range(steps):
            ev[k][0].record(stream)
            tree.diff_forward(rays, W, H, V, lights, p_rgb, p_n, rgb, hit_leaf=leaf, stream=stream,
                              param_stride=stride)
            ev[k][1].record(stream)
            if fused:
                ev[k][2].record(stream)
                tree.diff_backward_l2(rays, W, H, V, lights, p_rgb, p_n, rgb, target, scale, g_rgb, g_n,
                                      hit_leaf=leaf, loss_sum=loss_sum[k:k + 1], leaves=leaves, stream=stream,
                                      param_stride=stride)
            else:
                torch.sub(rgb, target, out=d_rgb)
                loss_sum[k:k + 1] = d_rgb.double().square().sum()
                d_rgb.mul_(scale)
                ev[k][2].record(stream)
                tree.diff_backward(rays, W, H, V, lights, p_rgb, p_n, d_rgb, g_rgb, g_n, hit_leaf=leaf,
                                   stream=stream)
            ev[k][3].record(stream)
            opt.step(stream)
        e1.record(stream)
        torch.cuda.synchronize()
        fwd = [e[0].elapsed_time(e[1]) for e in ev]
        bwd = [e[2].elapsed_time(e[3]) for e in ev]
        loss = (loss_sum / (3 * R)).cpu().numpy()
        return {"step_ms": e0.elapsed_time(e1) / steps, "fwd_ms": sum(fwd) / steps, "bwd_ms": sum(bwd) / steps,
                "loss": loss, "touched_leaves": leaves.size() if fused else None}

    main = train(n_steps, fused=True)
    dense = train(min(20, n_steps), fused=False)
    fb = main["fwd_ms"] + main["bwd_ms"]
    nd = len(dense["loss"])
    if check is not None:
        check = shading_check(tree, rays.cpu().numpy(), lights.cpu().numpy(), W * H, check)
    return {"workload": "512^3 sphere union (160 spheres, seed 7), %d octree words; 24 views 512x512; per-leaf FP32 "
                        "rgb+normal params; L2 loss vs 3-octave noise colour field; Adam lr 1e-2" % nw,
            "rays_per_step": R, "steps": n_steps, "fwd_ms": round(main["fwd_ms"], 3),
            "bwd_ms": round(main["bwd_ms"], 3), "fwd_bwd_mrays_s": round(R / fb / 1e3, 1),
            "fwd_bwd_note": "svo_diff_forward + svo_diff_backward_l2 kernel time (CUDA events), parameters as 8-float "
                            "leaf records; the adjoint forms the L2 loss gradient and the loss itself; "
                            "step_ms_with_adam adds svo_adam_step_leaves over the leaves the adjoint has touched "
                            "(identical to the dense Adam pass)",
            "step_ms_with_adam": round(main["step_ms"], 3), "touched_leaves": main["touched_leaves"],
            "loss_first_last": [[0, round(float(main["loss"][0]), 6)],
                                [n_steps - 1, round(float(main["loss"][-1]), 6)]],
            "dense_path": {"steps": nd, "step_ms_with_adam": round(dense["step_ms"], 3),
                           "bwd_ms": round(dense["bwd_ms"], 3),
                           "what": "loss gradient in torch, svo_diff_backward, dense svo_adam_step over every word",
                           "loss_max_rel_diff_vs_fused": float(np.max(np.abs(dense["loss"] - main["loss"][:nd]) /
                                                                      main["loss"][:nd]))},
            "setup_s": round(setup_s, 1), "check": check}


def shading_check(tree, rays, lights, per_view, c, n_leaves=256, h=1e-3):
    """The leaf-shading leg's forward and adjoint at the initial parameters
    against the oracle: every ray's hit leaf against the oracle's raymarch
    (VoxelOctree::raymarch, leaf index at VoxelOctree.cpp:282), and the
    adjoint's gradient against plain FP64 central differences (h = 1e-3) of
    the same L2 loss on 256 random hit leaves (oracle/diff_oracle.py)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import diff_oracle
    import pyoracle
    pyoracle.build_oracle(with_reference=False)
    oracle = pyoracle.Oracle()
    t0 = time.perf_counter()
    ref = oracle.raymarch(tree.words(), rays, threads=cpu_threads())
    leaf = np.where(ref["hit"] == 1, ref["leaf"], np.uint32(0xFFFFFFFF)).astype(np.uint32)
    hit_exact = bool(np.array_equal(leaf, c["leaf"]))
    hit_leaves = np.unique(leaf[leaf != 0xFFFFFFFF])
    pick = np.random.default_rng(5).choice(hit_leaves, size=min(n_leaves, hit_leaves.size), replace=False)
    ray_light = np.repeat(lights, per_view, axis=0)
    w = 1.0 / (3 * rays.shape[0])
    fd_rgb, fd_n, kink = diff_oracle.finite_differences(leaf, rays[:, 3:], ray_light, c["p_rgb"], c["p_n"],
                                                        c["target"], w, pick, h=h)
    li = pick.astype(np.int64)
    rel = lambda g, r: np.linalg.norm(g - r, axis=-1) / np.linalg.norm(r, axis=-1)
    smooth = ~kink.any(axis=1)
    e_rgb = rel(c["g_rgb"][li], fd_rgb)
    e_n = rel(c["g_n"][li][smooth], fd_n[smooth])
    fd_max = float(max(e_rgb.max(), e_n.max() if smooth.any() else 0.0))
    # the same differences against the FP64 analytic gradient (how far plain
    # central differences at this h are from the exact derivative: their
    # O(h^2) term grows as 1/|p|^2 for short normal parameters), and the
    # adjoint against Richardson-extrapolated differences (h, h/2)
    a_rgb, a_n = diff_oracle.gradient(leaf, rays[:, 3:], ray_light, c["p_rgb"], c["p_n"], c["target"], w,
                                      c["p_rgb"].shape[0], leaves=pick)
    fd_floor = float(max(rel(a_rgb, fd_rgb).max(), rel(a_n[smooth], fd_n[smooth]).max() if smooth.any() else 0.0))
    r_rgb, r_n, _ = diff_oracle.finite_differences(leaf, rays[:, 3:], ray_light, c["p_rgb"], c["p_n"], c["target"],
                                                   w, pick, h=h, richardson=True)
    rich = float(max(rel(c["g_rgb"][li], r_rgb).max(), rel(c["g_n"][li][smooth], r_n[smooth]).max()))
    exact = float(max(rel(c["g_rgb"][li], a_rgb).max(), rel(c["g_n"][li], a_n).max()))
    worst = int(np.argmax(rel(c["g_n"][li], fd_n)))
    return {"hit_leaves_exact": hit_exact, "rays": int(rays.shape[0]), "hit_rays": int((leaf != 0xFFFFFFFF).sum()),
            "fd_leaves": int(pick.size), "fd_h": h, "fd_max_rel": round(fd_max, 8),
            "fd_rgb_max_rel": round(float(e_rgb.max()), 8),
            "fd_normal_max_rel": round(float(e_n.max()), 8) if smooth.any() else None,
            "fd_kink_leaves_left_out": int((~smooth).sum()),
            "fp64_analytic_vs_fd_max_rel": round(fd_floor, 8),
            "worst_leaf_normal_param_norm": round(float(np.linalg.norm(c["p_n"][li[worst]])), 4),
            "richardson_fd_max_rel": round(rich, 8), "fp64_analytic_max_rel": round(exact, 8),
            "check_s": round(time.perf_counter() - t0, 1),
            "what": "initial parameters: hit leaf of every ray vs the oracle's raymarch; adjoint gradient vs plain "
                    "FP64 central differences, vs Richardson-extrapolated ones and vs the FP64 analytic gradient "
                    "(relative error of each leaf's 3-vector); fp64_analytic_vs_fd is the plain differences' own "
                    "truncation error at this h"}


def profiled_traffic(rays):
    """DRAM bytes per launch from the committed ncu summaries (per ray, times
    the launch's rays), and where the figure comes from: it is read from a
    committed capture, not measured in this run."""
    for name, what in (("dram_trace_terrain2048.txt", "one-pass ncu capture (dram__bytes_read.sum + "
                                                      "dram__bytes_write.sum) of this kernel on this workload"),
                       ("trace_image_terrain1024.txt", "ncu capture of this kernel on the 1024^3 case")):
        try:
            for line in open(os.path.join(ROOT, "profiles", name)):
                if line.startswith("dram_bytes_per_ray:"):
                    b = float(line.split(":")[1])
                    return int(b * rays), "profiles/%s: %s, %.1f B/ray x this launch's rays; not measured in " \
                                          "this run" % (name, what, b)
        except OSError:
            pass
    return None, None


def profiled_issue():
    """Issue utilisation of the primary-ray kernel from the committed ncu
    summary: the bound this kernel actually meets (it is issue-bound on the
    ALU pipe, with DRAM at about 5% of peak)."""
    path = os.path.join(ROOT, "profiles", "trace_image_terrain1024.txt")
    import re
    out = {}
    first = lambda line: float(re.findall(r"(?<![\w.])(\d+\.\d+|\d+)(?![\w.])", line.split(")")[-1] if ")" in line
                                          else line.split(None, 1)[1])[0])
    try:
        for line in open(path):
            if line.startswith("smsp__issue_active"):
                out["issue_active_pct"] = first(line)
            elif line.startswith("sm__inst_executed_pipe_alu"):
                out["alu_pipe_pct"] = first(line)
            elif line.startswith("smsp__thread_inst_executed_per_inst_executed"):
                out["simt_lanes_of_32"] = first(line)
    except (OSError, ValueError, IndexError):
        return None
    out["source"] = "profiles/trace_image_terrain1024.txt (ncu --set full, same kernel, smaller case)"
    return out or None


def run_reference(args):
    """The reference's raymarch (VoxelOctree::raymarch restated in C, the
    oracle) over all host threads, on the same octree and rays as our arm.
    Setup uses no GPU code: the scene and octree come from oracle/scene_build.c
    and the rays from scenes.py (both bit-identical to the GPU generators)."""
    rank, world, local = dist_setup(args)
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import importlib.util
    import pyoracle
    pyoracle.build_oracle(with_reference=False)
    oracle = pyoracle.Oracle()
    spec = importlib.util.spec_from_file_location("svo_scenes_cpu",
                                                  os.path.join(ROOT, "sparse-voxel-octrees_gb300", "scenes.py"))
    scenes = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(scenes)
    threads = cpu_threads()
    side = args.side
    log_side = side.bit_length() - 1
    t0 = time.perf_counter()
    heights, centers, radii = scenes.terrain_scene_params(side, N_SPHERES, SCENE_SEED)
    boxes = scenes.sphere_boxes((side,) * 3, centers, radii)
    params = np.concatenate([centers, radii[:, None]], 1)
    keys, pay = oracle.scene_voxels(side, heights, boxes, params, threads=threads)
    words = oracle.build_sorted(keys, pay, log_side)
    n_vox = keys.size
    del keys, pay
    center = np.array([0.5, 0.5, 0.5], np.float32)
    cams = rank_cameras(scenes, args.cams, rank, center)
    prims = [scenes.camera_rays(c, args.width, args.height) for c in cams]
    shadows = []
    for r in prims:  # primary pass once to derive the shadow rays, as in our arm
        out = oracle.raymarch(words, r, threads=threads)
        hit = out["hit"] == 1
        p = r[hit, :3] + out["t"][hit, None] * r[hit, 3:]
        so = p + shadow_offset(side)
        shadows.append(np.concatenate([so, np.broadcast_to(LIGHT, so.shape)], 1).astype(np.float32))
    setup_s = time.perf_counter() - t0
    Rp = sum(p.shape[0] for p in prims)
    Rs = sum(x.shape[0] for x in shadows)

    def step():
        # the whole workload: every camera's primary rays, then its shadow rays
        for p, sh in zip(prims, shadows):
            oracle.raymarch(words, p, light=LIGHT, threads=threads)
            oracle.raymarch(words, sh, threads=threads)
        return Rp + Rs

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    rays = 0
    for _ in range(args.steps):
        rays += step()
    secs = time.perf_counter() - t0
    value = rays / secs / 1e6
    sample = ("the full step, all %d cameras (primary + shadow rays, %d rays) per step; %d rays in %.1f s on %d "
              "host threads; oracle C restatement of VoxelOctree::raymarch + shade (the reference's own sources are "
              "absent on the GPU host)" % (len(prims), Rp + Rs, rays, secs, threads))
    line = {
        "impl": "reference", "metric": "Mrays/s", "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded terrain + spheres, seeded orbit cameras)",
        "config": workload_config(args, words.size, n_vox, Rp, Rs, world),
        "api": "oracle raymarch (VoxelOctree::raymarch restated in C) over all host threads, rows interleaved",
        "setup_s": round(setup_s, 1),
        "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
