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
    p.add_argument("--config", type=int, default=1, choices=[1, 2, 3, 4],
                   help="workload of the main line: 1 plain traversal of the 2048^3 terrain (default); 2 the "
                        "327,680-triangle mesh build at 1024^3; 3 batched vs plain over 96 octrees and views; "
                        "4 differentiable leaf shading fwd+bwd on the 512^3 sphere union")
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
                                          "--format=csv,noheader,nounits", "-lms", "20"],
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
                "samples": len(sm), "interval_ms": 20}


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
                              "gpu_launches": 2 * r4["steps"]}))
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
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    smi_index = vis.split(",")[local] if vis else local
    with ClockSampler(smi_index) as clk:
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
        for _ in range(max(1, args.warmup)):
            tree.trace_image_host(hp_pin, W, H, light=LIGHT, out=op)
            tree.trace_host(hs_pin, out=os_)
        if world > 1:
            torch.distributed.barrier()
        t_calls = [0.0, 0.0]
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ta = time.perf_counter()
            tree.trace_image_host(hp_pin, W, H, light=LIGHT, out=op)
            tb = time.perf_counter()
            tree.trace_host(hs_pin, out=os_)
            t_calls[0] += tb - ta
            t_calls[1] += time.perf_counter() - tb
        _, e2e_s = reduce_over_ranks(torch, 0, time.perf_counter() - t0, "cuda")
        exact_e2e = all(np.array_equal(op[k].view(np.uint32), ref_p[k].cpu().numpy().view(np.uint32))
                        for k in op) and np.array_equal(os_["hit"], ref_s.cpu().numpy())
        e2e = {"value": round(total_rays / e2e_s / 1e6, 2), "unit": "Mrays/s",
               "h2d_bytes_per_step": (Rp + Rs) * 24, "d2h_bytes_per_step": Rp * 12 + Rs * 1,
               "api": "svo_trace_image_host (primary) + svo_trace_host (shadow): pinned host rays in, "
                      "t/word/rgba8 and shadow hit out", "exact": bool(exact_e2e),
               "call_ms": {"primary": round(t_calls[0] / args.steps * 1e3, 3),
                           "shadow": round(t_calls[1] / args.steps * 1e3, 3)}}
        del hp_pin, hs_pin, op, os_

    peaks, peak_kind = load_peaks()
    t_prim_avg = sum(t_prim) / len(t_prim)
    achieved = bytes_prim / (t_prim_avg / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": profiled_traffic(Rp),
                "kernel": "k_trace_single (svo_trace_image, primary rays)", "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": bytes_prim, "issue_bound": profiled_issue(),
                "bytes_per_ray": round(bytes_prim / Rp, 2), "launch_ms": round(t_prim_avg, 3)}

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
        oracle_parity = {"cameras": ncam, "rays": n, "exact": bool(exact_cpu),
                         "what": "the timed step's primary t, leaf word and RGBA8 and shadow hit flags against "
                                 "the oracle's raymarch + shade on the same words and rays, bit for bit"}
    if not args.no_extra and world == 1:
        center = tree.center()
        cams = rank_cameras(scenes, args.cams, rank, center)
        frames = {"scene": run_frames(args, torch, svo, tree, cams, oracle, words),
                  "dragon": run_dragon_frames(args, torch, svo, scenes, oracle)}
    del words

    extra = extra2 = extra4 = extra_vf = None
    if not args.no_extra and world == 1:
        del prim, shadow, out_p, out_s, ref_p, ref_s, tree
        torch.cuda.empty_cache()
        extra = run_batched(args, torch, svo, scenes)
        torch.cuda.empty_cache()
        extra4 = run_leaf_shading(args, torch, svo, scenes)
        torch.cuda.empty_cache()
        extra2 = run_mesh_build(args, torch, svo, scenes, steps=3, warmup=1, check=not args.no_cpu)
        torch.cuda.empty_cache()
        extra_vf = run_voxel_file(args, torch, svo, scenes)

    if rank == 0:
        line = {
            "metric": "Mrays/s", "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded terrain + spheres, seeded orbit cameras)",
            "config": {"workload": "plain traversal: %d^3 octree (terrain + %d spheres), %d cams %dx%d primary rays "
                                   "+ 1 shadow ray per hit" % (args.side, N_SPHERES, args.cams, args.width,
                                                               args.height),
                       "shadow_ray_order": "per camera, by 8x4 pixel tile",
                       "outputs": {"primary": "t, leaf word (raymarch's normal), RGBA8 colour (renderTile's "
                                              "packing of shade()): 12 B/ray", "shadow": "hit flag: 1 B/ray"},
                       "api": "svo_trace_image (primary, 8x4-pixel tiles, persistent) + svo_trace (shadow)",
                       "octree_words": info["words"], "voxels": info["voxels"], "primary_rays": Rp,
                       "shadow_rays": Rs, "rays_per_step": rays_per_step,
                       "l2": "no flush: octree %.2f GB and rays %.2f GB exceed L2" % (info["words"] * 4 / 1e9,
                                                                                      rays_per_step * 24 / 1e9),
                       "parallelism": "replicas x%d" % world},
            "e2e": e2e, "gpu_launches": 2 * args.steps, "roofline": roofline, "cpu_baseline": cpu,
            "oracle_parity": oracle_parity,
            "clocks": clk.summary(),
            "plain": {"api": "svo_trace for primary (row order) and shadow rays",
                      "ms_per_step": round(ms_plain, 3), "mrays_s": round(rays_per_step / ms_plain / 1e3, 1),
                      "exact_vs_value_path": bool(exact_plain)},
            "alt_outputs": alt_outputs,
            "batched": {"api": "svo_batch: 32 image views + shadow view, autotuned, CUDA graph",
                        "ms_per_step": round(ms_batched, 3), "mrays_s": round(rays_per_step / ms_batched / 1e3, 1),
                        "config": cfg.as_dict(), "exact_vs_value_path": bool(exact_batched)},
            "batched_vs_plain": extra,
            "fwd_bwd": extra4,
            "mesh_build": extra2,
            "viewer_frames": frames,
            "voxel_file_build": extra_vf,
            "build": {"build_s": round(info["build_s"], 3), "scene_gen_s": round(info["gen_s"], 3),
                      "voxels_per_s": round(info["voxels"] / info["build_s"], 1),
                      "build_warm_s": round(info["build_warm_s"], 4),
                      "warm_voxels_per_s": round(info["voxels"] / info["build_warm_s"], 1),
                      "warm_words_equal": info["warm_same"],
                      "build_note": "build_s is the process's first build (first-touch device allocations); "
                                    "build_warm_s the same build again, scratch from the library's pool",
                      "descriptor_table_s": round(info["table_s"], 4),
                      "descriptor_table_entries": info["table_entries"],
                      "descriptor_table_bytes": info["table_entries"] * 16},
            "kernel_ms": {"primary": round(t_prim_avg, 3), "shadow": round(sum(t_shadow) / len(t_shadow), 3)},
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def batched_views(n_views, seed=3):
    """96 (octree, view) pairs: depth U{7..11}, even index -> sphere-union
    generator (48 spheres), odd -> terrain generator (200 spheres), scene seed
    = index; one orbit camera each, pixel count log-uniform in
    [256x256, 1920x1080] at 16:9 clipped to [256, 1920] x [256, 1080]."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(1, n_views + 1):
        depth = int(rng.integers(7, 12))
        pix = float(np.exp(rng.uniform(np.log(256 * 256), np.log(1920 * 1080))))
        W = int(min(1920, max(256, round((pix * 16 / 9) ** 0.5))))
        H = int(min(1080, max(256, round(pix / W))))
        specs.append((i, 1 << depth, "sphere" if i % 2 == 0 else "terrain", W, H))
    return specs


def run_batched(args, torch, svo, scenes, tune_cache=None):
    """Batched persistent launch (graph-captured, autotuned) against the plain
    per-view kernel over the 96 views of batched_views; checks exact parity."""
    t0 = time.perf_counter()
    views, plain_out, rays_list = [], [], []
    trees = []
    total_rays = 0
    for (i, side, gen, W, H) in batched_views(args.views):
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
        out_b, out_p = mk(), mk()
        views.append({"octree": tree, "rays": rays, "width": W, "height": H, "light": light, "out": out_b})
        plain_out.append((tree, rays, light, out_p))
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
        for tree, rays, light, out in plain_out:
            tree.trace(rays, out=out, light=light, stream=stream)

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
    ms_batched = timed(batched_step)
    same = lambda: all(torch.equal(v["out"][k], po[3][k]) for v, po in zip(views, plain_out)
                       for k in ("t", "leaf", "rgb"))
    exact = same()
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
    depth_hi = min(11, args.max_side.bit_length() - 1) if args.max_side else 11
    return {"workload": "%d octrees (depth 7-%d, sphere/terrain generators, seeds 1..%d), one view each, "
                        "256x256..1920x1080 log-uniform pixels" % (len(views), depth_hi, len(views)),
            "rays_per_step": total_rays, "octree_words": int(sum(t.num_words() for t in trees)),
            "plain_ms": round(ms_plain, 3), "batched_ms": round(ms_batched, 3),
            "plain_mrays_s": round(total_rays / ms_plain / 1e3, 1),
            "batched_mrays_s": round(total_rays / ms_batched / 1e3, 1),
            "speedup": round(ms_plain / ms_batched, 3), "exact_hit_parity": bool(exact),
            "table_cache_sweep": {"shape": {k: v for k, v in base.items() if k not in ("cache_entries", "reg_cap")},
                                  "ms_by_cache_entries": cache_sweep},
            "register_budget_sweep": {"shape": {k: v for k, v in rbase.items() if k != "reg_cap"},
                                      "ms_by_reg_cap": reg_sweep},
            "config": cfg.as_dict(), "autotune_s": round(tune_s, 1), "setup_s": round(setup_s, 1),
            "launches": {"plain": len(views), "batched": 1}}


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
    (profiles/mesh_build_config2.md)."""
    try:
        for line in open(os.path.join(ROOT, "profiles", "mesh_build_config2.md")):
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
    p_rgb = torch.rand((nw, 3), generator=gen, device="cuda").requires_grad_()
    p_n = torch.rand((nw, 3), generator=gen, device="cuda").requires_grad_()
    opt = svo.LeafAdam([p_rgb, p_n], lr=1e-2)  # svo_adam_step: one pass per tensor, zeroes the gradient
    rgb = torch.empty((R, 3), dtype=torch.float32, device="cuda")
    leaf = torch.empty(R, dtype=torch.int32, device="cuda")
    d_rgb = torch.empty((R, 3), dtype=torch.float32, device="cuda")
    g_rgb = torch.zeros_like(p_rgb)
    g_n = torch.zeros_like(p_n)
    scale = 2.0 / (3 * R)
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(n_steps)]
    losses = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for k in range(n_steps):
        ev[k][0].record(stream)
        tree.diff_forward(rays, W, H, V, lights, p_rgb.detach(), p_n.detach(), rgb, hit_leaf=leaf, stream=stream)
        ev[k][1].record(stream)
        torch.sub(rgb, target, out=d_rgb)
        if k % 20 == 0 or k == n_steps - 1:
            losses.append((k, d_rgb.square().sum() / (3 * R)))
        d_rgb.mul_(scale)
        ev[k][2].record(stream)
        tree.diff_backward(rays, W, H, V, lights, p_rgb.detach(), p_n.detach(), d_rgb, g_rgb, g_n, hit_leaf=leaf,
                           stream=stream)
        ev[k][3].record(stream)
        p_rgb.grad = g_rgb
        p_n.grad = g_n
        opt.step(stream)  # also zeroes g_rgb and g_n for the next adjoint
    e1.record(stream)
    torch.cuda.synchronize()
    fwd = [e[0].elapsed_time(e[1]) for e in ev]
    bwd = [e[2].elapsed_time(e[3]) for e in ev]  # the adjoint kernel
    step_ms = e0.elapsed_time(e1) / n_steps
    fb = (sum(fwd) + sum(bwd)) / n_steps
    return {"workload": "512^3 sphere union (160 spheres, seed 7), %d octree words; 24 views 512x512; per-leaf FP32 "
                        "rgb+normal params; L2 loss vs 3-octave noise colour field; Adam lr 1e-2" % nw,
            "rays_per_step": R, "steps": n_steps, "fwd_ms": round(sum(fwd) / n_steps, 3),
            "bwd_ms": round(sum(bwd) / n_steps, 3), "fwd_bwd_mrays_s": round(R / fb / 1e3, 1),
            "fwd_bwd_note": "svo_diff_forward + svo_diff_backward kernel time (CUDA events); step_ms_with_adam adds "
                            "the loss gradient and svo_adam_step (one pass per parameter tensor, gradient zeroed "
                            "in the same pass)",
            "step_ms_with_adam": round(step_ms, 3),
            "loss": [[k, round(float(v.item()), 6)] for k, v in losses], "setup_s": round(setup_s, 1)}


def profiled_traffic(rays):
    """DRAM bytes per launch from the committed ncu summaries (per ray, times
    the launch's rays): the full-size one-pass capture, else the small case."""
    for name in ("dram_config1_fullsize.txt", "trace_image_config1.txt"):
        try:
            for line in open(os.path.join(ROOT, "profiles", name)):
                if line.startswith("dram_bytes_per_ray:"):
                    return int(float(line.split(":")[1]) * rays)
        except OSError:
            pass
    return None


def profiled_issue():
    """Issue utilisation of the primary-ray kernel from the committed ncu
    summary: the bound this kernel actually meets (it is issue-bound on the
    ALU pipe, with DRAM at about 5% of peak)."""
    path = os.path.join(ROOT, "profiles", "trace_image_config1.txt")
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
    out["source"] = "profiles/trace_image_config1.txt (ncu --set full, same kernel, smaller case)"
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
    per_step = 4  # cameras per timed step (a bounded sample of the 32-camera step)

    def step(k):
        n = 0
        for j in range(per_step):
            i = (k * per_step + j) % len(prims)
            oracle.raymarch(words, prims[i], light=LIGHT, threads=threads)
            oracle.raymarch(words, shadows[i], threads=threads)
            n += prims[i].shape[0] + shadows[i].shape[0]
        return n

    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    rays = 0
    for k in range(args.steps):
        rays += step(args.warmup + k)
    secs = time.perf_counter() - t0
    value = rays / secs / 1e6
    rays_full = sum(p.shape[0] for p in prims) + sum(s.shape[0] for s in shadows)
    sample = ("%d cameras (primary + shadow rays) per step of the %d-camera workload; %d rays in %.1f s on %d host "
              "threads; oracle C restatement of VoxelOctree::raymarch (the reference's own build needs its sources, "
              "absent on the GPU host)" % (per_step, len(prims), rays, secs, threads))
    line = {
        "impl": "reference", "metric": "Mrays/s", "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded terrain + spheres, seeded orbit cameras)",
        "config": {"workload": "plain traversal: %d^3 octree (terrain + %d spheres), %d cams %dx%d primary rays "
                               "+ 1 shadow ray per hit" % (side, N_SPHERES, args.cams, args.width, args.height),
                   "octree_words": int(words.size), "voxels": int(n_vox), "rays_per_full_step": int(rays_full),
                   "setup_s": round(setup_s, 1)},
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
