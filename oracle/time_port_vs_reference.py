"""Speed of the oracle's raymarch (the C restatement that the benchmark's CPU
baseline times) against the reference's own VoxelOctree::raymarch
(VoxelOctree.cpp:207-346, compiled in place into _ref/libsvo_ref.so), on the
same octree words, the same rays and the same thread count.

TEST INFRASTRUCTURE ONLY.  Needs the reference's sources, so it runs where
they are (SVO_REFERENCE_DIR); it prints one JSON line per workload:

  python oracle/time_port_vs_reference.py [--threads N] [--repeats K]

Workloads: the 256^3 sphere union with 12 views at 1024x768, and the 2048^3
terrain (4 of its 32 orbit cameras at 1920x1080, primary rays).  Results
are also compared ray for ray (hit, t bits, word).
"""
import argparse
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
import pyoracle  # noqa: E402


def _scenes():
    spec = importlib.util.spec_from_file_location("svo_scenes_cpu",
                                                  os.path.join(ROOT, "sparse-voxel-octrees_gb300", "scenes.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _best(fn, repeats):
    best = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        fn()
        s = time.perf_counter() - t0
        best = s if best is None else min(best, s)
    return best


def compare(oracle, ref, words, rays, threads, repeats, label):
    tree = ref.tree_from_words(words, np.full(3, 0.5, np.float32))
    R = rays.shape[0]
    outs = ("hit", "t", "word")  # what the reference's raymarch returns
    o = oracle.raymarch(words, rays, threads=threads, outputs=outs)
    h, t, w = ref.raymarch(tree, rays, threads=threads)
    hit = h == 1
    # t is compared where the ray hits (the two report a miss's t differently)
    same = bool(np.array_equal(o["hit"], h) and np.array_equal(o["t"][hit].view(np.uint32), t[hit].view(np.uint32))
                and np.array_equal(o["word"], w))
    s_port = _best(lambda: oracle.raymarch(words, rays, threads=threads, outputs=outs), repeats)
    s_ref = _best(lambda: ref.raymarch(tree, rays, threads=threads), repeats)
    ref.free(tree)
    return {"workload": label, "rays": R, "threads": threads, "port_mrays_s": round(R / s_port / 1e6, 2),
            "reference_mrays_s": round(R / s_ref / 1e6, 2), "port_over_reference": round(s_ref / s_port, 3),
            "identical_results": same}


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    p.add_argument("--repeats", type=int, default=3)
    p.add_argument("--skip-large", action="store_true")
    a = p.parse_args()
    pyoracle.build_oracle(with_reference=True)
    oracle = pyoracle.Oracle()
    ref = pyoracle.Reference()
    sc = _scenes()

    grid = sc.sphere_scene(256, 48, 0)
    words, center = oracle.build_dense(grid)
    cams = sc.orbit_cameras(12, 0, center, radius=2.0)
    rays = np.concatenate([sc.camera_rays(c, 1024, 768) for c in cams])
    print(json.dumps(compare(oracle, ref, words, rays, a.threads, a.repeats,
                             "256^3 sphere union, 12 views 1024x768")), flush=True)
    if a.skip_large:
        return
    side = 2048
    heights, centers, radii = sc.terrain_scene_params(side, 200, 1)
    keys, pay = oracle.scene_voxels(side, heights, sc.sphere_boxes((side,) * 3, centers, radii),
                                    np.concatenate([centers, radii[:, None]], 1), threads=a.threads)
    words = oracle.build_sorted(keys, pay, 11)
    del keys, pay
    cams = sc.orbit_cameras(32, 1000, np.full(3, 0.5, np.float32), radius=1.25, radius_hi=2.0, pitch=45.0)[:4]
    rays = np.concatenate([sc.camera_rays(c, 1920, 1080) for c in cams])
    print(json.dumps(compare(oracle, ref, words, rays, a.threads, a.repeats,
                             "2048^3 terrain + 200 spheres, 4 of the 32 cameras at 1920x1080 (primary rays)")),
          flush=True)


if __name__ == "__main__":
    main()
