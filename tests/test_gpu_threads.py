"""The viewer traces one octree from 16 host threads at once, each thread
calling VoxelOctree::raymarch for its own pixels (Main.cpp:342-367).  The
host-buffer calls that replace it are made the same way here: 16 threads on
two freshly built octrees (so the first calls race to build the descriptor
table), mixing svo_trace_host, svo_trace_image_host and single-ray
raymarch, and every result is the oracle's, bit for bit."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_THREADS = 16
W, H = 96, 64


def _check(res, ref, what):
    assert np.array_equal(res["hit"], ref["hit"]), what
    assert np.array_equal(res["t"].view(np.uint32), ref["t"].view(np.uint32)), what
    assert np.array_equal(res["word"], ref["word"]), what
    assert np.array_equal(res["rgb"][:, 0].view(np.uint32), ref["grey"].view(np.uint32)), what


def test_host_calls_from_16_threads(svo, oracle, scenes):
    grids = [scenes.sphere_scene(128, 20, 5), scenes.terrain_scene(128, 20, 6)]
    built = [oracle.build_dense(g) for g in grids]
    trees = [svo.VoxelOctree(svo.VoxelData(g)) for g in grids]
    cams = [scenes.orbit_cameras(N_THREADS, 3 + k, built[k][1]) for k in range(2)]
    jobs = []
    for i in range(N_THREADS):
        k = i % 2
        cam = cams[k][i]
        jobs.append((k, scenes.camera_rays(cam, W, H), scenes.headlight(cam)))
    results = [None] * N_THREADS
    singles = [None] * N_THREADS
    errors = []
    start = threading.Barrier(N_THREADS)

    def work(i):
        try:
            k, rays, light = jobs[i]
            start.wait()
            for rep in range(3):
                if (i + rep) % 2:
                    r = trees[k].trace_host(rays, light=light, outputs=("hit", "t", "word", "rgb"))
                else:
                    r = trees[k].trace_image_host(rays, W, H, light=light, outputs=("hit", "t", "word", "rgb"))
                if rep == 0:
                    results[i] = r
                else:
                    for key in r:
                        if not np.array_equal(r[key], results[i][key]):
                            raise AssertionError("thread %d call %d differs in %s" % (i, rep, key))
            # the reference's own call shape: one ray per call
            singles[i] = [trees[k].raymarch(rays[j, :3], rays[j, 3:]) for j in range(0, rays.shape[0], 97)]
        except Exception as e:  # re-raised on the main thread
            errors.append((i, e))

    threads = [threading.Thread(target=work, args=(i,)) for i in range(N_THREADS)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in threads)
    assert not errors, errors
    hits = 0
    for i, (k, rays, light) in enumerate(jobs):
        ref = oracle.raymarch(built[k][0], rays, light=light)
        _check(results[i], ref, "thread %d" % i)
        hits += int((ref["hit"] == 1).sum())
        for n, j in enumerate(range(0, rays.shape[0], 97)):
            hit, word, t = singles[i][n]
            assert hit == (ref["hit"][j] != 0), (i, j)
            if ref["hit"][j] == 1:
                assert word == int(ref["word"][j]) and np.float32(t) == ref["t"][j], (i, j)
    assert hits > N_THREADS * 500
