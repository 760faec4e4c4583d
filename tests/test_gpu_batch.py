"""Batched persistent traversal (svo_batch_*): one launch over many octrees
and views of uneven sizes, bit-identical per view to the oracle's
VoxelOctree::raymarch + shade(), under every launch shape, in a captured CUDA
graph and with the autotuned configuration."""
import numpy as np
import pytest

from test_gpu_trace import pack_rgba8

pytestmark = pytest.mark.gpu


def _outputs(torch, n):
    return {"hit": torch.empty(n, dtype=torch.uint8, device="cuda"),
            "t": torch.empty(n, dtype=torch.float32, device="cuda"),
            "leaf": torch.empty(n, dtype=torch.int32, device="cuda"),
            "word": torch.empty(n, dtype=torch.int32, device="cuda"),
            "rgb": torch.empty((n, 3), dtype=torch.float32, device="cuda"),
            "rgba8": torch.empty(n, dtype=torch.int32, device="cuda")}


def _host(out):
    r = {k: v.cpu().numpy() for k, v in out.items()}
    for k in ("leaf", "word", "rgba8"):
        r[k] = r[k].view(np.uint32)
    return r


def _same(res, ref, grey=True):
    assert np.array_equal(res["hit"], ref["hit"])
    assert np.array_equal(res["t"].view(np.uint32), ref["t"].view(np.uint32))
    assert np.array_equal(res["leaf"], ref["leaf"])
    assert np.array_equal(res["word"], ref["word"])
    if grey:
        assert np.array_equal(res["rgb"][:, 0].view(np.uint32), ref["grey"].view(np.uint32))
        assert np.array_equal(res["rgba8"], pack_rgba8(ref["grey"], ref["hit"]))


@pytest.fixture(scope="module")
def scene(cuda, svo, oracle, scenes, golden):
    torch = cuda
    g = golden["dragon"]
    trees = []
    dragon = svo.VoxelOctree.from_words(g["words"], g["center"])
    trees.append((dragon, g["words"], g["center"]))
    for side, seed in ((64, 1), (128, 2)):
        grid = scenes.sphere_scene(side, 16, seed)
        w, c = oracle.build_dense(grid)
        trees.append((svo.VoxelOctree.from_words(w, c), w, c))
    far = scenes.random_grid((64, 64, 64), 0.5, 3)
    w, c = oracle.build_dense(far)
    trees.append((svo.VoxelOctree.from_words(w, c), w, c))
    views, refs = [], []
    rng = np.random.default_rng(0)
    sizes = [(64, 48), (37, 23), (128, 96), (1, 1), (200, 7)]
    k = 0
    for ti, (tree, words, center) in enumerate(trees):
        for vi in range(3):
            W, H = sizes[k % len(sizes)]
            k += 1
            cam = scenes.orbit_cameras(1, 100 * ti + vi, center, radius=1.5)[0]
            rays = scenes.camera_rays(cam, W, H)
            light = scenes.headlight(cam)
            kind = (ti + vi) % 3
            out = _outputs(torch, W * H)
            if kind == 0:    # camera rays generated in the kernel
                v = {"octree": tree, "camera": scenes.camera_constants(cam, W, H), "width": W, "height": H,
                     "light": light, "out": out}
            elif kind == 1:  # row-major image rays from memory
                v = {"octree": tree, "rays": torch.from_numpy(rays).cuda(), "width": W, "height": H,
                     "light": light, "out": out}
            else:            # linear rays, some with a level-of-detail scale
                rays = scenes.random_rays(int(rng.integers(1, 5000)), 10 * ti + vi)
                out = _outputs(torch, rays.shape[0])
                v = {"octree": tree, "rays": torch.from_numpy(rays).cuda(), "light": light, "out": out,
                     "ray_scale": 0.01 if vi == 2 else 0.0}
            views.append(v)
            refs.append(oracle.raymarch(words, rays, ray_scale=v.get("ray_scale", 0.0), light=light, threads=4))
    return views, refs


def _check(torch, views, refs):
    torch.cuda.synchronize()
    for v, ref in zip(views, refs):
        _same(_host(v["out"]), ref, grey=v.get("ray_scale", 0.0) == 0.0)


def _clear(torch, views):
    for v in views:
        for t in v["out"].values():
            t.fill_(0x5A if t.dtype == torch.uint8 else 7)


def test_batch_default(cuda, svo, scene):
    torch = cuda
    views, refs = scene
    b = svo.Batch(views)
    _clear(torch, views)
    b.trace()
    _check(torch, views, refs)
    assert b.status() == 0


@pytest.mark.parametrize("cfg", [dict(refill_idle=0), dict(refill_idle=0, chunk=96, tile_w=4),
                                 dict(tile_w=4), dict(tile_w=16), dict(tile_w=32), dict(refill_idle=1),
                                 dict(refill_idle=32, steps_per_round=1), dict(block_threads=128, chunk=32),
                                 dict(steps_per_round=64, chunk=256),
                                 # per-warp table caches: above and below the trees' table sizes, 16 to 64 KB
                                 # of shared memory per CTA (above 48 KB needs the opt-in)
                                 dict(refill_idle=0, cache_entries=64),
                                 dict(refill_idle=0, cache_entries=512, block_threads=128, tile_w=4, chunk=128),
                                 dict(refill_idle=0, cache_entries=32, block_threads=1024, chunk=32),
                                 dict(refill_idle=0, cache_entries=256, block_threads=512, tile_w=16),
                                 # the 48-register build of the lane-refill kernel
                                 dict(reg_cap=48), dict(reg_cap=48, refill_idle=1, block_threads=128),
                                 dict(reg_cap=48, refill_idle=32, steps_per_round=64, tile_w=4)])
def test_batch_launch_shapes(cuda, svo, scene, cfg):
    torch = cuda
    views, refs = scene
    b = svo.Batch(views)
    _clear(torch, views)
    b.trace(svo.default_config(**cfg))
    _check(torch, views, refs)


def test_batch_graph_replay(cuda, svo, scene):
    torch = cuda
    views, refs = scene
    b = svo.Batch(views)
    b.capture_graph(svo.default_config(tile_w=16))
    for _ in range(3):
        _clear(torch, views)
        b.launch_graph(torch.cuda.current_stream())
        _check(torch, views, refs)


def test_batch_graph_replay_cached(cuda, svo, scene):
    torch = cuda
    views, refs = scene
    b = svo.Batch(views)
    b.capture_graph(svo.default_config(refill_idle=0, cache_entries=128, tile_w=4))
    for _ in range(2):
        _clear(torch, views)
        b.launch_graph(torch.cuda.current_stream())
        _check(torch, views, refs)


@pytest.mark.parametrize("cfg", [dict(refill_idle=16, cache_entries=64),  # the cache needs the tile schedule
                                 dict(refill_idle=0, cache_entries=48),   # not a multiple of 32
                                 dict(refill_idle=0, cache_entries=544),  # above 512
                                 dict(refill_idle=0, cache_entries=512, block_threads=512),  # 128 KB per CTA
                                 dict(reg_cap=32)])                                          # no such build
def test_batch_rejects_bad_config(cuda, svo, scene, cfg):
    views, _ = scene
    b = svo.Batch(views)
    with pytest.raises(svo.SvoError):
        b.trace(svo.default_config(**cfg))


def test_batch_autotune(cuda, svo, scene, tmp_path, monkeypatch):
    torch = cuda
    monkeypatch.setenv("SVO_AUTOTUNE_CACHE", str(tmp_path / "tune.jsonl"))
    views, refs = scene
    b = svo.Batch(views)
    cfg, ms = b.autotune()
    assert ms > 0 and cfg.block_threads in (128, 256, 512)
    cfg2, ms2 = b.autotune()  # answered from the cache
    assert ms2 == -1.0 and cfg2.as_dict() == cfg.as_dict()
    _clear(torch, views)
    b.trace(cfg)
    _check(torch, views, refs)


def test_batch_matches_plain_kernel(cuda, svo, oracle, scenes, golden):
    torch = cuda
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    rays = scenes.random_rays(300_000, 77, lo=0.0, hi=3.0)
    d_rays = torch.from_numpy(rays).cuda()
    plain = _outputs(torch, rays.shape[0])
    tree.trace(d_rays, out=plain, light=(0.0, 1.0, 0.0))
    batched = _outputs(torch, rays.shape[0])
    b = svo.Batch([{"octree": tree, "rays": d_rays, "out": batched, "light": (0.0, 1.0, 0.0)}])
    b.trace()
    torch.cuda.synchronize()
    p, q = _host(plain), _host(batched)
    for k in p:
        assert np.array_equal(p[k], q[k]), k
