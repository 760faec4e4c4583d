"""GPU traversal parity: svo_trace / svo_trace_host against the oracle's
restatement of VoxelOctree::raymarch and the viewer's shade() — bit-exact
hit flags, t bits, leaf indices, leaf words and shaded colours."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_trace(cuda, svo, tree, rays, ray_scale=0.0, light=(0.0, 0.0, 1.0)):
    torch = cuda
    R = rays.shape[0]
    d_rays = torch.from_numpy(np.ascontiguousarray(rays)).cuda()
    out = {
        "hit": torch.empty(R, dtype=torch.uint8, device="cuda"),
        "t": torch.empty(R, dtype=torch.float32, device="cuda"),
        "leaf": torch.empty(R, dtype=torch.int32, device="cuda"),
        "word": torch.empty(R, dtype=torch.int32, device="cuda"),
        "rgb": torch.empty((R, 3), dtype=torch.float32, device="cuda"),
        "rgba8": torch.empty(R, dtype=torch.int32, device="cuda"),
    }
    tree.trace(d_rays, ray_scale=ray_scale, light=light, out=out)
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    for k in ("leaf", "word", "rgba8"):
        res[k] = res[k].view(np.uint32)
    assert tree.device_status() == 0
    return res


def pack_rgba8(grey, hit):
    """The viewer's packed colour of a traced pixel (renderTile,
    Main.cpp:126-131): uint32(std::min(shade, 1.0f) * 255.0) with the product
    in double, in the three colour bytes, alpha 0xFF; shade 0 without a leaf."""
    g = np.where(hit == 1, grey, np.float32(0.0)).astype(np.float32)
    g = np.where(np.float32(1.0) < g, np.float32(1.0), g)
    c = (g.astype(np.float64) * 255.0).astype(np.uint32)
    return c | (c << 8) | (c << 16) | np.uint32(0xFF000000)


def _assert_same(res, ref, grey=True):
    assert np.array_equal(res["hit"], ref["hit"])
    assert np.array_equal(res["t"].view(np.uint32), ref["t"].view(np.uint32))
    assert np.array_equal(res["leaf"], ref["leaf"])
    assert np.array_equal(res["word"], ref["word"])
    if grey:
        g = ref["grey"]
        assert np.array_equal(res["rgb"][:, 0].view(np.uint32), g.view(np.uint32))
        assert np.array_equal(res["rgb"][:, 1], res["rgb"][:, 0])
        assert np.array_equal(res["rgb"][:, 2], res["rgb"][:, 0])
        if "rgba8" in res:
            assert np.array_equal(res["rgba8"], pack_rgba8(g, ref["hit"]))


def test_dragon_golden_rays(cuda, svo, golden, oracle):
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    light = np.array([0.3, -0.8, 0.52], np.float32)
    res = _device_trace(cuda, svo, tree, g["rays"], light=light)
    # against the reference's own outputs
    hit = res["hit"] == 1
    assert np.array_equal(hit.astype(np.uint8), g["hit"])
    assert np.array_equal(res["t"][hit].view(np.uint32), g["t"][hit].view(np.uint32))
    assert np.array_equal(res["word"][hit], g["word"][hit])
    # and every output against the oracle
    _assert_same(res, oracle.raymarch(g["words"], g["rays"], light=light, threads=4))


def test_dragon_lod(cuda, svo, golden, oracle):
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    res = _device_trace(cuda, svo, tree, g["rays"], ray_scale=0.02)
    hit = res["hit"] > 0
    assert np.array_equal(hit.astype(np.uint8), g["lod_hit"])
    assert np.array_equal(res["t"][hit].view(np.uint32), g["lod_t"][hit].view(np.uint32))
    _assert_same(res, oracle.raymarch(g["words"], g["rays"], ray_scale=0.02, threads=4), grey=False)


def test_dragon_camera_views(cuda, svo, golden, oracle, scenes):
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    for cam in scenes.orbit_cameras(3, 7, g["center"], radius=1.5):
        rays = scenes.camera_rays(cam, 320, 240)
        light = scenes.headlight(cam)
        res = _device_trace(cuda, svo, tree, rays, light=light)
        ref = oracle.raymarch(g["words"], rays, light=light, threads=4)
        _assert_same(res, ref)
        assert (ref["hit"] == 1).mean() > 0.05


def test_sphere_scene_random_and_edge_rays(cuda, svo, oracle, scenes):
    grid = scenes.sphere_scene(128, 24, 0)
    words, center = oracle.build_dense(grid)
    tree = svo.VoxelOctree.from_words(words, center)
    rays = scenes.random_rays(200_000, 5)
    res = _device_trace(cuda, svo, tree, rays, light=(0.0, 1.0, 0.0))
    _assert_same(res, oracle.raymarch(words, rays, light=(0.0, 1.0, 0.0), threads=4))


def test_far_pointer_tree(cuda, svo, oracle, scenes):
    grid = scenes.random_grid((64, 64, 64), 0.5, 3)
    words, center = oracle.build_dense(grid)
    assert ((words >> 17) & 1).sum() > 0
    tree = svo.VoxelOctree.from_words(words, center)
    rays = scenes.random_rays(100_000, 6)
    _assert_same(_device_trace(cuda, svo, tree, rays), oracle.raymarch(words, rays, threads=4))


def test_trace_host_matches_device(cuda, svo, golden, oracle, scenes):
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    rays = np.concatenate([scenes.random_rays(3_000_000, 8, lo=0.0, hi=3.0), g["rays"]])
    host = tree.trace_host(rays, light=(0.0, 0.0, 1.0))
    ref = oracle.raymarch(g["words"], rays, light=(0.0, 0.0, 1.0), threads=8)
    _assert_same(host, ref)


def test_single_ray_api(svo, golden, oracle):
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    for i in range(0, 64):
        r = g["rays"][i]
        hit, normal, t = tree.raymarch(r[:3], r[3:])
        assert hit == bool(g["hit"][i])
        if hit:
            assert normal == int(g["word"][i]) and np.float32(t) == g["t"][i]


def test_count_loads_matches_oracle(cuda, svo, golden, oracle):
    torch = cuda
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    rays = torch.from_numpy(g["rays"]).cuda()
    loads = torch.zeros(rays.shape[0], dtype=torch.int32, device="cuda")
    tree.count_loads(rays, loads=loads)
    torch.cuda.synchronize()
    ref = oracle.raymarch(g["words"], g["rays"], loads=True, threads=4)
    assert np.array_equal(loads.cpu().numpy().view(np.uint32), ref["loads"])


def test_corrupt_tree_raises_device_flag(cuda, svo):
    # A descriptor whose child offset points past the end: the kernel's bounds
    # check ends the ray and sets the handle's error flag (no fault).
    words = np.array([(0x3FFF << 18) | (0xFF << 8) | 0xFF], np.uint32)
    tree = svo.VoxelOctree.from_words(words, (0.5, 0.5, 0.5))
    rays = np.array([[1.5, 1.5, -1.0, 0.0, 0.0, 1.0]], np.float32)
    with pytest.raises(svo.SvoError) as e:
        tree.trace_host(rays)
    assert e.value.code == svo.SVO_ERR_DEVICE


@pytest.mark.parametrize("W,H", [(320, 240), (37, 23), (1, 1), (1000, 3), (7, 401)])
def test_trace_image_matches_oracle(cuda, svo, golden, oracle, scenes, W, H):
    torch = cuda
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    cam = scenes.orbit_cameras(1, W * 7 + H, g["center"], radius=1.4)[0]
    rays = scenes.camera_rays(cam, W, H)
    light = scenes.headlight(cam)
    R = rays.shape[0]
    out = {"hit": torch.empty(R, dtype=torch.uint8, device="cuda"),
           "t": torch.empty(R, dtype=torch.float32, device="cuda"),
           "leaf": torch.empty(R, dtype=torch.int32, device="cuda"),
           "word": torch.empty(R, dtype=torch.int32, device="cuda"),
           "rgb": torch.empty((R, 3), dtype=torch.float32, device="cuda")}
    for scale in (0.0, 0.01):
        tree.trace_image(torch.from_numpy(rays).cuda(), W, H, ray_scale=scale, light=light, out=out)
        torch.cuda.synchronize()
        res = {k: v.cpu().numpy() for k, v in out.items()}
        res["leaf"] = res["leaf"].view(np.uint32)
        res["word"] = res["word"].view(np.uint32)
        _assert_same(res, oracle.raymarch(g["words"], rays, ray_scale=scale, light=light, threads=4), grey=scale == 0)
    assert tree.device_status() == 0


def test_trace_image_host_matches_oracle(svo, oracle, scenes):
    grid = scenes.sphere_scene(128, 24, 5)
    words, center = oracle.build_dense(grid)
    tree = svo.VoxelOctree.from_words(words, center)
    cams = scenes.orbit_cameras(4, 3, center)
    W, H = 1003, 777  # 2.2 M rays: several staged chunks of whole rows
    rays = np.concatenate([scenes.camera_rays(c, W, H // 4 + 1)[:W * (H // 4)] for c in cams] +
                          [scenes.camera_rays(cams[0], W, H - 4 * (H // 4))])
    host = tree.trace_image_host(rays, W, H, light=(0.0, 1.0, 0.0))
    _assert_same(host, oracle.raymarch(words, rays, light=(0.0, 1.0, 0.0), threads=8))


def test_host_pipelines_long_calls(cuda, svo, oracle, scenes):
    """Host calls of several staged chunks (full 4 M-ray chunks and a
    remainder, alternating between the two trace streams and staging halves)
    give the device-resident entry points' results on the same rays."""
    torch = cuda
    grid = scenes.sphere_scene(128, 24, 5)
    words, center = oracle.build_dense(grid)
    tree = svo.VoxelOctree.from_words(words, center)
    cam = scenes.orbit_cameras(1, 9, center)[0]
    W, H = 1024, 10_611  # 10.9 M rays: image chunks of 4096 rows, linear chunks of 4 M rays
    rays = scenes.camera_rays(cam, W, H)
    light = (0.0, 1.0, 0.0)
    ref = _device_trace(cuda, svo, tree, rays, light=light)
    ref["grey"] = ref["rgb"][:, 0].copy()
    _assert_same(tree.trace_host(rays, light=light, outputs=svo.TRACE_OUTPUTS), ref)
    d_rays = torch.from_numpy(rays).cuda()
    out = {"hit": torch.empty(W * H, dtype=torch.uint8, device="cuda"),
           "t": torch.empty(W * H, dtype=torch.float32, device="cuda"),
           "leaf": torch.empty(W * H, dtype=torch.int32, device="cuda"),
           "word": torch.empty(W * H, dtype=torch.int32, device="cuda"),
           "rgb": torch.empty((W * H, 3), dtype=torch.float32, device="cuda"),
           "rgba8": torch.empty(W * H, dtype=torch.int32, device="cuda")}
    tree.trace_image(d_rays, W, H, light=light, out=out)
    torch.cuda.synchronize()
    img = {k: v.cpu().numpy() for k, v in out.items()}
    for k in ("leaf", "word", "rgba8"):
        img[k] = img[k].view(np.uint32)
    _assert_same(img, ref)
    _assert_same(tree.trace_image_host(rays, W, H, light=light, outputs=svo.TRACE_OUTPUTS), ref)
    assert tree.device_status() == 0


def test_host_async_calls_match_sync_calls(cuda, svo, oracle, scenes):
    """svo_trace_host_async / svo_trace_image_host_async queue on the host
    pipeline and give, after svo_octree_synchronize, what the waiting calls
    give: several calls in a row (their chunks share the staging buffers),
    a small call followed by one that needs a larger staging arena (the
    queued work is drained before it is replaced), and a pending call at
    close."""
    grid = scenes.sphere_scene(128, 24, 5)
    words, center = oracle.build_dense(grid)
    tree = svo.VoxelOctree.from_words(words, center)
    cams = scenes.orbit_cameras(2, 13, center)
    W, H = 1024, 4500  # 4.6 M rays: two image chunks, two linear chunks
    img_rays = scenes.camera_rays(cams[0], W, H)
    lin_rays = scenes.random_rays(300_000, 23)
    small = scenes.camera_rays(cams[1], 40, 30)
    light = (0.0, 1.0, 0.0)
    outs = svo.TRACE_OUTPUTS
    ref_img = tree.trace_image_host(img_rays, W, H, light=light, outputs=outs)
    ref_lin = tree.trace_host(lin_rays, light=light, outputs=outs)
    ref_small = tree.trace_host(small, light=light, outputs=outs)
    tree.close()
    tree = svo.VoxelOctree.from_words(words, center)  # fresh staging: the small call comes first
    a = tree.trace_host(small, light=light, outputs=outs, wait=False)
    b = tree.trace_image_host(img_rays, W, H, light=light, outputs=outs, wait=False)
    c = tree.trace_host(lin_rays, light=light, outputs=outs, wait=False)
    d = tree.trace_image_host(img_rays, W, H, light=light, outputs=outs, wait=False)
    tree.synchronize()
    for got, ref in ((a, ref_small), (b, ref_img), (c, ref_lin), (d, ref_img)):
        for k in outs:
            assert np.array_equal(np.asarray(got[k]).view(np.uint8), np.asarray(ref[k]).view(np.uint8)), k
    tree.synchronize()  # nothing queued: returns at once
    tree.trace_host(lin_rays, light=light, outputs=outs, wait=False)
    tree.close()  # waits for the queued call before freeing the handle


def test_sphere_union_256_views_match_oracle(cuda, svo, oracle, scenes):
    """The small plain-traversal workload in full: the 256^3 union of 48
    spheres (seed 0), built on the GPU, and 12 orbit views (radius 2, seeded
    yaw and pitch) at 1024x768 with headlights, traced by the image entry
    point; every output of all 9.4 M rays bit-exact against the oracle."""
    torch = cuda
    grid = scenes.sphere_scene(256, 48, 0)
    words, center = oracle.build_dense(grid)
    tree = svo.VoxelOctree(svo.VoxelData(grid))
    assert np.array_equal(tree.words(), words)
    W, H = 1024, 768
    hits = 0
    for cam in scenes.orbit_cameras(12, 0, center, radius=2.0):
        d_rays = scenes.gpu_camera_rays(cam, W, H)
        light = scenes.headlight(cam)
        out = {k: torch.empty(W * H, dtype=dt, device="cuda")
               for k, dt in (("hit", torch.uint8), ("t", torch.float32), ("leaf", torch.int32),
                             ("word", torch.int32), ("rgba8", torch.int32))}
        out["rgb"] = torch.empty((W * H, 3), dtype=torch.float32, device="cuda")
        tree.trace_image(d_rays, W, H, light=light, out=out)
        torch.cuda.synchronize()
        res = {k: v.cpu().numpy() for k, v in out.items()}
        for k in ("leaf", "word", "rgba8"):
            res[k] = res[k].view(np.uint32)
        ref = oracle.raymarch(words, d_rays.cpu().numpy(), light=light, threads=os.cpu_count() or 4)
        _assert_same(res, ref)
        hits += int((ref["hit"] == 1).sum())
    assert hits > 1_000_000
    assert tree.device_status() == 0


def test_nan_and_infinite_rays(cuda, svo, golden, oracle):
    """Rays with NaN corner distances (NaN components, or an infinite origin
    along an infinite direction) end as misses after one pass, in every
    entry point; rays with other infinite components traverse as usual."""
    torch = cuda
    nan, inf = np.float32(np.nan), np.float32(np.inf)
    odd = np.array([[nan, nan, nan, 0.0, 0.0, 1.0], [1.5, 1.5, -1.0, nan, nan, nan],
                    [1.5, 1.5, -1.0, nan, 0.0, 1.0], [1.5, nan, -1.0, 0.0, 0.0, 1.0],
                    [inf, 1.5, 1.5, -inf, 0.0, 0.0], [inf, 1.5, 1.5, -1.0, 0.0, 0.0],
                    [1.5, 1.5, -1.0, 0.0, 0.0, inf]], np.float32)
    g = golden["dragon"]
    rays = np.concatenate([odd, g["rays"][:4000], odd])
    R = rays.shape[0]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    ref = oracle.raymarch(g["words"], rays, loads=True, threads=4)
    assert (ref["hit"][:5] == 0).all()
    _assert_same(_device_trace(cuda, svo, tree, rays), ref)
    _assert_same(tree.trace_host(rays), ref)
    # image form (one row) and the batched persistent kernels
    d_rays = torch.from_numpy(rays).cuda()
    out = {"hit": torch.empty(R, dtype=torch.uint8, device="cuda"),
           "t": torch.empty(R, dtype=torch.float32, device="cuda"),
           "leaf": torch.empty(R, dtype=torch.int32, device="cuda"),
           "word": torch.empty(R, dtype=torch.int32, device="cuda"),
           "rgb": torch.empty((R, 3), dtype=torch.float32, device="cuda")}
    tree.trace_image(d_rays, R, 1, out=out)
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    res["leaf"] = res["leaf"].view(np.uint32)
    res["word"] = res["word"].view(np.uint32)
    _assert_same(res, ref)
    for cfg in (dict(refill_idle=0), dict(refill_idle=1)):
        for v in out.values():
            v.fill_(7)
        b = svo.Batch([{"octree": tree, "rays": d_rays, "out": out}])
        b.trace(svo.default_config(**cfg))
        torch.cuda.synchronize()
        res = {k: v.cpu().numpy() for k, v in out.items()}
        res["leaf"] = res["leaf"].view(np.uint32)
        res["word"] = res["word"].view(np.uint32)
        _assert_same(res, ref)
        assert b.status() == 0
        b.close()
    loads = torch.zeros(R, dtype=torch.int32, device="cuda")
    tree.count_loads(d_rays, loads=loads)
    torch.cuda.synchronize()
    assert np.array_equal(loads.cpu().numpy().view(np.uint32), ref["loads"])
    # a frame from a NaN camera position: every corner and pixel ray is NaN
    frame = tree.render_frame(np.eye(3, dtype=np.float32).ravel(), (nan, 1.5, -1.0), 64, 48, 4)
    torch.cuda.synchronize()
    assert not frame.any()
    assert tree.device_status() == 0


def test_table_and_word_traversal_agree(cuda, svo, golden, oracle, scenes):
    """The descriptor-table traversal (the default) and the word traversal
    give identical outputs; the table has one entry per reachable node."""
    g = golden["dragon"]
    trees = [(g["words"], g["center"])]
    trees.append(oracle.build_dense(scenes.random_grid((64, 64, 64), 0.5, 3)))
    trees.append(oracle.build_dense(scenes.sphere_scene(256, 40, 2)))
    rays = np.concatenate([scenes.random_rays(300_000, 17), g["rays"]])
    for words, center in trees:
        tree = svo.VoxelOctree.from_words(words, center)
        nd, _ = tree.validate()
        assert tree.table_size() == nd
        ref = oracle.raymarch(words, rays, threads=8)
        tab = _device_trace(cuda, svo, tree, rays)
        tree.set_table(False)
        plain = _device_trace(cuda, svo, tree, rays)
        _assert_same(tab, ref)
        _assert_same(plain, ref)
        tree.close()


def test_table_refused_for_corrupt_trees(cuda, svo):
    for words in ([(0x3FFF << 18) | (0xFF << 8) | 0xFF], [(0xFF << 8) | 0xFF] + [0] * 8,
                  [(1 << 18) | (0x01 << 8) | 0x02, 0]):
        tree = svo.VoxelOctree.from_words(np.array(words, np.uint32), (0.5, 0.5, 0.5))
        assert tree.table_size() == 0
        tree.close()
