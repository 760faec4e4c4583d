"""Octree words and traced results at the benchmark workloads' full sizes,
against the oracle.

- The plain-traversal octree: 2048^3 terrain + 200 spheres, 488 M words.
- The batched workload's octrees (depth 7-11, scenes.batched_views): every
  octree of depth <= 10 (79 of the 96) and three of depth 11.
- The differentiable-shading octree (512^3, 160 spheres, seed 7):
  - its words against the faithful VoxelData build;
  - the hit leaves of all 24 x 512^2 rays against the oracle's raymarch;
  - the adjoint's gradients against plain FP64 central differences
    (h = 1e-3) on 256 random hit leaves, to 1e-4 relative, and against the
    Richardson-extrapolated differences.

Octree words must be bit-exact.  The large oracle builds use
oracle/scene_build.c: its CPU scene generator and its sorted-voxel build,
which tests/test_cpu_scene_build.py holds to the faithful restatement of
VoxelOctree(VoxelData*) (VoxelOctree.cpp:125-205, ChunkedAllocator.hpp:76-114).
The traversal being differentiated is VoxelOctree::raymarch
(VoxelOctree.cpp:207-346); the shading is the viewer's shade (Main.cpp:81-90).
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

import diff_oracle

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4
CORES = os.cpu_count() or 4


def _oracle_scene_words(oracle, scenes, side, heights, centers, radii, threads):
    boxes = scenes.sphere_boxes((side,) * 3, centers, radii)
    params = np.concatenate([centers, radii[:, None]], 1)
    keys, pay = oracle.scene_voxels(side, heights, boxes, params, threads=threads)
    words = oracle.build_sorted(keys, pay, side.bit_length() - 1)
    return words, keys.size


def _gpu_words(svo, scenes, side, heights, centers, radii, mem=1 << 30):
    grid = scenes.gpu_payload_grid(scenes.gpu_occupancy(side, heights, centers, radii), side)
    tree = svo.VoxelOctree(svo.VoxelData(grid, mem))
    del grid
    words, center = tree.words(), tree.center()
    tree.close()
    return words, center


def test_plain_traversal_octree_words(cuda, svo, oracle, scenes):
    """The 2048^3 terrain octree of the plain-traversal workload, built with
    its 8 GiB budget."""
    side = 2048
    heights, centers, radii = scenes.terrain_scene_params(side, 200, 1)
    gw, gc = _gpu_words(svo, scenes, side, heights, centers, radii, mem=8 << 30)
    cuda.cuda.empty_cache()
    ow, n_vox = _oracle_scene_words(oracle, scenes, side, heights, centers, radii, CORES)
    assert n_vox > 400_000_000
    assert gw.size == ow.size == 488_339_379
    assert np.array_equal(gw, ow)
    assert np.array_equal(gc, np.full(3, 0.5, np.float32))


def test_batched_workload_octree_words(cuda, svo, oracle, scenes):
    """Every octree of depth <= 10 of the batched workload, plus its first
    depth-11 terrain and first two depth-11 sphere unions."""
    specs = scenes.batched_views(96)
    small = [s for s in specs if s[1] <= 1024]
    big = [s for s in specs if s[1] == 2048]
    big = [s for s in big if s[2] == "terrain"][:1] + [s for s in big if s[2] == "sphere"][:2]
    assert len(small) == 79 and len(big) == 3
    workers = 4

    def oracle_job(spec):
        i, side, gen, _, _ = spec
        h, c, r = scenes.scene_spec_params(side, gen, i)
        return _oracle_scene_words(oracle, scenes, side, h, c, r, max(1, CORES // workers))[0]

    checked = 0
    # the oracle's builds run on host threads (ctypes releases the GIL) while
    # the GPU builds the same octrees in order
    with cf.ThreadPoolExecutor(workers) as ex:
        futures = [ex.submit(oracle_job, s) for s in small]
        for spec, fut in zip(small, futures):
            i, side, gen, _, _ = spec
            gw, gc = _gpu_words(svo, scenes, side, *scenes.scene_spec_params(side, gen, i))
            ow = fut.result()
            assert np.array_equal(gw, ow), spec
            assert np.array_equal(gc, np.full(3, 0.5, np.float32))
            checked += 1
    for spec in big:
        i, side, gen, _, _ = spec
        gw, gc = _gpu_words(svo, scenes, side, *scenes.scene_spec_params(side, gen, i))
        cuda.cuda.empty_cache()
        ow, _ = _oracle_scene_words(oracle, scenes, side, *scenes.scene_spec_params(side, gen, i), CORES)
        assert np.array_equal(gw, ow), spec
        checked += 1
        del gw, ow
    assert checked == 82


# ------------------------------------------------ differentiable shading, 512^3


@pytest.fixture(scope="module")
def shading(cuda, svo, oracle, scenes):
    """The differentiable-shading workload: 512^3 union of 160 spheres
    (seed 7), 24 orbit views at 512x512, per-word FP32 rgb and normal
    parameters ~U[0,1], random targets; the oracle's raymarch gives the
    reference's hit leaf for every ray."""
    torch = cuda
    side, W, H, V = 512, 512, 512, 24
    grid = scenes.gpu_sphere_scene(side, 160, 7)
    tree = svo.VoxelOctree(svo.VoxelData(grid))
    host_grid = grid.cpu().numpy().view(np.uint32)
    del grid
    words, center = tree.words(), tree.center()
    ref_words, ref_center = oracle.build_dense(host_grid)
    del host_grid
    cams = scenes.orbit_cameras(V, 7, center, radius=2.0)
    rays = torch.empty((V * W * H, 6), dtype=torch.float32, device="cuda")
    for i, c in enumerate(cams):
        scenes.gpu_camera_rays(c, W, H, out=rays[i * W * H:(i + 1) * W * H])
    h_rays = rays.cpu().numpy()
    lights = np.stack([scenes.headlight(c) for c in cams]).astype(np.float32)
    ref = oracle.raymarch(ref_words, h_rays, threads=CORES)
    leaf = np.where(ref["hit"] == 1, ref["leaf"], np.uint32(0xFFFFFFFF)).astype(np.uint32)
    rng = np.random.default_rng(3)
    nw = words.size
    p_rgb = rng.random((nw, 3), dtype=np.float32)
    p_n = rng.random((nw, 3), dtype=np.float32)
    target = rng.random((h_rays.shape[0], 3)).astype(np.float32)
    return dict(tree=tree, words=words, center=center, ref_words=ref_words, ref_center=ref_center, W=W, H=H, V=V,
                rays=rays, h_rays=h_rays, lights=lights, ray_light=np.repeat(lights, W * H, axis=0), leaf=leaf,
                p_rgb=p_rgb, p_n=p_n, target=target, w=1.0 / (3 * h_rays.shape[0]))


def _forward_backward(torch, pb):
    """GPU forward (recording hit leaves) and adjoint of
    L = sum w (rgb - target)^2: (rgb, hit leaf, dL/drgb params, dL/dnormal params)."""
    R = pb["h_rays"].shape[0]
    lights = torch.from_numpy(pb["lights"]).cuda()
    p_rgb = torch.from_numpy(pb["p_rgb"]).cuda()
    p_n = torch.from_numpy(pb["p_n"]).cuda()
    rgb = torch.empty((R, 3), dtype=torch.float32, device="cuda")
    hit = torch.empty(R, dtype=torch.int32, device="cuda")
    args = (pb["rays"], pb["W"], pb["H"], pb["V"], lights, p_rgb, p_n)
    pb["tree"].diff_forward(*args, rgb, hit_leaf=hit)
    d_rgb = (rgb - torch.from_numpy(pb["target"]).cuda()) * (2.0 * pb["w"])
    g_rgb, g_n = torch.zeros_like(p_rgb), torch.zeros_like(p_n)
    pb["tree"].diff_backward(*args, d_rgb, g_rgb, g_n, hit_leaf=hit)
    torch.cuda.synchronize()
    return rgb.cpu().numpy(), hit.cpu().numpy().view(np.uint32), g_rgb.cpu().numpy(), g_n.cpu().numpy()


def _leaf_rel_err(g, ref):
    """Per-leaf relative error of a 3-vector gradient, ||g - ref|| / ||ref||."""
    return np.linalg.norm(g - ref, axis=-1) / np.linalg.norm(ref, axis=-1)


def test_shading_octree_and_hit_leaves(cuda, shading):
    pb = shading
    assert pb["words"].size == pb["ref_words"].size
    assert np.array_equal(pb["words"], pb["ref_words"])
    assert np.array_equal(pb["center"], pb["ref_center"])
    rgb, hit, _, _ = _forward_backward(cuda, pb)
    # every one of the 6.29 M rays hits the reference's leaf, or misses as it does
    assert hit.size == 24 * 512 * 512
    assert np.array_equal(hit, pb["leaf"])
    assert (pb["leaf"] != 0xFFFFFFFF).sum() > 500_000
    ref = diff_oracle.shade(pb["leaf"], pb["h_rays"][:, 3:], pb["ray_light"], pb["p_rgb"], pb["p_n"])
    assert np.max(np.abs(rgb - ref)) < 2e-6


def test_shading_gradients_plain_central_differences(cuda, shading):
    """Plain central differences, (L(p + h e_k) - L(p - h e_k)) / 2h with
    h = 1e-3 in FP64, on 256 random hit leaves: the adjoint's gradient of
    every leaf's rgb and normal parameters within 1e-4 relative (vector norm
    per leaf).  Normal components whose +-h step crosses a kink of |l.n| or
    max(l.r, 0) for some ray are not differentiable there; their share is
    printed, and they are left out of the normal check."""
    pb = shading
    _, _, g_rgb, g_n = _forward_backward(cuda, pb)
    hit_leaves = np.unique(pb["leaf"][pb["leaf"] != 0xFFFFFFFF])
    leaves = np.random.default_rng(5).choice(hit_leaves, size=256, replace=False)
    fd_rgb, fd_n, kink = diff_oracle.finite_differences(pb["leaf"], pb["h_rays"][:, 3:], pb["ray_light"], pb["p_rgb"],
                                                        pb["p_n"], pb["target"], pb["w"], leaves, h=1e-3)
    li = leaves.astype(np.int64)
    err_rgb = _leaf_rel_err(g_rgb[li], fd_rgb)
    smooth = ~kink.any(axis=1)
    err_n = _leaf_rel_err(g_n[li][smooth], fd_n[smooth])
    print("plain FD h=1e-3 on 256 leaves: rgb max rel %.3g, normal max rel %.3g over %d smooth leaves "
          "(%d with a kink left out)" % (err_rgb.max(), err_n.max(), smooth.sum(), (~smooth).sum()))
    assert err_rgb.max() < REL_TOL
    assert smooth.sum() > 0 and err_n.max() < REL_TOL


def test_shading_gradients_richardson_and_analytic(cuda, shading):
    """The same leaves against Richardson-extrapolated central differences
    (h and h/2), and every hit leaf against the FP64 analytic gradient."""
    pb = shading
    _, _, g_rgb, g_n = _forward_backward(cuda, pb)
    hit_leaves = np.unique(pb["leaf"][pb["leaf"] != 0xFFFFFFFF])
    leaves = np.random.default_rng(5).choice(hit_leaves, size=256, replace=False)
    fd_rgb, fd_n, kink = diff_oracle.finite_differences(pb["leaf"], pb["h_rays"][:, 3:], pb["ray_light"], pb["p_rgb"],
                                                        pb["p_n"], pb["target"], pb["w"], leaves, h=1e-3,
                                                        richardson=True)
    li = leaves.astype(np.int64)
    smooth = ~kink.any(axis=1)
    assert _leaf_rel_err(g_rgb[li], fd_rgb).max() < REL_TOL
    assert _leaf_rel_err(g_n[li][smooth], fd_n[smooth]).max() < REL_TOL
    r_rgb, r_n = diff_oracle.gradient(pb["leaf"], pb["h_rays"][:, 3:], pb["ray_light"], pb["p_rgb"], pb["p_n"],
                                      pb["target"], pb["w"], pb["words"].size)
    hl = hit_leaves.astype(np.int64)
    for gpu, ref in ((g_rgb, r_rgb), (g_n, r_n)):
        num = np.linalg.norm(gpu[hl] - ref[hl], axis=-1)
        den = np.linalg.norm(ref[hl], axis=-1)
        keep = den >= 1e-3 * den.max()  # below that an FP32 sum of cancelling terms has no relative accuracy
        assert keep.mean() > 0.95 and (num[keep] / den[keep]).max() < REL_TOL
    miss = np.ones(pb["words"].size, bool)
    miss[hl] = False
    assert not g_rgb[miss].any() and not g_n[miss].any()
