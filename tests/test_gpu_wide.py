"""Octrees above 2^32-1 words: the traversal with 64-bit word indices.

Far offsets of such octrees carry bits above 32 in the descriptor's top 14
bits (VoxelOctree.cpp:190-194, decoded at :277-280).  Two checks:
  - the 64-bit kernel forced on ordinary octrees gives the 32-bit kernel's
    (and the oracle's) outputs bit for bit, leaf indices included;
  - real octrees of more than 2^32 words, made from an ordinary octree T by
    moving everything below the root up by a gap G (the root keeps its
    descriptor bits and gets a far word holding the new offset; every other
    offset is relative and unchanged), trace exactly as T does.  One gap puts
    the root's child block above 2^32 (offset high bits 1), another makes the
    block straddle 2^32 (parents and stack entries on both sides).
Each shifted octree holds about 17 GB of device memory.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_OUTS = ("hit", "t", "leaf", "word", "rgb")


def _device_trace(torch, tree, rays, outputs=_OUTS, ray_scale=0.0, light=(0.0, 0.0, 1.0)):
    R = rays.shape[0]
    d_rays = torch.from_numpy(np.ascontiguousarray(rays)).cuda()
    shapes = {"hit": ((R,), torch.uint8), "t": ((R,), torch.float32), "leaf": ((R,), torch.int32),
              "word": ((R,), torch.int32), "rgb": ((R, 3), torch.float32)}
    out = {k: torch.empty(*shapes[k][0], dtype=shapes[k][1], device="cuda") for k in outputs}
    tree.trace(d_rays, ray_scale=ray_scale, light=light, out=out)
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    for k in ("leaf", "word"):
        if k in res:
            res[k] = res[k].view(np.uint32)
    assert tree.device_status() == 0
    return res


def _assert_same(res, ref):
    assert np.array_equal(res["hit"], ref["hit"])
    assert np.array_equal(res["t"].view(np.uint32), ref["t"].view(np.uint32))
    assert np.array_equal(res["word"], ref["word"])
    if "leaf" in res:
        assert np.array_equal(res["leaf"], ref["leaf"])
    g = ref["grey"]
    for c in range(3):
        assert np.array_equal(res["rgb"][:, c].view(np.uint32), g.view(np.uint32))


def _trees(golden, oracle, scenes):
    g = golden["dragon"]
    yield "dragon", g["words"], g["center"]
    grid = scenes.random_grid((64, 64, 64), 0.5, 3)
    words, center = oracle.build_dense(grid)
    assert ((words >> 17) & 1).sum() > 0  # far words below the root
    yield "far", words, center


def test_forced_wide_index_matches_narrow(cuda, svo, golden, oracle, scenes):
    torch = cuda
    for name, words, center in _trees(golden, oracle, scenes):
        rays = np.concatenate([scenes.random_rays(200_000, 11, lo=-0.5, hi=3.5),
                               golden["dragon"]["rays"]])
        tree = svo.VoxelOctree.from_words(words, center)
        narrow = _device_trace(torch, tree, rays)
        tree.set_index_width(64)
        wide = _device_trace(torch, tree, rays)
        ref = oracle.raymarch(words, rays, light=(0.0, 0.0, 1.0), threads=8)
        _assert_same(narrow, ref)
        _assert_same(wide, ref)
        host = tree.trace_host(rays)
        _assert_same(host, ref)
        # the LOD exit as well
        lod = _device_trace(torch, tree, rays, outputs=("hit", "t"), ray_scale=0.02)
        lref = oracle.raymarch(words, rays, ray_scale=0.02, threads=8)
        assert np.array_equal(lod["hit"], lref["hit"])
        assert np.array_equal(lod["t"].view(np.uint32), lref["t"].view(np.uint32))
        tree.set_index_width(32)
        tree.close()


def test_index_width_argument_checks(cuda, svo, golden):
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    for bad in (0, 16, 48, 128):
        with pytest.raises(svo.SvoError) as e:
            tree.set_index_width(bad)
        assert e.value.code == svo.SVO_ERR_INVALID


def _shifted(words, gap):
    """T with everything below the root moved up by `gap` words: the root
    gets a far word (at index 1) holding the child block's new offset."""
    n = 2 + gap + (words.size - 1)
    big = np.zeros(n, np.uint32)  # calloc'd: untouched pages stay unmapped
    off = 2 + gap
    big[0] = (int(words[0]) & 0x1FFFF) | 0x20000 | ((off >> 32) << 18)
    big[1] = off & 0xFFFFFFFF
    big[off:] = words[1:]
    return big


@pytest.mark.parametrize("where", ["above", "straddle"])
def test_octree_above_2e32_words(cuda, svo, golden, oracle, scenes, where):
    torch = cuda
    free, _ = torch.cuda.mem_get_info()
    if free < 24 << 30:
        pytest.skip("needs about 20 GB of free device memory")
    grid = scenes.random_grid((64, 64, 64), 0.5, 3)
    words, center = oracle.build_dense(grid)
    gap = (1 << 32) + 5 if where == "above" else (1 << 32) - words.size // 2
    big = _shifted(words, gap)
    assert big.size > 0xFFFFFFFF
    rays = np.concatenate([scenes.random_rays(300_000, 12, lo=-0.5, hi=3.5),
                           scenes.random_rays(20_000, 13, lo=0.9, hi=2.1)])
    ref = oracle.raymarch(words, rays, light=(0.0, 0.0, 1.0), threads=8)
    tree = svo.VoxelOctree.from_words(big, center)
    del big
    try:
        assert tree.num_words() == 2 + gap + words.size - 1
        res = _device_trace(torch, tree, rays, outputs=("hit", "t", "word", "rgb"))
        _assert_same(res, ref)
        assert (ref["hit"] == 1).sum() > 1000
        host = tree.trace_host(rays, outputs=("hit", "t", "word", "rgb"))
        _assert_same(host, ref)
        lod = _device_trace(torch, tree, rays, outputs=("hit", "t"), ray_scale=0.02)
        lref = oracle.raymarch(words, rays, ray_scale=0.02, threads=8)
        assert np.array_equal(lod["hit"], lref["hit"])
        assert np.array_equal(lod["t"].view(np.uint32), lref["t"].view(np.uint32))
        # what the 32-bit interfaces cannot express is refused, not truncated
        d_rays = torch.from_numpy(rays[:64].copy()).cuda()
        leaf = torch.empty(64, dtype=torch.int32, device="cuda")
        with pytest.raises(svo.SvoError) as e:
            tree.trace(d_rays, out={"leaf": leaf})
        assert e.value.code == svo.SVO_ERR_LIMIT
        with pytest.raises(svo.SvoError) as e:
            tree.set_index_width(32)
        assert e.value.code == svo.SVO_ERR_LIMIT
        with pytest.raises(svo.SvoError) as e:
            tree.trace_image(d_rays, 8, 8)
        assert e.value.code == svo.SVO_ERR_LIMIT
        with pytest.raises(svo.SvoError) as e:
            tree.count_loads(d_rays, loads=leaf)
        assert e.value.code == svo.SVO_ERR_LIMIT
        with pytest.raises(svo.SvoError) as e:
            tree.render_frame(np.eye(3, dtype=np.float32).ravel(), (0.5, 0.5, -2.0), 64, 64, 4)
        assert e.value.code == svo.SVO_ERR_LIMIT
    finally:
        tree.close()
        torch.cuda.synchronize()


def _mem_available_host():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def test_build_above_2e32_words(cuda, svo, oracle):
    """A real build past 2^32 words: a 1600^3 grid with about 3% holes
    (3.97 G voxels; each voxel's word is its linear index + 1) gives an
    octree of about 4.6 G words whose upper far offsets exceed 32 bits.  The
    host walk checks every offset and counts the leaves; the 64-bit trace
    matches the oracle's traversal of the same words bit for bit, and every
    hit lies in the voxel its word names."""
    torch = cuda
    torch.cuda.empty_cache()
    svo.trim_memory()
    free, _ = torch.cuda.mem_get_info()
    if free < 200 << 30:
        pytest.skip("needs about 200 GB of free device memory")
    if _mem_available_host() < 64 << 30:
        pytest.skip("needs about 64 GB of available host memory")
    W = H = D = 1600
    g = torch.empty((D, H, W), dtype=torch.int32, device="cuda")
    yy, xx = torch.meshgrid(torch.arange(H, device="cuda", dtype=torch.int64),
                            torch.arange(W, device="cuda", dtype=torch.int64), indexing="ij")
    plane = xx + W * yy
    hx = (xx * 73856093) ^ (yy * 19349663)
    n_vox = torch.zeros((), dtype=torch.int64, device="cuda")
    for z in range(D):
        hole = ((hx ^ (z * 83492791)) & 31) == 0
        v = torch.where(hole, torch.zeros_like(plane), plane + (W * H * z + 1))
        g[z] = v.to(torch.int32)  # the low 32 bits: indices above 2^31 wrap to negative int32
        n_vox += (~hole).sum()
    del yy, xx, plane, hx, hole, v
    n_vox = int(n_vox.item())
    assert 3_900_000_000 < n_vox < 0xFFFFFFFF
    tree = svo.VoxelOctree(svo.VoxelData(g))
    del g
    torch.cuda.empty_cache()
    svo.trim_memory()
    try:
        n_words = tree.num_words()
        assert n_words > 0xFFFFFFFF
        nd, nl = tree.validate()
        assert nl == n_vox
        print("octree of %d words: %d descriptors, %d leaves" % (n_words, nd, nl))
        S = 2048.0  # the virtual side: voxel (x, y, z) spans [1 + x/S, 1 + (x+1)/S] per axis
        rng = np.random.default_rng(21)
        R = 200_000
        o = rng.uniform(0.8, 1.0 + 1600 / S + 0.2, (R, 3)).astype(np.float32)
        d = rng.normal(size=(R, 3)).astype(np.float32)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rays = np.concatenate([o, d], axis=1).astype(np.float32)
        res = _device_trace(torch, tree, rays, outputs=("hit", "t", "word", "rgb"))
        words = tree.words()
        ref = oracle.raymarch(words, rays, light=(0.0, 0.0, 1.0), threads=16)
        del words
        _assert_same(res, ref)
        hit = res["hit"] == 1
        assert hit.mean() > 0.3
        lin = res["word"][hit].astype(np.int64) - 1
        z, rem = np.divmod(lin, W * H)
        y, x = np.divmod(rem, W)
        vox = np.stack([x, y, z], 1).astype(np.float64)
        p = o[hit].astype(np.float64) + d[hit].astype(np.float64) * res["t"][hit].astype(np.float64)[:, None]
        tol = 1e-3
        inside = np.all((p >= 1.0 + vox / S - tol) & (p <= 1.0 + (vox + 1) / S + tol), axis=1)
        assert inside.all()
        # the root's last child block (all coordinates >= 1024) holds the
        # last ~220 M words, all above 2^32: hits there too
        assert np.all(vox >= 1024, axis=1).sum() > 100
    finally:
        tree.close()
        svo.trim_memory()
        torch.cuda.synchronize()
