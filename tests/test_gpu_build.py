"""GPU build parity: svo_octree_build_dense / _voxel_file against the oracle's
restatement of VoxelOctree(VoxelData*) and the reference's committed word
streams — octree words bit-exact, centers exact."""
import numpy as np
import pytest

import pyoracle
from conftest import golden_builds

pytestmark = pytest.mark.gpu


def _build(svo, grid, mem=1 << 30):
    tree = svo.VoxelOctree(svo.VoxelData(grid, mem))
    return tree.words(), tree.center(), tree


def test_golden_builds(svo, golden):
    for grid, mem, words, center in golden_builds(golden):
        w, c, _ = _build(svo, grid, mem)
        assert np.array_equal(w, words), (grid.shape, mem)
        assert np.array_equal(c, center)


@pytest.mark.parametrize("seed", range(8))
def test_random_grids(svo, oracle, scenes, seed):
    rng = np.random.default_rng(1000 + seed)
    done = 0
    for _ in range(25):
        w, h, d = (int(v) for v in rng.integers(1, 72, 3))
        mem = int(rng.choice([1 << 30, 1 << 30, 200000, 20000, 4096, 3000]))
        if max(w, h, d) < 2 or oracle.cache_block(w, h, d, mem) < 2:
            continue
        dens = float(rng.choice([0.0, 0.001, 0.03, 0.3, 0.8, 1.0]))
        grid = scenes.random_grid((d, h, w), dens, int(rng.integers(1 << 30)))
        ow, oc = oracle.build_dense(grid, mem)
        gw, gc, _ = _build(svo, grid, mem)
        assert np.array_equal(gw, ow), (w, h, d, mem, dens)
        assert np.array_equal(gc, oc)
        done += 1
    assert done >= 10


def test_edge_grids(svo, oracle):
    cases = [np.zeros((2, 2, 2), np.uint32), np.ones((2, 2, 2), np.uint32), np.zeros((16, 16, 16), np.uint32)]
    for i in range(8):  # one voxel in each octant of a 4^3 grid
        g = np.zeros((4, 4, 4), np.uint32)
        g[(i >> 2) * 3, ((i >> 1) & 1) * 3, (i & 1) * 3] = 7 + i
        cases.append(g)
    cases.append(np.arange(1, 1 + 32 ** 3, dtype=np.uint32).reshape(32, 32, 32))  # full tree
    cases.append(np.ones((1, 1, 3), np.uint32))
    for g in cases:
        ow, oc = oracle.build_dense(g)
        gw, gc, _ = _build(svo, g)
        assert np.array_equal(gw, ow), g.shape
        assert np.array_equal(gc, oc)
    assert np.array_equal(_build(svo, np.zeros((2, 2, 2), np.uint32))[0], np.array([1 << 18], np.uint32))


def _morton_grid(side, keep):
    """A side^3 grid holding a voxel at each Morton code m < side^3 with
    keep(m) true (value m + 1), laid out z, y, x."""
    m = np.arange(side ** 3, dtype=np.int64)
    x = np.zeros_like(m)
    y = np.zeros_like(m)
    z = np.zeros_like(m)
    for b in range(int(np.log2(side))):
        x |= ((m >> (3 * b)) & 1) << b
        y |= ((m >> (3 * b + 1)) & 1) << b
        z |= ((m >> (3 * b + 2)) & 1) << b
    g = np.zeros((side, side, side), np.uint32)
    sel = keep(m)
    g[z[sel], y[sel], x[sel]] = (m[sel] + 1).astype(np.uint32)
    return g


def test_level_grouping_runs_and_tiles(svo, oracle):
    """Runs of siblings that cross 32-child rounds and 2048-child tiles (the
    level grouping finishes them from the next round's leading run, or past a
    tile from the keys after it), ragged last tiles, and dense rounds."""
    side = 64
    cases = [
        _morton_grid(side, lambda k: np.ones_like(k, bool)),  # every code: full runs of 8
        _morton_grid(side, lambda k: (k % 8) >= 3),  # runs of 5 starting at octant 3
        _morton_grid(side, lambda k: (k // 8) % 3 != 1),  # full runs with gaps between parents
        _morton_grid(side, lambda k: (k % 8 == 7) | (k % 16 == 8)),  # runs of 1 and 2
        _morton_grid(side, lambda k: k < 2048 * 5 + 37),  # a ragged last tile at level 1
        _morton_grid(side, lambda k: (k >= 2048 - 5) & (k < 2048 + 3)),  # one run across a tile
    ]
    rng = np.random.default_rng(77)
    for _ in range(3):  # random run lengths: each parent keeps a random prefix of its octants
        lens = rng.integers(0, 9, side ** 3 // 8)
        cases.append(_morton_grid(side, lambda k, lens=lens: (k % 8) < lens[k // 8]))
    for g in cases:
        ow, oc = oracle.build_dense(g)
        gw, gc, _ = _build(svo, g)
        assert np.array_equal(gw, ow), int((g != 0).sum())
        assert np.array_equal(gc, oc)


def test_odd_slice_empty_descriptor(svo, oracle):
    # Cache blocks of 8^3 (mem 3000 at side 64) and odd depth 41: a block whose
    # only voxels lie in the last z slice becomes a descriptor with no children.
    g = np.zeros((41, 40, 40), np.uint32)
    g[40, 3, 3] = 5
    g[40, 20, 33] = 6
    g[10, 10, 10] = 9
    ow, _ = oracle.build_dense(g, 3000)
    gw, _, _ = _build(svo, g, 3000)
    assert np.array_equal(gw, ow)
    assert 9 in ow and 5 not in ow[1:]  # the last slice's voxels are dropped
    # two descriptors with no children (offset set, masks 0), one per such block
    assert sum(1 for x in ow[1:] if (int(x) & 0x1FFFF) == 0 and int(x) >> 18) == 2


def test_far_pointers(svo, oracle, scenes):
    g = scenes.random_grid((96, 96, 96), 0.4, 7)
    ow, _ = oracle.build_dense(g)
    gw, _, tree = _build(svo, g)
    assert np.array_equal(gw, ow)
    assert ((gw >> 16) & 1).sum() > 0  # hasLargeChildren somewhere
    nd, nl = tree.validate()
    assert nl == int((g != 0).sum())


def test_sphere_scene_256(svo, oracle, scenes):
    g = scenes.sphere_scene(256, 48, 0)
    ow, oc = oracle.build_dense(g)
    gw, gc, tree = _build(svo, g)
    assert np.array_equal(gw, ow) and np.array_equal(gc, oc)
    nd, nl = tree.validate()
    assert nl == int((g != 0).sum())


def test_device_grid_input(cuda, svo, oracle, scenes):
    torch = cuda
    g = scenes.terrain_scene(128, 20, 3)
    ow, _ = oracle.build_dense(g)
    dg = torch.from_numpy(g.view(np.int32)).cuda()
    tree = svo.VoxelOctree(svo.VoxelData(dg))
    assert np.array_equal(tree.words(), ow)


def test_voxel_file_build_and_save_load(svo, oracle, scenes, tmp_path):
    g = scenes.random_grid((37, 50, 61), 0.2, 9)
    vf = str(tmp_path / "g.voxel")
    pyoracle.write_voxel_file(vf, g)
    tree = svo.VoxelOctree(svo.VoxelData(vf, 20000))
    ow, oc = oracle.build_dense(g, 20000)
    assert np.array_equal(tree.words(), ow)
    p = str(tmp_path / "t.oct")
    tree.save(p)
    back = svo.VoxelOctree(p)
    assert np.array_equal(back.words(), ow) and np.array_equal(back.center(), oc)
    w2, c2 = oracle.oct_decode(open(p, "rb").read())
    assert np.array_equal(w2, ow)


def _streamed(svo, path, mem, slices, plane):
    tree = svo.VoxelOctree(svo.VoxelData(path, mem, slab_bytes=slices * plane * 4))
    return tree.words(), tree.center()


def test_streamed_voxel_file_golden(svo, golden, tmp_path):
    """The streamed .voxel build (16-slice slabs) against the reference's own
    word streams."""
    n = 0
    for grid, mem, words, center in golden_builds(golden):
        d, h, w = grid.shape
        if max(w, h, d) < 16:
            continue
        path = str(tmp_path / "g.voxel")
        pyoracle.write_voxel_file(path, grid)
        ws, c = _streamed(svo, path, mem, 16, w * h)
        assert np.array_equal(ws, words), (grid.shape, mem)
        assert np.array_equal(c, center)
        n += 1
    assert n >= 8


@pytest.mark.parametrize("shape,density,mem,slices", [((77, 90, 101), 0.02, 1 << 30, 16),
                                                        ((64, 64, 63), 0.3, 20000, 32),
                                                        ((200, 150, 131), 0.001, 100000, 48),
                                                        ((17, 300, 47), 0.05, 60000, 16)])
def test_streamed_voxel_file_matches_oracle(svo, oracle, scenes, tmp_path, shape, density, mem, slices):
    grid = scenes.random_grid(shape, density, sum(shape))
    d, h, w = grid.shape
    path = str(tmp_path / "r.voxel")
    pyoracle.write_voxel_file(path, grid)
    ow, oc = oracle.build_dense(grid, mem)
    ws, c = _streamed(svo, path, mem, slices, w * h)
    assert np.array_equal(ws, ow) and np.array_equal(c, oc)
    # the whole-grid form of the same file agrees
    tree = svo.VoxelOctree(svo.VoxelData(path, mem))
    assert np.array_equal(tree.words(), ow)


def test_streamed_terrain_scene(svo, oracle, scenes, tmp_path):
    grid = scenes.terrain_scene(256, 20, 3)
    path = str(tmp_path / "t.voxel")
    pyoracle.write_voxel_file(path, grid)
    ow, oc = oracle.build_dense(grid, 1 << 20)
    ws, c = _streamed(svo, path, 1 << 20, 64, 256 * 256)
    assert np.array_equal(ws, ow) and np.array_equal(c, oc)


def test_grid_alignment_paths(cuda, svo, oracle, scenes):
    """Bricks wholly inside a grid whose rows start on 16-byte boundaries are
    read as uint4; the same grid at a 4-byte offset, or with a width that is
    not a multiple of 4, is read word by word.  Both give the oracle's words,
    with cache blocks larger and smaller than a brick (the budget 3000 gives
    8^3 blocks, whose flags the count kernel sets voxel by voxel)."""
    torch = cuda
    for shape in ((48, 40, 64), (33, 50, 36), (32, 32, 30)):
        g = scenes.random_grid(shape, 0.3, 11)
        n = g.size
        flat = torch.from_numpy(g.reshape(-1).view(np.int32)).cuda()
        buf = torch.zeros(n + 8, dtype=torch.int32, device="cuda")
        for mem in (1 << 30, 3000):
            ow, oc = oracle.build_dense(g, mem)
            for off in (0, 1, 4):  # 16-byte aligned, 4-byte aligned, 16-byte aligned
                buf[off:off + n] = flat
                tree = svo.VoxelOctree(svo.VoxelData(buf[off:off + n].view(shape), mem))
                assert np.array_equal(tree.words(), ow), (shape, mem, off)
                assert np.array_equal(tree.center(), oc)
