"""svo_octree_build_dense_noalloc: the GPU build for callers that cannot
allocate device memory while they run (an application whose device memory is
already handed to its own pool, or a frame loop that must avoid the
device-wide synchronisation of cudaMalloc/cudaFree).  It works inside one
fixed device arena of the library, so this test calls it twice in a row
(and once more) and checks every result against the allocating entry point,
svo_octree_build_dense, and against the oracle's restatement of
VoxelOctree(VoxelData*).  Collected last so that a failure here never hides
the other tests' results."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_build(svo, torch, grid, mem, capacity=None):
    d, h, w = grid.shape
    dg = torch.from_numpy(np.ascontiguousarray(grid).view(np.int32)).cuda()
    cap = capacity if capacity is not None else 4 * grid.size + 16
    out = torch.zeros(cap, dtype=torch.int32, device="cuda")
    n = ctypes.c_uint64()
    c = np.zeros(3, np.float32)
    rc = svo.lib.svo_octree_build_dense_noalloc(ctypes.c_void_p(dg.data_ptr()), w, h, d, ctypes.c_uint64(mem),
                                                ctypes.c_void_p(out.data_ptr()), ctypes.c_uint64(cap),
                                                ctypes.byref(n), c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                None)
    return rc, out[:n.value].cpu().numpy().view(np.uint32) if rc == 0 else None, c, n.value


def _reference_build(svo, grid, mem):
    tree = svo.VoxelOctree(svo.VoxelData(grid, mem))
    return tree.words(), tree.center()


def test_noalloc_build_matches_allocating_build(cuda, svo, scenes, oracle):
    torch = cuda
    svo.lib.svo_octree_build_dense_noalloc.restype = ctypes.c_int
    # a grid with several cache blocks and an odd depth (empty descriptors),
    # then a sphere scene with one cache block, then the first grid again:
    # each call must start from a clean arena.
    g1 = np.zeros((41, 40, 40), np.uint32)
    g1[40, 3, 3] = 5
    g1[40, 20, 33] = 6
    g1[10:20, 10:30, 5:25] = np.arange(1, 1 + 10 * 20 * 20, dtype=np.uint32).reshape(10, 20, 20)
    g2 = scenes.sphere_scene(64, 10, 3)
    for grid, mem in ((g1, 3000), (g2, 1 << 30), (g1, 3000)):
        rc, words, center, n = _noalloc_build(svo, torch, grid, mem)
        assert rc == 0, svo.lib.svo_last_error()
        ref_words, ref_center = _reference_build(svo, grid, mem)
        assert n == ref_words.size
        assert np.array_equal(words, ref_words)
        assert np.array_equal(center, ref_center)
        # and the oracle's restatement of VoxelOctree(VoxelData*) itself
        o_words, o_center = oracle.build_dense(grid, mem)
        assert np.array_equal(words, o_words)
        assert np.array_equal(center, o_center)


def test_noalloc_build_rejects_sizes_beyond_its_limits(cuda, svo):
    torch = cuda
    svo.lib.svo_octree_build_dense_noalloc.restype = ctypes.c_int
    full = np.ones((128, 128, 128), np.uint32)  # 2,097,152 voxels > 262,144
    rc, _, _, _ = _noalloc_build(svo, torch, full, 1 << 30)
    assert rc == svo.SVO_ERR_LIMIT and b"262144" in svo.lib.svo_last_error()
    big = np.zeros((1, 1, 300), np.uint32)  # virtual side 512 > 256
    rc, _, _, _ = _noalloc_build(svo, torch, big, 1 << 30)
    assert rc == svo.SVO_ERR_LIMIT
    # a side past 2^30 is refused before the grid is touched
    n = ctypes.c_uint64()
    c = np.zeros(3, np.float32)
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
    rc = svo.lib.svo_octree_build_dense_noalloc(ctypes.c_void_p(dummy.data_ptr()), 1, 1, (1 << 30) + 1,
                                                ctypes.c_uint64(1 << 30), ctypes.c_void_p(dummy.data_ptr()),
                                                ctypes.c_uint64(16), ctypes.byref(n),
                                                c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), None)
    assert rc == svo.SVO_ERR_LIMIT
    small = np.ones((8, 8, 8), np.uint32)
    rc, _, _, n = _noalloc_build(svo, torch, small, 1 << 30, capacity=4)
    assert rc == svo.SVO_ERR_LIMIT and n == _reference_build(svo, small, 1 << 30)[0].size
