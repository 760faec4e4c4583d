"""The CPU-only setup of the benchmark's reference leg (oracle/scene_build.c):
its scenes equal scenes.py's, and its sorted-voxel build equals the faithful
restatement of VoxelOctree(VoxelData*)."""
import numpy as np
import pytest


def _morton(x, y, z):
    key = np.zeros(x.shape, np.uint64)
    for b in range(21):
        key |= ((x.astype(np.uint64) >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b)
        key |= ((y.astype(np.uint64) >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b + 1)
        key |= ((z.astype(np.uint64) >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b + 2)
    return key


def _sparse(grid):
    z, y, x = np.nonzero(grid)
    keys = _morton(x, y, z)
    order = np.argsort(keys, kind="stable")
    return keys[order], grid[z, y, x][order]


@pytest.mark.parametrize("side", [32, 64])
def test_scene_voxels_match_numpy(oracle, scenes, side):
    heights, centers, radii = scenes.terrain_scene_params(side, 40, 2)
    ref = scenes.terrain_scene(side, 40, 2)
    boxes = scenes.sphere_boxes((side,) * 3, centers, radii)
    params = np.concatenate([centers, radii[:, None]], 1)
    keys, pay = oracle.scene_voxels(side, heights, boxes, params, threads=4)
    rk, rp = _sparse(ref)
    assert np.array_equal(keys, rk) and np.array_equal(pay, rp)


def test_sphere_scene_voxels_match_numpy(oracle, scenes):
    side = 128
    centers, radii = scenes.sphere_scene_params(side, 30, 4)
    ref = scenes.sphere_scene(side, 30, 4)
    params = np.concatenate([centers, radii[:, None]], 1)
    keys, pay = oracle.scene_voxels(side, None, scenes.sphere_boxes((side,) * 3, centers, radii), params, threads=3)
    rk, rp = _sparse(ref)
    assert np.array_equal(keys, rk) and np.array_equal(pay, rp)


@pytest.mark.parametrize("side,density,seed", [(2, 0.5, 1), (8, 0.3, 2), (16, 0.0, 3), (32, 1.0, 4),
                                               (64, 0.05, 5), (64, 0.4, 6), (128, 0.01, 7)])
def test_build_sorted_matches_faithful_build(oracle, scenes, side, density, seed):
    grid = scenes.random_grid((side, side, side), density, seed)
    ref, _ = oracle.build_dense(grid)
    keys, pay = _sparse(grid)
    log_side = side.bit_length() - 1
    assert np.array_equal(oracle.build_sorted(keys, pay, log_side), ref)


def test_build_sorted_scene(oracle, scenes):
    grid = scenes.sphere_scene(256, 48, 0)
    ref, _ = oracle.build_dense(grid)
    keys, pay = _sparse(grid)
    assert np.array_equal(oracle.build_sorted(keys, pay, 8), ref)
