"""The oracle restatement against the reference compiled in place (CPU only;
skipped where the reference sources are absent)."""
import os

import numpy as np
import pytest

import pyoracle


def test_dragon_decode_and_raymarch(oracle, reference, scenes):
    path = os.path.join(pyoracle.REF_SRC, "models", "XYZRGB-Dragon.oct")
    words, center = oracle.oct_decode(open(path, "rb").read())
    tree = reference.load(path)
    rw, rc = reference.words(tree)
    assert np.array_equal(words, rw) and np.array_equal(center, rc)
    rays = scenes.random_rays(50000, 21, lo=-1.0, hi=4.0)
    for scale in (0.0, 0.003, 0.05):
        h, t, w = reference.raymarch(tree, rays, scale, threads=4)
        out = oracle.raymarch(words, rays, ray_scale=scale, threads=4)
        hit = out["hit"] > 0
        assert np.array_equal(hit.astype(np.uint8), h)
        assert np.array_equal(out["t"][hit].view(np.uint32), t[h == 1].view(np.uint32))
        leaf = out["hit"] == 1
        assert np.array_equal(out["word"][leaf], w[leaf])
    reference.free(tree)


@pytest.mark.parametrize("seed", range(6))
def test_random_builds(oracle, reference, scenes, tmp_path, seed):
    rng = np.random.default_rng(100 + seed)
    vf = str(tmp_path / "g.voxel")
    done = 0
    for _ in range(30):
        w, h, d = (int(v) for v in rng.integers(1, 40, 3))
        mem = int(rng.choice([1 << 30, 200000, 20000, 4096, 3000]))
        if max(w, h, d) < 2 or oracle.cache_block(w, h, d, mem) < 2:
            continue
        grid = scenes.random_grid((d, h, w), float(rng.choice([0.0, 0.02, 0.2, 0.6, 1.0])), int(rng.integers(1 << 30)))
        pyoracle.write_voxel_file(vf, grid)
        ow, oc = oracle.build_dense(grid, mem)
        rw, rc = reference.build_voxel_file(vf, mem)
        assert np.array_equal(ow, rw), (w, h, d, mem)
        assert np.array_equal(oc, rc)
        done += 1
    assert done > 10


def test_sphere_scene_build_and_trace(oracle, reference, scenes, tmp_path):
    grid = scenes.sphere_scene(128, 24, 0)
    vf = str(tmp_path / "s.voxel")
    pyoracle.write_voxel_file(vf, grid)
    ow, oc = oracle.build_dense(grid)
    (rw, rc), tree = reference.build_voxel_file(vf, keep=True)
    assert np.array_equal(ow, rw)
    cam = scenes.orbit_cameras(1, 3, oc)[0]
    rays = scenes.camera_rays(cam, 160, 120)
    h, t, w = reference.raymarch(tree, rays, threads=4)
    out = oracle.raymarch(ow, rays, threads=4)
    assert np.array_equal(out["hit"], h)
    assert np.array_equal(out["t"][h == 1].view(np.uint32), t[h == 1].view(np.uint32))
    assert np.array_equal(out["word"][h == 1], w[h == 1])
    reference.free(tree)


def test_reference_exits_are_rejected_by_oracle(oracle):
    # The reference exits the process when no cache block fits (VoxelData.cpp:236-240)
    # and recurses forever for a virtual side of 1; the oracle reports both.
    with pytest.raises(RuntimeError):
        oracle.build_dense(np.ones((40, 40, 40), np.uint32), mem=100)
    with pytest.raises(RuntimeError):
        oracle.build_dense(np.ones((1, 1, 1), np.uint32))


@pytest.mark.parametrize("scene", ["dragon", "spheres"])
def test_viewer_frames(oracle, reference, scenes, golden, scene):
    """render_oracle.c against the reference's renderBatch / renderTile
    (oracle/ref_render.cpp) over seeded orbit cameras, full and half size."""
    if scene == "dragon":
        words, center = golden["dragon"]["words"], golden["dragon"]["center"]
    else:
        words, center = oracle.build_dense(scenes.sphere_scene(128, 24, 9))
    tree = reference.tree_from_words(words, center)
    rng = np.random.default_rng(31)
    for k in range(4):
        rot, trans, pos = scenes.viewer_camera(rng.uniform(0, 360), rng.uniform(-80, 80), rng.uniform(0.6, 2.5),
                                               center)
        half = k % 2 == 1
        ref = reference.render_frame(tree, rot, trans, half)
        img = oracle.render_frame(words, rot, pos, 1280, 720, 16, 3 if half else 1, threads=4)
        assert np.array_equal(img, ref), (scene, k)
    reference.free(tree)
