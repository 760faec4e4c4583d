"""The viewer's frame (svo_render_frame) against the reference's own
renderBatch + renderTile frames of the dragon (tests/golden/frames.npz) and
the oracle's restatement (oracle/render_oracle.c, pinned to those frames):
bit-identical RGBA8 frames across cameras, strip layouts, half-size mode and
frame sizes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frame(cuda, tree, cam, **kw):
    return tree.render_frame(cam[:9], cam[9:12], **kw).cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("W,H,strips,stride", [(1280, 720, 16, 1), (1280, 720, 16, 3), (640, 480, 7, 1),
                                               (333, 211, 5, 2), (64, 40, 1, 1), (17, 9, 9, 1)])
def test_dragon_frames_match_oracle(cuda, svo, golden, oracle, scenes, W, H, strips, stride):
    g = golden["dragon"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    for cam in scenes.orbit_cameras(3, W + H + strips, g["center"], radius=1.2, radius_hi=2.5):
        img = _frame(cuda, tree, cam, width=W, height=H, n_strips=strips, pixel_stride=stride)
        ref = oracle.render_frame(g["words"], cam[:9], cam[9:12], W, H, strips, stride, threads=4)
        assert np.array_equal(img, ref)
        assert (ref != 0).mean() > 0.02
    assert tree.device_status() == 0


def test_scene_frame_and_strip_dependence(cuda, svo, oracle, scenes):
    grid = scenes.terrain_scene(256, 12, 4)
    words, center = oracle.build_dense(grid)
    tree = svo.VoxelOctree.from_words(words, center)
    cam = scenes.camera(40.0, 25.0, 1.3, center)
    a = _frame(cuda, tree, cam, n_strips=16)
    assert np.array_equal(a, oracle.render_frame(words, cam[:9], cam[9:12], 1280, 720, 16, 1, threads=8))
    b = _frame(cuda, tree, cam, n_strips=12)
    assert np.array_equal(b, oracle.render_frame(words, cam[:9], cam[9:12], 1280, 720, 12, 1, threads=8))
    assert (a != 0).mean() > 0.3


def test_inside_the_tree_and_empty_view(cuda, svo, oracle, scenes):
    grid = scenes.sphere_scene(128, 30, 2)
    words, center = oracle.build_dense(grid)
    tree = svo.VoxelOctree.from_words(words, center)
    inside = scenes.camera(10.0, 5.0, 0.05, center)  # camera inside the octree's cube
    away = scenes.camera(0.0, 0.0, -3.0, center)     # looking away from it
    for cam in (inside, away):
        img = _frame(cuda, tree, cam, width=320, height=200, n_strips=4)
        assert np.array_equal(img, oracle.render_frame(words, cam[:9], cam[9:12], 320, 200, 4, 1, threads=4))


def test_frames_match_reference_renderer(cuda, svo, golden):
    g, f = golden["dragon"], golden["frames"]
    tree = svo.VoxelOctree.from_words(g["words"], g["center"])
    for rot, pos, half, ref in zip(f["rot"], f["pos"], f["half"], f["frames"]):
        img = tree.render_frame(rot, pos, 1280, 720, 16, 3 if half else 1).cpu().numpy().view(np.uint32)
        assert np.array_equal(img, ref)
    assert tree.device_status() == 0
