"""The GPU scene generators (libsvo_scenes.so) reproduce scenes.py bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("side,seed", [(64, 0), (128, 3)])
def test_sphere_scene(cuda, scenes, side, seed):
    ref = scenes.sphere_scene(side, 24, seed)
    got = scenes.gpu_sphere_scene(side, 24, seed).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("side", [32, 128])
def test_terrain_scene(cuda, scenes, side):
    ref = scenes.terrain_scene(side, 30, 5)
    got = scenes.gpu_terrain_scene(side, 30, 5).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, ref)


def test_camera_rays(cuda, scenes):
    for cam in scenes.orbit_cameras(4, 9, (0.5, 0.5, 0.5), radius=1.3, radius_hi=2.2):
        ref = scenes.camera_rays(cam, 211, 97)
        got = scenes.gpu_camera_rays(cam, 211, 97).cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
