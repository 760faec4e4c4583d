"""The reference-side binding: include/svo_voxel_octree.hpp, the
VoxelOctree-shaped C++ class a maintainer of the reference would add
(src/VoxelOctree.hpp:37-58), compiled with g++ as C++11 (the reference's
standard) and linked against libsvo_gb300.so.

Without a GPU: the program builds with -Wall -Werror, its .oct read/write
through the C ABI round-trips the reference's dragon words, and loading a
missing file throws instead of leaving a broken object.
On the GPU: VoxelOctreeGpu(path), center(), save() and both raymarch forms
return what the reference's own VoxelOctree::raymarch returned for the
dragon's golden rays (tests/golden/dragon.npz, written from the reference)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "sparse-voxel-octrees_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "voxel_octree_main.cpp")


@pytest.fixture(scope="module")
def program(svo, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("cpp") / "voxel_octree_main")
    cmd = ["g++", "-std=c++11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", PKG_DIR, "-lsvo_gb300", "-Wl,-rpath," + PKG_DIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_wrapper_host_paths(program, svo, golden, tmp_path):
    g = golden["dragon"]
    src, dst = str(tmp_path / "in.oct"), str(tmp_path / "out.oct")
    svo.oct_write(src, g["words"], g["center"])
    r = subprocess.run([program, "host", src, dst], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "words %d" % g["words"].size in r.stdout
    assert "error: " in r.stdout and "missing.oct" in r.stdout
    w, c = svo.oct_read(dst)
    assert np.array_equal(w, g["words"]) and np.array_equal(c, g["center"])


@pytest.mark.gpu
def test_wrapper_matches_reference_raymarch(cuda, program, svo, golden, tmp_path):
    g = golden["dragon"]
    src, saved = str(tmp_path / "dragon.oct"), str(tmp_path / "saved.oct")
    rays_bin, res_bin = str(tmp_path / "rays.bin"), str(tmp_path / "res.bin")
    svo.oct_write(src, g["words"], g["center"])
    rays = np.ascontiguousarray(g["rays"], np.float32)
    rays.tofile(rays_bin)
    r = subprocess.run([program, "gpu", src, saved, rays_bin, res_bin], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    c = np.array([float(x) for x in r.stdout.split("center")[1].split()[:3]], np.float32)
    assert np.array_equal(c, g["center"])
    w, c2 = svo.oct_read(saved)
    assert np.array_equal(w, g["words"]) and np.array_equal(c2, g["center"])

    n = rays.shape[0]
    buf = open(res_bin, "rb").read()
    off = 0

    def take(dtype):
        nonlocal off
        a = np.frombuffer(buf, dtype, n, off)
        off += n * np.dtype(dtype).itemsize
        return a

    hit, t, normal = take(np.uint8), take(np.float32), take(np.uint32)
    lod_hit, lod_t = take(np.uint8), take(np.float32)
    one_hit, one_t, one_normal = take(np.uint8), take(np.float32), take(np.uint32)
    # the reference's results: hit flag, and t and word where it hit
    ref_hit = g["hit"] == 1
    assert np.array_equal(hit == 1, ref_hit)
    assert np.array_equal(t[ref_hit].view(np.uint32), g["t"][ref_hit].view(np.uint32))
    assert np.array_equal(normal[ref_hit], g["word"][ref_hit])
    # level-of-detail exits count as hits, with the exit's t
    ref_lod = g["lod_hit"] == 1
    assert np.array_equal(lod_hit != 0, ref_lod)
    assert np.array_equal(lod_t[ref_lod].view(np.uint32), g["lod_t"][ref_lod].view(np.uint32))
    # the one-ray form
    assert np.array_equal(one_hit == 1, ref_hit)
    assert np.array_equal(one_t[ref_hit].view(np.uint32), g["t"][ref_hit].view(np.uint32))
    assert np.array_equal(one_normal[ref_hit], g["word"][ref_hit])
    assert not one_t[~ref_hit].any() and not one_normal[~ref_hit].any()
    assert ref_hit.sum() > 500
