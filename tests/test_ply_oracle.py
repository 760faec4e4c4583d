"""The oracle's mesh path (ply_oracle.c: PlyLoader + VoxelData(PlyLoader*)
+ VoxelOctree) against the reference compiled in place, and against the
committed ply.npz fixture.  CPU only."""
import os

import numpy as np
import pytest

from conftest import golden_ply, golden_volumes


def _be_floats(v):
    """What the reference reads for FP32 values stored big-endian: plyfile
    reads the bytes in host order and converts float -> double -> float
    (which quiets signalling-NaN patterns), then PlyLoader swaps the bytes."""
    g = np.asarray(v, np.float32).astype(">f4").view("<f4")
    with np.errstate(invalid="ignore"):
        g = g.astype(np.float64).astype(np.float32)
    return g.view(">f4").astype(np.float32)


def test_golden_ply_builds(oracle, golden):
    n = 0
    for mesh, side, threads, mem, words, center in golden_ply(golden):
        w, c = oracle.build_mesh(mesh["pos"], mesh["faces"], side, threads, mem, colors=mesh["colors"],
                                 normals=mesh["normals"])
        assert np.array_equal(w, words), (side, threads, mem)
        assert np.array_equal(c, center)
        n += 1
    assert n == 6


def test_tri_box_overlap_matches_reference(oracle, reference):
    rng = np.random.default_rng(0)
    for i in range(4000):
        c = rng.random(3).astype(np.float32)
        h = (rng.random(3) * 0.1 + 0.01).astype(np.float32)
        v = (c + rng.normal(size=(3, 3)) * (0.05 if i % 2 else 0.2)).astype(np.float32)
        if i % 7 == 0:  # a vertex on a box face
            v[0, i % 3] = c[i % 3] + h[i % 3]
        assert oracle.tri_box_overlap(c, h, v) == reference.tri_box_overlap(c, h, v)


@pytest.mark.parametrize("side,threads,mem", [(48, 1, 1 << 30), (48, 8, 1 << 30), (80, 4, 5 * 16 ** 3 + 3000),
                                              (57, 16, 5 * 8 ** 3 + 2000), (128, 6, 5 * 32 ** 3 + 40000)])
def test_mesh_build_matches_reference(oracle, reference, scenes, tmp_path, side, threads, mem):
    pos, faces, col = scenes.edge_case_mesh(3, side)
    path = str(tmp_path / "m.ply")
    scenes.write_ply(path, pos, faces, colors=col)
    rw, rc = reference.build_ply(path, side, mem, threads=threads)
    ow, oc = oracle.build_mesh(pos, faces, side, threads, mem, colors=col.astype(np.float32))
    assert np.array_equal(rw, ow)
    assert np.array_equal(rc, oc)


def test_ascii_and_normals_match_reference(oracle, reference, scenes, tmp_path):
    pos, faces, col = scenes.edge_case_mesh(2, 9)
    nrm = np.random.default_rng(2).normal(size=pos.shape).astype(np.float32)
    path = str(tmp_path / "a.ply")
    scenes.write_ply(path, pos, faces, colors=col, normals=nrm, binary=False)
    rw, _ = reference.build_ply(path, 64, 1 << 30, threads=4)
    ow, _ = oracle.build_mesh(pos, faces, 64, 4, 1 << 30, colors=col.astype(np.float32), normals=nrm)
    assert np.array_equal(rw, ow)
    flat, _ = oracle.build_mesh(pos, faces, 64, 4, 1 << 30, colors=col.astype(np.float32))
    assert not np.array_equal(flat, ow)  # the file's normals were used


def test_big_endian_matches_reference(oracle, reference, scenes, tmp_path):
    pos, faces, col = scenes.edge_case_mesh(3, 4)
    path = str(tmp_path / "be.ply")
    scenes.write_ply(path, pos, faces, colors=col, big_endian=True)
    rw, rc = reference.build_ply(path, 64, 1 << 30, threads=4)
    # colours: uchar -> float, then swapped (garbage, as in the reference)
    c2 = col.astype(np.float32).astype(">f4").view("<f4").astype(np.float32)
    ow, oc = oracle.build_mesh(_be_floats(pos), faces, 64, 4, 1 << 30, colors=c2)
    assert np.array_equal(rw, ow) and np.array_equal(rc, oc)


def test_thread_count_and_budget_change_the_result(oracle, scenes):
    """The reference's voxelization depends on its thread count and memory
    budget (sub-block lists are culled with boxes offset one voxel from the
    voxels they feed); the restatement reproduces that dependence."""
    pos, f, col = scenes.displaced_icosphere(4, 1)
    a, _ = oracle.build_mesh(pos, f, 128, 1, 1 << 30, colors=col)
    b, _ = oracle.build_mesh(pos, f, 128, 8, 1 << 30, colors=col)
    c, _ = oracle.build_mesh(pos, f, 128, 8, 5 * 16 ** 3 + 3000, colors=col)
    assert not np.array_equal(a, b) and not np.array_equal(b, c)


def test_icosphere_counts(scenes):
    v, f = scenes.icosphere(3)
    assert v.shape == (642, 3) and f.shape == (1280, 3)
    # every edge shared by exactly two faces
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, cnt = np.unique(e[:, 0] * 10000 + e[:, 1], return_counts=True)
    assert (cnt == 2).all()


@pytest.mark.parametrize("side,threads,mem", [(48, 1, 1 << 30), (48, 8, 1 << 30), (57, 16, 1 << 30),
                                              (64, 6, 62 * 62 * 20),   # slabs of 20 slices, never cleared between
                                              (41, 4, 39 * 39 * 7 + 5)])  # 7 slabs of 6 slices over an odd depth
def test_mesh_to_volume_matches_reference(oracle, reference, scenes, tmp_path, side, threads, mem):
    """PlyLoader::convertToVolume (the builder's --mode 1): the oracle's
    restatement against the reference's own setupBlockProcessing and
    processBlock steps, in one slab and in several."""
    pos, faces, col = scenes.edge_case_mesh(3, side)
    path = str(tmp_path / "m.ply")
    scenes.write_ply(path, pos, faces, colors=col)
    rv = reference.ply_volume(path, side, mem, threads=threads)
    ov = oracle.mesh_to_volume(pos, faces, side, threads, mem, colors=col.astype(np.float32))
    assert rv.shape == ov.shape == tuple(reversed(oracle.mesh_dims(pos, faces, side)))
    assert np.count_nonzero(rv) > 100
    assert np.array_equal(rv, ov)


def test_golden_volumes(oracle, golden):
    """The oracle's convertToVolume against the reference's volumes in the
    committed fixture (one slab twice, four slabs once)."""
    n = 0
    for mesh, side, threads, mem, vol in golden_volumes(golden):
        ov = oracle.mesh_to_volume(mesh["pos"], mesh["faces"], side, threads, mem, colors=mesh["colors"])
        assert np.array_equal(ov, vol), (side, threads, mem)
        n += 1
    assert n == 3
