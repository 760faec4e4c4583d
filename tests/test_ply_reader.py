"""Host-only PLY parsing (svo_ply_parse) against the values PlyLoader reads
through plyfile: binary and ascii, big-endian (plyfile's float -> double ->
float step, then PlyLoader's byte swap), fan triangulation, missing
channels, and the bounds.  CPU only."""
import numpy as np
import pytest


def _be_floats(v):
    g = np.asarray(v, np.float32).astype(">f4").view("<f4")
    with np.errstate(invalid="ignore"):
        g = g.astype(np.float64).astype(np.float32)
    return g.view(">f4").astype(np.float32)


def _fan(faces):
    out = []
    for f in faces:
        for c in range(2, len(f)):
            out.append((f[0], f[c - 1] if c > 2 else f[1], f[c]))
    return np.asarray(out, np.int32).reshape(-1, 3)


def _bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("binary", [True, False])
def test_parse_matches_written_mesh(svo, scenes, tmp_path, binary):
    pos, faces, col = scenes.edge_case_mesh(3, 7)
    nrm = np.random.default_rng(1).normal(size=pos.shape).astype(np.float32)
    path = str(tmp_path / "m.ply")
    scenes.write_ply(path, pos, faces, colors=col, normals=nrm, binary=binary)
    m = svo.ply_parse(path)
    assert _bits_equal(m["positions"], pos)
    assert _bits_equal(m["normals"], nrm)
    assert _bits_equal(m["colors"], col.astype(np.float32))
    assert np.array_equal(m["triangles"], _fan(faces))
    assert _bits_equal(m["lower"], pos.min(0)) and _bits_equal(m["upper"], pos.max(0))


def test_large_binary_mesh_parallel_path(svo, scenes, tmp_path):
    pos, f, col = scenes.displaced_icosphere(6, 2)  # above the parallel threshold
    path = str(tmp_path / "m.ply")
    scenes.write_ply(path, pos, f, colors=col)
    m = svo.ply_parse(path)
    assert _bits_equal(m["positions"], pos) and _bits_equal(m["colors"], col.astype(np.float32))
    assert np.array_equal(m["triangles"], f) and m["normals"] is None
    assert _bits_equal(m["lower"], pos.min(0)) and _bits_equal(m["upper"], pos.max(0))
    # one quad among the triangles: the uniform-triangle path must notice
    faces = [list(map(int, t)) for t in f]
    faces[len(faces) // 2] = faces[len(faces) // 2] + [int(f[0, 0])]
    scenes.write_ply(path, pos, faces, colors=col)
    assert np.array_equal(svo.ply_parse(path)["triangles"], _fan(faces))


def test_big_endian(svo, scenes, tmp_path):
    pos, faces, col = scenes.edge_case_mesh(3, 4)
    path = str(tmp_path / "be.ply")
    scenes.write_ply(path, pos, faces, colors=col, big_endian=True)
    m = svo.ply_parse(path)
    assert _bits_equal(m["positions"], _be_floats(pos))
    assert _bits_equal(m["colors"], col.astype(np.float32).astype(">f4").view("<f4"))
    assert np.array_equal(m["triangles"], _fan(faces))
    # signalling-NaN bit patterns do occur among the misread positions
    raw = pos.astype(">f4").view("<u4")
    snan = ((raw & 0x7F800000) == 0x7F800000) & ((raw & 0x7FFFFF) != 0) & ((raw & 0x400000) == 0)
    assert snan.any()


def test_missing_channels_and_other_elements(svo, tmp_path):
    txt = ("ply\nformat ascii 1.0\ncomment x\nelement camera 1\nproperty float k\n"
           "element vertex 4\nproperty float y\nproperty float x\nproperty float z\nproperty uchar green\n"
           "property int extra\nelement face 2\nproperty uchar flags\nproperty list uchar int vertex_indices\n"
           "end_header\n9\n1 0 0 10 5\n2 1 0 20 6\n3 0 1 30 7\n4 1 1 40 8\n0 4 0 1 2 3\n1 2 1 2\n")
    p = tmp_path / "a.ply"
    p.write_text(txt)
    m = svo.ply_parse(str(p))
    assert np.array_equal(m["positions"], np.array([[0, 1, 0], [1, 2, 0], [0, 3, 1], [1, 4, 1]], np.float32))
    assert np.array_equal(m["colors"][:, 1], [10, 20, 30, 40]) and (m["colors"][:, [0, 2]] == 255).all()
    assert np.array_equal(m["triangles"], [[0, 1, 2], [0, 2, 3]])
