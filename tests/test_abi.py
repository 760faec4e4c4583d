"""The C-ABI library without a GPU: it loads, exports every declared entry
point, and its host-only paths (.oct codec, argument checks) behave."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import pyoracle
from conftest import ROOT


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(svo_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(svo):
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", svo.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (svo_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(svo.lib, n)


def test_version_and_errors(svo):
    assert svo.lib.svo_version() >= 100
    h = ctypes.c_void_p()
    rc = svo.lib.svo_octree_load(b"/nonexistent/file.oct", ctypes.byref(h))
    assert rc == svo.SVO_ERR_IO
    assert b"cannot open" in svo.lib.svo_last_error()
    assert svo.lib.svo_octree_load(None, ctypes.byref(h)) == svo.SVO_ERR_INVALID
    assert svo.lib.svo_trace(None, None, 0, 0.0, None, None, None) == svo.SVO_ERR_INVALID
    assert svo.lib.svo_octree_build_dense(None, 4, 4, 4, 1 << 30, 0, None, ctypes.byref(h)) == svo.SVO_ERR_INVALID


def test_build_argument_checks_before_device_use(svo):
    h = ctypes.c_void_p()
    g = np.ones(1, np.uint32)
    # virtual side 1: the reference would recurse forever
    assert svo.lib.svo_octree_build_dense(g.ctypes.data_as(ctypes.c_void_p), 1, 1, 1, 1 << 30, 0, None,
                                          ctypes.byref(h)) == svo.SVO_ERR_INVALID
    # budget too small for any cache block: the reference exits the process
    g = np.ones(64 * 64 * 64, np.uint32)
    assert svo.lib.svo_octree_build_dense(g.ctypes.data_as(ctypes.c_void_p), 64, 64, 64, 100, 0, None,
                                          ctypes.byref(h)) == svo.SVO_ERR_MEMORY


def test_ply_errors_before_device_use(svo, scenes, tmp_path):
    h = ctypes.c_void_p()
    assert svo.lib.svo_mesh_load_ply(str(tmp_path / "missing.ply").encode(), ctypes.byref(h)) == svo.SVO_ERR_IO
    bad = tmp_path / "bad.ply"
    bad.write_bytes(b"ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\nend_header\n0\n")
    assert svo.lib.svo_mesh_load_ply(str(bad).encode(), ctypes.byref(h)) == svo.SVO_ERR_FORMAT
    assert b"triangles and vertices" in svo.lib.svo_last_error()
    trunc = tmp_path / "trunc.ply"
    pos, faces, col = scenes.edge_case_mesh(1, 1)
    scenes.write_ply(str(trunc), pos, faces, colors=col)
    trunc.write_bytes(trunc.read_bytes()[:-7])
    assert svo.lib.svo_mesh_load_ply(str(trunc).encode(), ctypes.byref(h)) == svo.SVO_ERR_FORMAT
    with pytest.raises(svo.SvoError) as e:  # index past the vertex array
        svo.PlyLoader.from_arrays(pos, faces + [[0, 1, pos.shape[0]]])
    assert e.value.code == svo.SVO_ERR_FORMAT
    nan = pos.copy()
    nan[3, 1] = np.nan
    with pytest.raises(svo.SvoError) as e:
        svo.PlyLoader.from_arrays(nan, faces)
    assert e.value.code == svo.SVO_ERR_FORMAT


def test_oct_read_reference_dragon_fixture_roundtrip(svo, oracle, golden, tmp_path):
    g = golden["dragon"]
    p = str(tmp_path / "d.oct")
    svo.oct_write(p, g["words"], g["center"])
    w, c = svo.oct_read(p)
    assert np.array_equal(w, g["words"]) and np.array_equal(c, g["center"])
    # the oracle's independent decoder reads our encoder's output
    w2, c2 = oracle.oct_decode(open(p, "rb").read())
    assert np.array_equal(w2, g["words"])
    assert os.path.getsize(p) < g["words"].nbytes


def test_oct_read_shipped_dragon(svo):
    path = os.path.join(pyoracle.REF_SRC, "models", "XYZRGB-Dragon.oct")
    if not os.path.exists(path):
        pytest.skip("reference sources not present")
    w, c = svo.oct_read(path)
    assert w.size == 119887 and int(w[0]) == 0x00052323


def test_oct_multiblock_interop_with_reference(svo, reference, tmp_path):
    # > 64 MiB of payload: several LZ4 blocks, where the reference's streaming
    # compressor may reference the previous block.
    rng = np.random.default_rng(0)
    n = 20_000_000
    words = (rng.integers(0, 64, n, dtype=np.uint32) * np.uint32(0x01010101))
    center = np.array([0.5, 0.25, 0.125], np.float32)
    ours = str(tmp_path / "ours.oct")
    svo.oct_write(ours, words, center)
    tree = reference.load(ours)  # the reference's loader reads our encoder's blocks
    rw, rc = reference.words(tree)
    assert np.array_equal(rw, words) and np.array_equal(rc, center)
    theirs = str(tmp_path / "theirs.oct")
    reference.save(tree, theirs)  # and we read the reference's streaming blocks
    reference.free(tree)
    w2, c2 = svo.oct_read(theirs)
    assert np.array_equal(w2, words) and np.array_equal(c2, center)


@pytest.mark.parametrize("cut", [5, 19, 27, 200])
def test_oct_read_truncated(svo, golden, tmp_path, cut):
    g = golden["dragon"]
    p = str(tmp_path / "d.oct")
    svo.oct_write(p, g["words"], g["center"])
    data = open(p, "rb").read()
    open(p, "wb").write(data[:cut])
    with pytest.raises(svo.SvoError) as e:
        svo.oct_read(p)
    assert e.value.code == svo.SVO_ERR_FORMAT


def test_oct_read_corrupt(svo, golden, tmp_path):
    g = golden["dragon"]
    p = str(tmp_path / "d.oct")
    svo.oct_write(p, g["words"], g["center"])
    data = bytearray(open(p, "rb").read())
    data[28:36] = b"\xff" * 8  # first token and literals
    data[40:48] = b"\xff" * 8
    open(p, "wb").write(bytes(data))
    with pytest.raises(svo.SvoError):
        svo.oct_read(p)


def test_struct_layouts_match_header(svo, tmp_path):
    """The ctypes mirrors of svo_trace_out, svo_view and svo_trace_config have
    the C header's size and field offsets (compiled here with the system C
    compiler, which follows the same ABI as the library's host code)."""
    mirrors = {"svo_trace_out": svo.TraceOut, "svo_view": svo.View, "svo_trace_config": svo.TraceConfig}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "svo.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, field, cname, field))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {(ln.split()[0], ln.split()[1]): int(ln.split()[2]) for ln in out if ln.strip()}
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)
