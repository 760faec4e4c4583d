"""The library's traversal step (csrc/svo_device.cuh), compiled for the host
by tests/host_traversal.cpp, against the oracle: both word-index widths, the
table traversal over the breadth-first descriptor table (csrc/octree_table.cuh),
the level-of-detail exit, rays with NaN or infinite components, and an octree
of more than 2^32 words (its untouched pages stay unmapped).  No GPU needed."""
import ctypes
import os
import subprocess

import numpy as np
import pytest
from conftest import golden_builds

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("host_traversal") / "libhost_traversal.so")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC",
                    "-I", os.path.join(ROOT, "sparse-voxel-octrees_gb300", "csrc"),
                    os.path.join(HERE, "host_traversal.cpp"), "-o", so], check=True)
    L = ctypes.CDLL(so)
    L.host_traverse.restype = None
    L.host_traverse.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_float,
                                ctypes.c_int, ctypes.c_uint64] + [ctypes.c_void_p] * 5

    def traverse(words, rays, ray_scale=0.0, wide=False, max_steps=1 << 24):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        n = rays.shape[0]
        out = {"hit": np.zeros(n, np.uint8), "t": np.zeros(n, np.float32), "leaf": np.zeros(n, np.uint64),
               "word": np.zeros(n, np.uint32), "steps": np.zeros(n, np.uint64)}
        L.host_traverse(words.ctypes.data, words.size, rays.ctypes.data, n, float(ray_scale), int(wide), max_steps,
                        out["hit"].ctypes.data, out["t"].ctypes.data, out["leaf"].ctypes.data,
                        out["word"].ctypes.data, out["steps"].ctypes.data)
        assert (out["hit"] != 255).all(), "a ray did not finish"
        assert (out["hit"] != 3).all(), "a ray ended at a bounds check"
        return out

    L.host_build_table.restype = ctypes.c_uint64
    L.host_build_table.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64]
    L.host_traverse_tab.restype = None
    L.host_traverse_tab.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                    ctypes.c_float, ctypes.c_uint64] + [ctypes.c_void_p] * 5

    def table(words):
        words = np.ascontiguousarray(words, dtype=np.uint32)
        tab = np.zeros((words.size, 4), np.uint32)
        n = L.host_build_table(words.ctypes.data, words.size, tab.ctypes.data, words.size)
        return tab[:n] if n else None

    def traverse_tab(words, tab, rays, ray_scale=0.0, max_steps=1 << 24):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        n = rays.shape[0]
        out = {"hit": np.zeros(n, np.uint8), "t": np.zeros(n, np.float32), "leaf": np.zeros(n, np.uint64),
               "word": np.zeros(n, np.uint32), "steps": np.zeros(n, np.uint64)}
        tab = np.ascontiguousarray(tab)
        L.host_traverse_tab(words.ctypes.data, tab.ctypes.data, rays.ctypes.data, n, float(ray_scale), max_steps,
                            out["hit"].ctypes.data, out["t"].ctypes.data, out["leaf"].ctypes.data,
                            out["word"].ctypes.data, out["steps"].ctypes.data)
        assert (out["hit"] != 255).all(), "a ray did not finish"
        return out

    traverse.table = table
    traverse.tab = traverse_tab
    return traverse


def _assert_same(res, ref, leaf=True):
    assert np.array_equal(res["hit"], ref["hit"])
    assert np.array_equal(res["t"].view(np.uint32), ref["t"].view(np.uint32))
    assert np.array_equal(res["word"], ref["word"])
    if leaf:
        h = ref["hit"] == 1
        assert np.array_equal(res["leaf"][h], ref["leaf"][h].astype(np.uint64))


def _nan_rays():
    nan, inf = np.float32(np.nan), np.float32(np.inf)
    rows = [
        [nan, nan, nan, 0.0, 0.0, 1.0],      # NaN origin
        [1.5, 1.5, -1.0, nan, nan, nan],     # a normalised zero vector
        [1.5, 1.5, -1.0, nan, 0.0, 1.0],     # NaN on one axis of the direction
        [1.5, nan, -1.0, 0.0, 0.0, 1.0],     # NaN on one axis of the origin
        [inf, 1.5, 1.5, -inf, 0.0, 0.0],     # infinite origin along an infinite direction
        [inf, 1.5, 1.5, -1.0, 0.0, 0.0],     # infinite origin, finite direction: an ordinary ray
        [1.5, 1.5, -1.0, 0.0, 0.0, inf],     # infinite direction: an ordinary ray
    ]
    return np.array(rows, np.float32)


def test_golden_rays_both_widths(host, oracle, golden):
    g = golden["dragon"]
    ref = oracle.raymarch(g["words"], g["rays"], threads=4)
    # the reference's own outputs, then the oracle's
    for wide in (False, True):
        res = host(g["words"], g["rays"], wide=wide)
        hit = g["hit"] == 1
        assert np.array_equal((res["hit"] == 1).astype(np.uint8), g["hit"])
        assert np.array_equal(res["t"][hit].view(np.uint32), g["t"][hit].view(np.uint32))
        assert np.array_equal(res["word"][hit], g["word"][hit])
        _assert_same(res, ref)
        lod = host(g["words"], g["rays"], ray_scale=0.02, wide=wide)
        _assert_same(lod, oracle.raymarch(g["words"], g["rays"], ray_scale=0.02, threads=4), leaf=False)


def test_random_rays_far_pointer_tree(host, oracle, scenes):
    grid = scenes.random_grid((64, 64, 64), 0.5, 3)
    words, _ = oracle.build_dense(grid)
    rays = scenes.random_rays(50_000, 6)
    ref = oracle.raymarch(words, rays, threads=4)
    for wide in (False, True):
        _assert_same(host(words, rays, wide=wide), ref)


def test_nan_rays_end_as_misses(host, oracle, golden):
    g = golden["dragon"]
    rays = np.concatenate([_nan_rays(), g["rays"][:64]])
    ref = oracle.raymarch(g["words"], rays, loads=True, threads=1)
    for wide in (False, True):
        res = host(g["words"], rays, wide=wide, max_steps=1 << 16)
        _assert_same(res, ref)
    res = host(g["words"], rays[:5], max_steps=4)
    assert (res["hit"] == 0).all() and (res["steps"] == 1).all()  # one pass, out of the root
    assert (ref["loads"][:5] == 1).all() and (res["t"] == np.float32(np.inf)).all()


def _shifted(words, gap):
    n = 2 + gap + (words.size - 1)
    big = np.zeros(n, np.uint32)  # calloc'd: pages never touched stay unmapped
    off = 2 + gap
    big[0] = (int(words[0]) & 0x1FFFF) | 0x20000 | ((off >> 32) << 18)
    big[1] = off & 0xFFFFFFFF
    big[off:] = words[1:]
    return big


@pytest.mark.parametrize("gap", [(1 << 32) + 5, (1 << 32) - 5000])
def test_octree_above_2e32_words(host, oracle, scenes, gap):
    grid = scenes.random_grid((32, 32, 32), 0.5, 4)
    words, _ = oracle.build_dense(grid)
    assert words.size > 10000
    rays = scenes.random_rays(20_000, 7)
    ref = oracle.raymarch(words, rays, threads=4)
    big = _shifted(words, gap)
    assert big.size > 0xFFFFFFFF
    res = host(big, rays, wide=True)
    _assert_same(res, ref, leaf=False)
    h = ref["hit"] == 1
    assert h.sum() > 1000
    # leaf indices move by the gap plus the root's far word
    assert np.array_equal(res["leaf"][h], ref["leaf"][h].astype(np.uint64) + np.uint64(gap + 1))
    assert (res["leaf"][h] > 0xFFFFFFFF).any()
    # the oracle (64-bit offsets, as the reference) reads the shifted words the same way
    _assert_same(oracle.raymarch(big, rays, threads=4), ref, leaf=False)


def _table_cases(golden, oracle, scenes):
    g = golden["dragon"]
    yield g["words"]
    yield oracle.build_dense(scenes.random_grid((64, 64, 64), 0.5, 3))[0]  # far words
    yield oracle.build_dense(scenes.sphere_scene(128, 24, 0))[0]
    for grid, mem, words, center in golden_builds(golden):
        yield words


def test_table_traversal_matches_oracle(host, oracle, golden, scenes):
    rays = np.concatenate([scenes.random_rays(30_000, 9), _nan_rays(), golden["dragon"]["rays"][:2000]])
    for words in _table_cases(golden, oracle, scenes):
        tab = host.table(words)
        assert tab is not None
        order = _bfs_order(words)
        assert tab.shape[0] == order.size
        assert np.array_equal(tab[:, 0], words[order])
        _assert_same(host.tab(words, tab, rays), oracle.raymarch(words, rays, threads=4))
        lod = host.tab(words, tab, rays, ray_scale=0.02)
        _assert_same(lod, oracle.raymarch(words, rays, ray_scale=0.02, threads=4), leaf=False)


def _bfs_order(words):
    """Word indices of the nodes reachable from the root, breadth first."""
    out, level = [], [0]
    while level:
        out.extend(level)
        nxt = []
        for d in level:
            w = int(words[d])
            valid, nonleaf = (w >> 8) & 0xFF, w & 0xFF
            if not valid:
                continue
            off = w >> 18
            if w & 0x20000:
                off = (off << 32) | int(words[d + 1])
            stride = 2 if w & 0x10000 else 1
            nxt.extend(d + off + j * stride for j in range(bin(nonleaf).count("1")))
        level = nxt
    return np.array(out, np.int64)


def test_table_refused_for_unsafe_trees(host):
    # child block past the end, a zero offset, a non-leaf bit outside the
    # valid mask, and internal children below level 21 each leave no table
    assert host.table(np.array([(0x3FFF << 18) | (0xFF << 8) | 0xFF], np.uint32)) is None
    assert host.table(np.array([(0xFF << 8) | 0xFF] + [0] * 8, np.uint32)) is None
    assert host.table(np.array([(1 << 18) | (0x01 << 8) | 0x02, 0], np.uint32)) is None
    chain = [(1 << 18) | (0x80 << 8) | 0x80] * 23 + [0]  # 23 nested single internal children
    assert host.table(np.array(chain, np.uint32)) is None
    assert host.table(np.array(chain[1:], np.uint32)) is not None  # 22 nested is fine
