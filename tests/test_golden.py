"""The oracle restatement against the committed reference outputs (CPU only)."""
import numpy as np

from conftest import golden_builds


def test_dragon_raymarch_matches_reference_outputs(oracle, golden):
    g = golden["dragon"]
    out = oracle.raymarch(g["words"], g["rays"], threads=4)
    hit = out["hit"] == 1
    assert np.array_equal(hit.astype(np.uint8), g["hit"])
    assert np.array_equal(out["t"][hit].view(np.uint32), g["t"][hit].view(np.uint32))
    assert np.array_equal(out["word"][hit], g["word"][hit])
    assert hit.sum() > 500


def test_dragon_lod_matches_reference_outputs(oracle, golden):
    g = golden["dragon"]
    out = oracle.raymarch(g["words"], g["rays"], ray_scale=0.02, threads=4)
    hit = out["hit"] > 0
    assert np.array_equal(hit.astype(np.uint8), g["lod_hit"])
    assert np.array_equal(out["t"][hit].view(np.uint32), g["lod_t"][hit].view(np.uint32))
    assert (out["hit"] == 2).sum() > 100


def test_dragon_known_answers(golden):
    g = golden["dragon"]
    assert g["words"].size == 119887
    assert int(g["words"][0]) == 0x00052323
    assert np.array_equal(g["center"], np.array([0.5, 0.2265625, 0.33203125], np.float32))
    assert bytes(g["file_sha256"]).hex() == "335282669fa1e4e3657926791b3c4c13e6e9d853f9149fe11ce7314462c1a02d"


def test_builds_match_reference(oracle, golden):
    n = 0
    for grid, mem, words, center in golden_builds(golden):
        w, c = oracle.build_dense(grid, mem)
        assert np.array_equal(w, words), grid.shape
        assert np.array_equal(c, center)
        n += 1
    assert n == 12


def test_codec_matches_reference(oracle, golden):
    g = golden["codec"]
    for i in range(0, g["normals"].shape[0], 7):
        assert oracle.compress_material(g["normals"][i], g["shade"][i]) == int(g["packed"][i])
        n, s = oracle.decompress_material(int(g["words"][i]))
        assert np.array_equal(n, g["dec_n"][i]) and np.float32(s) == g["dec_shade"][i]
    for x, y in zip(g["isqrt_x"][:256], g["isqrt_y"][:256]):
        assert np.float32(oracle.inv_sqrt(x)) == y


def test_numpy_codec_matches_reference(scenes, golden):
    g = golden["codec"]
    n = g["normals"]
    w = scenes.compress_material(n[:, 0], n[:, 1], n[:, 2], g["shade"])
    assert np.array_equal(w, g["packed"])
    assert np.array_equal(scenes.inv_sqrt(g["isqrt_x"]), g["isqrt_y"])


def test_viewer_frames_match_reference_outputs(oracle, golden):
    """render_oracle.c's frame against the reference's own renderBatch /
    renderTile (Main.cpp:92-202) frames of the dragon, 1280 x 720 in the
    viewer's 16 strips, full and half size."""
    g, f = golden["dragon"], golden["frames"]
    for rot, pos, half, ref in zip(f["rot"], f["pos"], f["half"], f["frames"]):
        img = oracle.render_frame(g["words"], rot, pos, 1280, 720, 16, 3 if half else 1, threads=4)
        assert np.array_equal(img, ref)
        assert (ref != 0).mean() > 0.1
    assert f["half"].any() and not f["half"].all()
