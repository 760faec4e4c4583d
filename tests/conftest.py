import importlib.util
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "sparse-voxel-octrees_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ORACLE_DIR)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


def load_package():
    """Import the package directory (its name has dashes) as `svo_gb300`."""
    if "svo_gb300" in sys.modules:
        return sys.modules["svo_gb300"]
    lib = os.path.join(PKG_DIR, "libsvo_gb300.so")
    spec_b = importlib.util.spec_from_file_location("svo_gb300_build", os.path.join(PKG_DIR, "build_lib.py"))
    b = importlib.util.module_from_spec(spec_b)
    spec_b.loader.exec_module(b)
    b.build()
    assert os.path.exists(lib)
    spec = importlib.util.spec_from_file_location("svo_gb300", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["svo_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def load_scenes():
    load_package()
    import svo_gb300.scenes as scenes  # noqa: E402
    return scenes


@pytest.fixture(scope="session")
def svo():
    return load_package()


@pytest.fixture(scope="session")
def scenes():
    return load_scenes()


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"], check=True)  # make decides staleness
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def reference():
    import pyoracle
    if not os.path.exists(pyoracle.REF_SO):
        if not os.path.isdir(os.path.join(pyoracle.REF_SRC, "src")):
            pytest.skip("reference sources not present on this machine")
        subprocess.run(["make", "-s", "-j8", "-C", ORACLE_DIR, "ref", "REF=" + pyoracle.REF_SRC], check=True)
    r = pyoracle.Reference()
    r.start_threads(4)
    return r


@pytest.fixture(scope="session")
def golden():
    return {
        "dragon": np.load(os.path.join(GOLDEN, "dragon.npz")),
        "builds": np.load(os.path.join(GOLDEN, "builds.npz")),
        "codec": np.load(os.path.join(GOLDEN, "codec.npz")),
        "ply": np.load(os.path.join(GOLDEN, "ply.npz")),
        "volumes": np.load(os.path.join(GOLDEN, "volumes.npz")),
        "frames": np.load(os.path.join(GOLDEN, "frames.npz")),
    }


def golden_builds(g):
    """Yields (grid (d,h,w), mem, words, center) for each golden build case."""
    b = g["builds"]
    go, wo = b["grid_offsets"], b["word_offsets"]
    for i, (w, h, d, mem) in enumerate(b["meta"]):
        grid = b["grids"][go[i]:go[i + 1]].reshape(int(d), int(h), int(w))
        yield grid, int(mem), b["words"][wo[i]:wo[i + 1]], b["centers"][i]


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for gpu-marked tests")
    return torch


def golden_ply(golden):
    """Yields (mesh, side, threads, mem, words, center) for ply.npz; mesh
    holds pos, faces (index lists), colors (float) and normals (or None)."""
    g = golden["ply"]
    flat = g["faces"].tolist()
    faces, i = [], 0
    while i < len(flat):
        faces.append(flat[i + 1:i + 1 + flat[i]])
        i += 1 + flat[i]
    wo = g["word_offsets"]
    for k, (side, threads, mem, with_n, binary) in enumerate(g["meta"].tolist()):
        mesh = {"pos": g["pos"], "faces": faces, "colors": g["colors"].astype(np.float32),
                "colors_u8": g["colors"], "normals": g["normals"] if with_n else None, "binary": bool(binary)}
        yield mesh, int(side), int(threads), int(mem), g["words"][wo[k]:wo[k + 1]], g["centers"][k]


def golden_volumes(golden):
    """Yields (mesh, side, threads, mem, volume (d, h, w)) for volumes.npz,
    whose mesh is ply.npz's (colours as written to its PLY)."""
    mesh = next(golden_ply(golden))[0]
    g = golden["volumes"]
    off = g["offsets"]
    for k, (side, threads, mem, w, h, d) in enumerate(g["meta"].tolist()):
        yield mesh, int(side), int(threads), int(mem), g["words"][off[k]:off[k + 1]].reshape(int(d), int(h), int(w))
