"""Build recipe for libsvo_gb300.so (sm_103a only).

Every translation unit in csrc/ is compiled by nvcc in parallel, then linked
into a shared library that exports the C ABI of include/svo.h.  Traversal,
shading, codec and scene code rely on -fmad=false (no FMA contraction) and
nvcc's default IEEE division and square root, so their float results match
the reference's x86-64 build bit for bit.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsvo_gb300.so")
SCENES_SRC = os.path.join(HERE, "scenes_gpu.cu")
SCENES_LIB = os.path.join(HERE, "libsvo_scenes.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libsvo_gb300.so")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _needs_rebuild():
    if not os.path.exists(LIB) or not os.path.exists(SCENES_LIB):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(SCENES_LIB))
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    deps += [os.path.abspath(__file__), SCENES_SRC]
    return any(os.path.getmtime(p) > t for p in deps)


def build(force=False, verbose=False):
    """Compile (if stale) and return the path of libsvo_gb300.so."""
    if not force and not _needs_rebuild():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        cmd = [nvcc] + ARCH + COMMON + ["-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc, "-x", "cu"] + ARCH + COMMON + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    srcs = sources() + [SCENES_SRC]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    scene_obj = objs.pop()

    def link(out, objects):
        tmp = out + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objects + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, out)

    link(LIB, objs)
    link(SCENES_LIB, [scene_obj])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
