"""ctypes bindings for the test oracles.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
(as the checker) and by bench.py's CPU-baseline and reference legs.

* ``Oracle``   — liboracle.so, the C restatement of the reference's hot path
                 (svo_oracle.c).  Built by ``make -C oracle``; builds anywhere.
* ``Reference`` — oracle/_ref/libsvo_ref.so, the reference's own sources
                 compiled in place (``make -C oracle ref``).  Exists only where
                 the reference sources are present.
"""
import ctypes
import multiprocessing
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsvo_ref.so")
REF_SRC = os.environ.get("SVO_REFERENCE_DIR", "/root/reference")

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p


def _ptr(a, t):
    if a is None:
        return None
    return a.ctypes.data_as(t)


def build_oracle(with_reference=None):
    """Compile liboracle.so (and, when the reference sources exist, _ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if with_reference is None:
        with_reference = os.path.isdir(os.path.join(REF_SRC, "src"))
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, "-j8", "ref", "REF=" + REF_SRC], check=True)


class Oracle:
    """The C restatement (svo_oracle.c)."""

    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build_oracle(with_reference=False)
        L = ctypes.CDLL(path)
        self.L = L
        L.svo_oracle_inv_sqrt.restype = ctypes.c_float
        L.svo_oracle_inv_sqrt.argtypes = [ctypes.c_float]
        L.svo_oracle_compress_material.restype = ctypes.c_uint32
        L.svo_oracle_compress_material.argtypes = [_f32p, ctypes.c_float]
        L.svo_oracle_decompress_material.argtypes = [ctypes.c_uint32, _f32p, _f32p]
        L.svo_oracle_shade.restype = ctypes.c_float
        L.svo_oracle_shade.argtypes = [ctypes.c_uint32, _f32p, _f32p]
        L.svo_oracle_raymarch_batch.argtypes = [_u32p, ctypes.c_uint64, _f32p, ctypes.c_uint64,
                                                ctypes.c_float, _f32p, _u8p, _f32p, _u32p, _u32p,
                                                _f32p, _u32p, ctypes.c_int]
        L.svo_oracle_build_dense.restype = ctypes.c_int
        L.svo_oracle_build_dense.argtypes = [_u32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_uint64, ctypes.POINTER(_u32p), _u64p, _f32p]
        L.svo_oracle_cache_block.restype = ctypes.c_uint64
        L.svo_oracle_cache_block.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_uint64, ctypes.c_uint64]
        L.svo_oracle_oct_decode.restype = ctypes.c_int
        L.svo_oracle_oct_decode.argtypes = [_u8p, ctypes.c_uint64, ctypes.POINTER(_u32p), _u64p, _f32p]
        L.svo_oracle_free.argtypes = [_vp]
        L.svo_oracle_scene_voxels.restype = ctypes.c_int
        L.svo_oracle_scene_voxels.argtypes = [ctypes.c_int, _f32p, ctypes.c_float, ctypes.POINTER(ctypes.c_int),
                                              _f32p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_u64p),
                                              ctypes.POINTER(_u32p), _u64p]
        L.svo_oracle_mesh_create.restype = _vp
        L.svo_oracle_mesh_create.argtypes = [_f32p, _f32p, _f32p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                             ctypes.c_int]
        L.svo_oracle_mesh_destroy.argtypes = [_vp]
        L.svo_oracle_mesh_num_tris.restype = ctypes.c_int
        L.svo_oracle_mesh_num_tris.argtypes = [_vp]
        L.svo_oracle_mesh_dims.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.svo_oracle_build_mesh.restype = ctypes.c_int
        L.svo_oracle_build_mesh.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(_u32p),
                                            _u64p, _f32p]
        L.svo_oracle_mesh_to_volume.restype = ctypes.c_int
        L.svo_oracle_mesh_to_volume.argtypes = [_vp, ctypes.c_int, ctypes.c_uint64, ctypes.c_int, _u32p]
        L.svo_oracle_render_frame.restype = ctypes.c_int
        L.svo_oracle_render_frame.argtypes = [_u32p, ctypes.c_uint64, _f32p, _f32p, ctypes.c_float, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_int, _u32p, ctypes.c_int]
        L.svo_oracle_plane_dist.restype = ctypes.c_float
        L.svo_oracle_tri_box_overlap.restype = ctypes.c_int
        L.svo_oracle_tri_box_overlap.argtypes = [_f32p, _f32p, _f32p]
        L.svo_oracle_build_sorted.restype = ctypes.c_int
        L.svo_oracle_build_sorted.argtypes = [_u64p, _u32p, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(_u32p),
                                              _u64p]

    # -- codec / shading
    def inv_sqrt(self, x):
        return self.L.svo_oracle_inv_sqrt(float(x))

    def compress_material(self, n, shade):
        a = np.ascontiguousarray(n, dtype=np.float32)
        return int(self.L.svo_oracle_compress_material(_ptr(a, _f32p), float(shade)))

    def decompress_material(self, word):
        n = np.zeros(3, np.float32)
        s = ctypes.c_float()
        self.L.svo_oracle_decompress_material(int(word), _ptr(n, _f32p), ctypes.byref(s))
        return n, s.value

    def shade(self, word, d, light):
        d = np.ascontiguousarray(d, dtype=np.float32)
        light = np.ascontiguousarray(light, dtype=np.float32)
        return self.L.svo_oracle_shade(int(word), _ptr(d, _f32p), _ptr(light, _f32p))

    # -- raymarch
    RAY_OUTPUTS = ("hit", "t", "leaf", "word", "grey")

    def raymarch(self, words, rays, ray_scale=0.0, light=(0.0, 0.0, 1.0), threads=1, loads=False,
                 outputs=RAY_OUTPUTS):
        """rays: (R, 6) float32.  Returns dict of the requested outputs among
        hit (u8), t, leaf, word, grey[, loads]; outputs not asked for are not
        computed (grey is the shade of a hit)."""
        words = np.ascontiguousarray(words, dtype=np.uint32)
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        light = np.ascontiguousarray(light, dtype=np.float32)
        R = rays.shape[0]
        types = {"hit": np.uint8, "t": np.float32, "leaf": np.uint32, "word": np.uint32, "grey": np.float32}
        out = {k: np.zeros(R, types[k]) for k in outputs}
        ld = np.zeros(R, np.uint32) if loads else None
        self.L.svo_oracle_raymarch_batch(_ptr(words, _u32p), words.size, _ptr(rays, _f32p), R,
                                         float(ray_scale), _ptr(light, _f32p),
                                         _ptr(out.get("hit"), _u8p), _ptr(out.get("t"), _f32p),
                                         _ptr(out.get("leaf"), _u32p), _ptr(out.get("word"), _u32p),
                                         _ptr(out.get("grey"), _f32p), _ptr(ld, _u32p), int(threads))
        if loads:
            out["loads"] = ld
        return out

    # -- build
    def build_dense(self, grid, mem=1 << 30):
        """grid: (d, h, w) uint32 array (x fastest).  Returns (words, center)."""
        grid = np.ascontiguousarray(grid, dtype=np.uint32)
        d, h, w = grid.shape
        p = _u32p()
        n = ctypes.c_uint64()
        c = np.zeros(3, np.float32)
        rc = self.L.svo_oracle_build_dense(_ptr(grid, _u32p), w, h, d, int(mem), ctypes.byref(p),
                                           ctypes.byref(n), _ptr(c, _f32p))
        if rc != 0:
            raise RuntimeError("svo_oracle_build_dense failed: %d" % rc)
        words = np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0, np.uint32)
        self.L.svo_oracle_free(ctypes.cast(p, _vp))
        return words, c

    def scene_voxels(self, side, heights=None, boxes=None, params=None, thickness=2.0, threads=None):
        """CPU scene generation (scene_build.c): Morton-ordered (keys, payload)."""
        threads = threads or os.cpu_count() or 1
        hp = None
        if heights is not None:
            heights = np.ascontiguousarray(heights, dtype=np.float32)
            hp = _ptr(heights, _f32p)
        n = 0 if boxes is None else len(boxes)
        bx = np.ascontiguousarray(np.asarray(boxes if n else np.zeros((1, 6)), dtype=np.int32))
        pr = np.ascontiguousarray(np.asarray(params if n else np.zeros((1, 4)), dtype=np.float32))
        kp, pp, nv = _u64p(), _u32p(), ctypes.c_uint64()
        rc = self.L.svo_oracle_scene_voxels(int(side), hp, float(thickness), bx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                            _ptr(pr, _f32p), n, int(threads), ctypes.byref(kp), ctypes.byref(pp),
                                            ctypes.byref(nv))
        if rc != 0:
            raise RuntimeError("svo_oracle_scene_voxels failed: %d" % rc)
        N = nv.value
        keys = np.ctypeslib.as_array(kp, shape=(N,)).copy() if N else np.zeros(0, np.uint64)
        pay = np.ctypeslib.as_array(pp, shape=(N,)).copy() if N else np.zeros(0, np.uint32)
        self.L.svo_oracle_free(ctypes.cast(kp, _vp))
        self.L.svo_oracle_free(ctypes.cast(pp, _vp))
        return keys, pay

    def build_sorted(self, keys, payload, log_side):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        payload = np.ascontiguousarray(payload, dtype=np.uint32)
        p, n = _u32p(), ctypes.c_uint64()
        rc = self.L.svo_oracle_build_sorted(_ptr(keys, _u64p), _ptr(payload, _u32p), keys.size, int(log_side),
                                            ctypes.byref(p), ctypes.byref(n))
        if rc != 0:
            raise RuntimeError("svo_oracle_build_sorted failed: %d" % rc)
        words = np.ctypeslib.as_array(p, shape=(n.value,)).copy()
        self.L.svo_oracle_free(ctypes.cast(p, _vp))
        return words

    def build_mesh(self, pos, faces, side, threads, mem=1 << 30, normals=None, colors=None):
        """VoxelData(PlyLoader*, side, mem) + VoxelOctree for a parsed mesh:
        pos (V, 3) float32, faces (F, k) int or a list of index lists,
        optional per-vertex normals and colours (float, colour default 255).
        `threads` is the reference's thread-pool size, which selects the
        sub-block partition.  Returns (words, center)."""
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        col = None if colors is None else np.ascontiguousarray(colors, dtype=np.float32).reshape(-1, 3)
        flat = flatten_faces(faces)
        n_faces = len(faces)
        m = self.L.svo_oracle_mesh_create(_ptr(pos, _f32p), _ptr(nrm, _f32p), _ptr(col, _f32p), pos.shape[0],
                                          flat.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n_faces)
        if not m:
            raise MemoryError("svo_oracle_mesh_create")
        try:
            p, n = _u32p(), ctypes.c_uint64()
            c = np.zeros(3, np.float32)
            rc = self.L.svo_oracle_build_mesh(m, int(side), int(threads), int(mem), ctypes.byref(p), ctypes.byref(n),
                                              _ptr(c, _f32p))
            if rc != 0:
                raise RuntimeError("svo_oracle_build_mesh failed: %d" % rc)
            words = np.ctypeslib.as_array(p, shape=(n.value,)).copy()
            self.L.svo_oracle_free(ctypes.cast(p, _vp))
            return words, c
        finally:
            self.L.svo_oracle_mesh_destroy(m)

    def mesh_to_volume(self, pos, faces, side, threads, mem=1 << 30, normals=None, colors=None):
        """PlyLoader::convertToVolume (the builder's --mode 1) for a parsed
        mesh: the (d, h, w) uint32 volume it writes after its header."""
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        col = None if colors is None else np.ascontiguousarray(colors, dtype=np.float32).reshape(-1, 3)
        flat = flatten_faces(faces)
        m = self.L.svo_oracle_mesh_create(_ptr(pos, _f32p), _ptr(nrm, _f32p), _ptr(col, _f32p), pos.shape[0],
                                          flat.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(faces))
        if not m:
            raise MemoryError("svo_oracle_mesh_create")
        try:
            dims = (ctypes.c_int * 3)()
            self.L.svo_oracle_mesh_dims(m, int(side), dims)
            w, h, d = dims
            out = np.zeros((d, h, w), np.uint32)
            rc = self.L.svo_oracle_mesh_to_volume(m, int(side), int(mem), int(threads), _ptr(out, _u32p))
            if rc != 0:
                raise RuntimeError("svo_oracle_mesh_to_volume failed: %d" % rc)
            return out
        finally:
            self.L.svo_oracle_mesh_destroy(m)

    def render_frame(self, words, rot, pos, W=1280, H=720, n_strips=16, pixel_stride=1, threads=None):
        """The viewer's frame (render_oracle.c): (H, W) uint32 RGBA8."""
        words = np.ascontiguousarray(words, dtype=np.uint32)
        rot = np.ascontiguousarray(rot, dtype=np.float32).reshape(9)
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(3)
        out = np.zeros((H, W), np.uint32)
        rc = self.L.svo_oracle_render_frame(_ptr(words, _u32p), words.size, _ptr(rot, _f32p), _ptr(pos, _f32p),
                                            self.L.svo_oracle_plane_dist(), W, H, n_strips, pixel_stride,
                                            _ptr(out, _u32p), threads or os.cpu_count() or 1)
        if rc:
            raise RuntimeError("svo_oracle_render_frame failed: %d" % rc)
        return out

    def mesh_dims(self, pos, faces, side):
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        flat = flatten_faces(faces)
        m = self.L.svo_oracle_mesh_create(_ptr(pos, _f32p), None, None, pos.shape[0],
                                          flat.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(faces))
        dims = (ctypes.c_int * 3)()
        self.L.svo_oracle_mesh_dims(m, int(side), dims)
        self.L.svo_oracle_mesh_destroy(m)
        return tuple(dims)

    def tri_box_overlap(self, center, half, verts):
        c = np.ascontiguousarray(center, dtype=np.float32)
        h = np.ascontiguousarray(half, dtype=np.float32)
        v = np.ascontiguousarray(verts, dtype=np.float32).reshape(9)
        return int(self.L.svo_oracle_tri_box_overlap(_ptr(c, _f32p), _ptr(h, _f32p), _ptr(v, _f32p)))

    def cache_block(self, w, h, d, mem, cell_cost=4):
        return int(self.L.svo_oracle_cache_block(w, h, d, int(mem), int(cell_cost)))

    def oct_decode(self, data):
        buf = np.frombuffer(data, dtype=np.uint8)
        p = _u32p()
        n = ctypes.c_uint64()
        c = np.zeros(3, np.float32)
        rc = self.L.svo_oracle_oct_decode(_ptr(buf, _u8p), buf.size, ctypes.byref(p), ctypes.byref(n),
                                          _ptr(c, _f32p))
        if rc != 0:
            raise ValueError("corrupt .oct stream (%d)" % rc)
        words = np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0, np.uint32)
        self.L.svo_oracle_free(ctypes.cast(p, _vp))
        return words, c


def flatten_faces(faces):
    """[count, idx...] runs as int32 (the layout svo_oracle_mesh_create takes)."""
    if isinstance(faces, np.ndarray) and faces.ndim == 2:
        f = np.asarray(faces, dtype=np.int32)
        return np.ascontiguousarray(np.concatenate([np.full((f.shape[0], 1), f.shape[1], np.int32), f], 1).ravel())
    out = []
    for f in faces:
        out.append(len(f))
        out.extend(int(i) for i in f)
    return np.asarray(out if out else [0], dtype=np.int32)


def _ref_worker_main(conn, path, threads):
    """Child process: runs reference builds sent over `conn` (the
    reference's progress output goes to /dev/null)."""
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    ref = Reference(path, isolated=False)
    ref.start_threads(threads)
    while True:
        try:
            msg = conn.recv()
        except (EOFError, OSError):  # the parent went away
            return
        if msg is None:
            return
        name, args = msg
        try:
            conn.send(("ok", getattr(ref, name)(*args)))
        except Exception as e:  # report, keep serving
            conn.send(("err", repr(e)))


class _RefBuildWorker:
    """Runs the reference's VoxelOctree(VoxelData*) builds in a spawned child.

    The reference's TaskGroup (thread/TaskGroup.hpp) sets its done flag and
    notifies its condition variable without holding the waiter's mutex, so a
    notification can land between the waiter's predicate check and its wait
    and be lost; VoxelData's enqueue()->wait() calls then block forever now
    and then.  A build that does not answer within `timeout` seconds is
    retried in a fresh process."""

    def __init__(self, path, threads, timeout=5.0, retries=6):
        self.path, self.threads, self.timeout, self.retries = path, threads, timeout, retries
        self.ctx = multiprocessing.get_context("spawn")
        self.proc = None

    def _start(self):
        self.conn, child = self.ctx.Pipe()
        self.proc = self.ctx.Process(target=_ref_worker_main, args=(child, self.path, self.threads), daemon=True)
        self.proc.start()

    def _stop(self):
        if self.proc is not None:
            self.proc.kill()
            self.proc.join(5)
            self.proc = None

    def call(self, name, *args, timeout=None):
        for _ in range(self.retries):
            if self.proc is None or not self.proc.is_alive():
                self._start()
            self.conn.send((name, args))
            if self.conn.poll(timeout or self.timeout):
                status, value = self.conn.recv()
                if status == "err":
                    raise RuntimeError(value)
                return value
            self._stop()  # lost wakeup in the reference's thread pool: retry in a new process
        raise RuntimeError("reference build did not finish after %d attempts" % self.retries)


class Reference:
    """The reference's own code, compiled in place from its sources.

    Builds (whose VoxelData waits on the reference's thread pool) run in a
    spawned worker process with a timeout; loads, saves and raymarches run
    in-process."""

    _threads_started = None

    def __init__(self, path=REF_SO, isolated=True):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.path = path
        self._isolated = isolated
        self._workers = {}
        self._worker = self._worker_for(4)
        L = ctypes.CDLL(path)
        self.L = L
        L.ref_start_threads.argtypes = [ctypes.c_int]
        L.ref_build_voxel_file.restype = _vp
        L.ref_build_voxel_file.argtypes = [ctypes.c_char_p, ctypes.c_uint64]
        L.ref_build_ply.restype = _vp
        L.ref_build_ply.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_uint64]
        L.ref_ply_to_voxel_file.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_uint64]
        L.ref_ply_volume.restype = ctypes.c_int
        L.ref_ply_volume.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int),
                                     _u32p]
        L.ref_load.restype = _vp
        L.ref_load.argtypes = [ctypes.c_char_p]
        L.ref_save.argtypes = [_vp, ctypes.c_char_p]
        L.ref_free.argtypes = [_vp]
        L.ref_num_words.restype = ctypes.c_uint64
        L.ref_num_words.argtypes = [_vp]
        L.ref_words.restype = _vp
        L.ref_words.argtypes = [_vp]
        L.ref_center.argtypes = [_vp, _f32p]
        L.ref_raymarch.argtypes = [_vp, _f32p, ctypes.c_uint64, ctypes.c_float, _u8p, _f32p, _u32p,
                                   ctypes.c_int]
        L.ref_compress_material.restype = ctypes.c_uint32
        L.ref_compress_material.argtypes = [_f32p, ctypes.c_float]
        L.ref_decompress_material.argtypes = [ctypes.c_uint32, _f32p, _f32p]
        L.ref_inv_sqrt.restype = ctypes.c_float
        L.ref_inv_sqrt.argtypes = [ctypes.c_float]
        L.ref_tri_box_overlap.restype = ctypes.c_int
        L.ref_tri_box_overlap.argtypes = [_f32p, _f32p, _f32p]
        L.ref_render_frame.restype = ctypes.c_int
        L.ref_render_frame.argtypes = [_vp, _f32p, _f32p, ctypes.c_int, _u32p]

    def _worker_for(self, threads):
        """The spawned build worker whose reference thread pool has `threads`
        threads (None in-process)."""
        if not self._isolated:
            return None
        if threads not in self._workers:
            self._workers[threads] = _RefBuildWorker(self.path, threads)
        return self._workers[threads]

    def start_threads(self, n):
        if Reference._threads_started != n:
            self.L.ref_start_threads(int(n))
            Reference._threads_started = n

    def _take(self, tree):
        n = self.L.ref_num_words(tree)
        p = self.L.ref_words(tree)
        words = np.ctypeslib.as_array((ctypes.c_uint32 * n).from_address(p)).copy() if n else \
            np.zeros(0, np.uint32)
        c = np.zeros(3, np.float32)
        self.L.ref_center(tree, _ptr(c, _f32p))
        return words, c

    def load(self, path):
        """Returns an opaque tree handle (free with ``free``)."""
        return self.L.ref_load(path.encode())

    def free(self, tree):
        self.L.ref_free(tree)

    def words(self, tree):
        return self._take(tree)

    def save(self, tree, path):
        self.L.ref_save(tree, path.encode())

    def build_voxel_file(self, path, mem=1 << 30, threads=None, keep=False):
        """(words, center); with keep=True also a loaded in-process tree
        handle of the result (for raymarching)."""
        if self._worker is not None:
            out = self._worker.call("build_voxel_file", path, mem)
        else:
            tree = self.L.ref_build_voxel_file(path.encode(), int(mem))
            out = self._take(tree)
            self.L.ref_free(tree)
        if keep:
            words, center = out
            return out, self.tree_from_words(words, center)
        return out

    def build_ply(self, path, side, mem=1 << 30, threads=4):
        """VoxelData(PlyLoader*, side, mem) + VoxelOctree with a `threads`-thread
        pool (the pool size selects the sub-block partition)."""
        if self._isolated:
            return self._worker_for(threads).call("build_ply", path, side, mem, timeout=60.0)
        tree = self.L.ref_build_ply(path.encode(), int(side), int(mem))
        out = self._take(tree)
        self.L.ref_free(tree)
        return out

    def ply_to_voxel_file(self, ply_path, voxel_path, side, mem=1 << 30, threads=4):
        if self._isolated:
            return self._worker_for(threads).call("ply_to_voxel_file", ply_path, voxel_path, side, mem, timeout=60.0)
        return self.L.ref_ply_to_voxel_file(ply_path.encode(), voxel_path.encode(), int(side), int(mem))

    def ply_volume(self, ply_path, side, mem=1 << 30, threads=4):
        """The reference's convertToVolume steps (ref_shim.cpp ref_ply_volume)
        with a `threads`-thread pool: the (d, h, w) uint32 volume."""
        if self._isolated:
            return self._worker_for(threads).call("ply_volume", ply_path, side, mem, timeout=60.0)
        dims = (ctypes.c_int * 3)()
        self.L.ref_ply_volume(ply_path.encode(), int(side), int(mem), dims, None)
        w, h, d = dims
        out = np.zeros((d, h, w), np.uint32)
        rc = self.L.ref_ply_volume(ply_path.encode(), int(side), int(mem), dims, _ptr(out, _u32p))
        if rc != 0:
            raise RuntimeError("ref_ply_volume failed: %d" % rc)
        return out

    def tree_from_words(self, words, center):
        """An in-process reference tree holding `words` (written to a
        temporary .oct and loaded by VoxelOctree(const char*))."""
        import tempfile
        from_words_path = tempfile.mktemp(suffix=".oct")
        with open(from_words_path, "wb") as f:
            f.write(np.asarray(center, np.float32).tobytes())
            f.write(np.uint64(words.size).tobytes())
            # a single uncompressed-literal LZ4 block per 64 MiB of payload
            raw = np.ascontiguousarray(words, np.uint32).tobytes()
            block = 64 << 20
            for off in range(0, len(raw), block):
                chunk = raw[off:off + block]
                lit = len(chunk)
                if lit < 15:
                    hdr = bytearray([lit << 4])
                else:
                    hdr = bytearray([0xF0])
                    rem = lit - 15
                    while rem >= 255:
                        hdr.append(255)
                        rem -= 255
                    hdr.append(rem)
                f.write(np.uint64(len(hdr) + lit).tobytes())
                f.write(bytes(hdr))
                f.write(chunk)
        tree = self.load(from_words_path)
        os.unlink(from_words_path)
        return tree

    def raymarch(self, tree, rays, ray_scale=0.0, threads=1):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        R = rays.shape[0]
        hit = np.zeros(R, np.uint8)
        t = np.zeros(R, np.float32)
        w = np.zeros(R, np.uint32)
        self.L.ref_raymarch(tree, _ptr(rays, _f32p), R, float(ray_scale), _ptr(hit, _u8p), _ptr(t, _f32p),
                            _ptr(w, _u32p), int(threads))
        return hit, t, w

    def render_frame(self, tree, rot, trans, half_size=False):
        """The viewer's 1280 x 720 frame by the reference's own renderBatch /
        renderTile (ref_render.cpp), with inverse model-view [rot | trans]:
        (720, 1280) uint32 RGBA8."""
        out = np.zeros((720, 1280), np.uint32)
        r = np.ascontiguousarray(rot, np.float32).reshape(9)
        t = np.ascontiguousarray(trans, np.float32).reshape(3)
        self.L.ref_render_frame(tree, _ptr(r, _f32p), _ptr(t, _f32p), 1 if half_size else 0, _ptr(out, _u32p))
        return out

    def compress_material(self, n, shade):
        a = np.ascontiguousarray(n, dtype=np.float32)
        return int(self.L.ref_compress_material(_ptr(a, _f32p), float(shade)))

    def decompress_material(self, word):
        n = np.zeros(3, np.float32)
        s = np.zeros(1, np.float32)
        self.L.ref_decompress_material(int(word), _ptr(n, _f32p), _ptr(s, _f32p))
        return n, float(s[0])

    def inv_sqrt(self, x):
        return self.L.ref_inv_sqrt(float(x))

    def tri_box_overlap(self, center, half, verts):
        c = np.ascontiguousarray(center, dtype=np.float32)
        h = np.ascontiguousarray(half, dtype=np.float32)
        v = np.ascontiguousarray(verts, dtype=np.float32).reshape(9)
        return int(self.L.ref_tri_box_overlap(_ptr(c, _f32p), _ptr(h, _f32p), _ptr(v, _f32p)))


def write_voxel_file(path, grid):
    """Write a reference .voxel file (PlyLoader.cpp:521-528 layout): int32 w, h, d
    then uint32 voxels with x fastest.  grid has shape (d, h, w)."""
    grid = np.ascontiguousarray(grid, dtype=np.uint32)
    d, h, w = grid.shape
    with open(path, "wb") as f:
        f.write(np.array([w, h, d], dtype=np.int32).tobytes())
        f.write(grid.tobytes())
