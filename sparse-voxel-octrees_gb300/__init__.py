"""Python host interface of the GB300 sparse-voxel-octree library.

A thin ctypes layer over the C ABI in include/svo.h (libsvo_gb300.so).  It
mirrors the reference's C++ interface (src/VoxelOctree.hpp:37-58,
src/VoxelData.hpp:101-144) so tests read like uses of the reference:

    VoxelData(path_or_grid, mem)       -> VoxelData(const char*, size_t) / in-memory grid
    VoxelOctree(path)                  -> VoxelOctree(const char *path)
    VoxelOctree(voxel_data)            -> VoxelOctree(VoxelData *)  (built on the GPU)
    octree.save(path)                  -> VoxelOctree::save
    octree.raymarch(o, d, ray_scale)   -> VoxelOctree::raymarch (one ray; returns (hit, normal, t))
    octree.center()                    -> VoxelOctree::center

plus batched forms (trace over device or host ray arrays).  Every compute call
goes through the CUDA library; importing this module fails loudly when the
library has not been built, and there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsvo_gb300.so")

SVO_OK = 0
SVO_ERR_INVALID = -1
SVO_ERR_IO = -2
SVO_ERR_FORMAT = -3
SVO_ERR_MEMORY = -4
SVO_ERR_CUDA = -5
SVO_ERR_LIMIT = -6
SVO_ERR_DEVICE = -7

DEFAULT_MEM = 1 << 30  # Main.cpp:269

_vp = ctypes.c_void_p
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)


class SvoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("svo error %d: %s" % (code, msg))
        self.code = code


class TraceOut(ctypes.Structure):
    _fields_ = [("hit", _vp), ("t", _vp), ("leaf", _vp), ("word", _vp), ("rgb", _vp), ("rgba8", _vp)]


# Per-ray outputs of the trace entry points (svo_trace_out): rgba8 is the
# viewer's packed 8-bit colour of a traced pixel (renderTile, Main.cpp:126-131).
TRACE_OUTPUTS = ("hit", "t", "leaf", "word", "rgb", "rgba8")


class View(ctypes.Structure):
    _fields_ = [("octree", _vp), ("rays", _vp), ("n_rays", ctypes.c_uint64), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("camera", ctypes.c_float * 17), ("ray_scale", ctypes.c_float),
                ("light", ctypes.c_float * 3), ("out", TraceOut)]


class TraceConfig(ctypes.Structure):
    _fields_ = [("block_threads", ctypes.c_int), ("blocks_per_sm", ctypes.c_int), ("refill_idle", ctypes.c_int),
                ("steps_per_round", ctypes.c_int), ("tile_w", ctypes.c_int), ("chunk", ctypes.c_int),
                ("cache_entries", ctypes.c_int), ("reg_cap", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libsvo_gb300.so is not built (run __graft_entry__.build() or "
                          "python sparse-voxel-octrees_gb300/build_lib.py)")
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "svo_last_error": (ctypes.c_char_p, []),
        "svo_version": (ctypes.c_int, []),
        "svo_octree_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
        "svo_octree_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "svo_oct_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_u32p), _u64p, _f32p]),
        "svo_oct_write": (ctypes.c_int, [ctypes.c_char_p, _vp, ctypes.c_uint64, _f32p]),
        "svo_free": (None, [_vp]),
        "svo_trim_memory": (ctypes.c_int, []),
        "svo_octree_from_words": (ctypes.c_int, [_vp, ctypes.c_uint64, _f32p, ctypes.POINTER(_vp)]),
        "svo_octree_destroy": (ctypes.c_int, [_vp]),
        "svo_octree_num_words": (ctypes.c_int, [_vp, _u64p]),
        "svo_octree_copy_words": (ctypes.c_int, [_vp, _vp, ctypes.c_uint64]),
        "svo_octree_set_index_width": (ctypes.c_int, [_vp, ctypes.c_int]),
        "svo_octree_set_table": (ctypes.c_int, [_vp, ctypes.c_int]),
        "svo_octree_table_size": (ctypes.c_int, [_vp, _u64p]),
        "svo_octree_device_words": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
        "svo_octree_center": (ctypes.c_int, [_vp, _f32p]),
        "svo_octree_device_status": (ctypes.c_int, [_vp, _u32p]),
        "svo_octree_validate": (ctypes.c_int, [_vp, _u64p, _u64p]),
        "svo_octree_build_dense": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                                  ctypes.c_int, _vp, ctypes.POINTER(_vp)]),
        "svo_octree_build_voxel_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint64, _vp, ctypes.POINTER(_vp)]),
        "svo_octree_build_voxel_file_streamed": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint64, ctypes.c_uint64, _vp,
                                                                ctypes.POINTER(_vp)]),
        "svo_mesh_load_ply": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
        "svo_mesh_from_arrays": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_uint64, _vp, ctypes.c_uint64,
                                                ctypes.POINTER(_vp)]),
        "svo_mesh_num_triangles": (ctypes.c_uint64, [_vp]),
        "svo_ply_parse": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_f32p), ctypes.POINTER(_f32p),
                                         ctypes.POINTER(_f32p), _u64p, ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)),
                                         _u64p, _f32p, _f32p]),
        "svo_mesh_dimensions": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
        "svo_mesh_to_volume": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, _vp, _vp]),
        "svo_mesh_write_voxel_file": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_uint64, _vp]),
        "svo_mesh_destroy": (None, [_vp]),
        "svo_octree_build_mesh": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, _vp,
                                                 ctypes.POINTER(_vp)]),
        "svo_octree_build_ply": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, _vp,
                                                ctypes.POINTER(_vp)]),
        "svo_trace": (ctypes.c_int, [_vp, _vp, ctypes.c_uint64, ctypes.c_float, _f32p, ctypes.POINTER(TraceOut), _vp]),
        "svo_trace_host": (ctypes.c_int, [_vp, _vp, ctypes.c_uint64, ctypes.c_float, _f32p,
                                          ctypes.POINTER(TraceOut)]),
        "svo_trace_count_loads": (ctypes.c_int, [_vp, _vp, ctypes.c_uint64, ctypes.c_float, _vp, _vp]),
        "svo_trace_image": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, _f32p,
                                           ctypes.POINTER(TraceOut), _vp]),
        "svo_trace_image_host": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, _f32p,
                                                ctypes.POINTER(TraceOut)]),
        "svo_trace_host_async": (ctypes.c_int, [_vp, _vp, ctypes.c_uint64, ctypes.c_float, _f32p,
                                                ctypes.POINTER(TraceOut)]),
        "svo_trace_image_host_async": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                                      _f32p, ctypes.POINTER(TraceOut)]),
        "svo_octree_synchronize": (ctypes.c_int, [_vp]),
        "svo_diff_forward": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp, _vp, _vp,
                                            _vp, _vp, _vp]),
        "svo_diff_backward": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp, _vp, _vp,
                                             _vp, _vp, _vp, _vp, _vp]),
        "svo_diff_backward_l2": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp, _vp,
                                                _vp, _vp, _vp, _vp, ctypes.c_float, _vp, _vp, _vp, _vp, _vp, _vp,
                                                ctypes.c_uint64, _vp]),
        "svo_diff_forward_stride": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp,
                                                   _vp, _vp, ctypes.c_uint32, _vp, _vp, _vp]),
        "svo_diff_backward_stride": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp,
                                                    _vp, _vp, ctypes.c_uint32, _vp, _vp, _vp, _vp, _vp]),
        "svo_diff_backward_l2_stride": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                                       _vp, _vp, _vp, ctypes.c_uint32, _vp, _vp, _vp, ctypes.c_float,
                                                       _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_uint64, _vp]),
        "svo_adam_step_leaves": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_uint64, ctypes.c_uint32, _vp, _vp,
                                                ctypes.c_uint64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                                ctypes.c_float, ctypes.c_int, ctypes.c_int, _vp]),
        "svo_render_frame": (ctypes.c_int, [_vp, _f32p, _f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                            ctypes.c_uint32, _vp, _vp]),
        "svo_adam_step": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_uint64, ctypes.c_float, ctypes.c_float,
                                         ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int, _vp]),
        "svo_batch_create": (ctypes.c_int, [ctypes.POINTER(View), ctypes.c_int, ctypes.POINTER(_vp)]),
        "svo_batch_default_config": (ctypes.c_int, [ctypes.POINTER(TraceConfig)]),
        "svo_batch_num_slots": (ctypes.c_int, [_vp, _u64p]),
        "svo_batch_trace": (ctypes.c_int, [_vp, ctypes.POINTER(TraceConfig), _vp]),
        "svo_batch_capture_graph": (ctypes.c_int, [_vp, ctypes.POINTER(TraceConfig)]),
        "svo_batch_launch_graph": (ctypes.c_int, [_vp, _vp]),
        "svo_batch_autotune": (ctypes.c_int, [_vp, ctypes.POINTER(TraceConfig), ctypes.POINTER(ctypes.c_float), _vp]),
        "svo_batch_status": (ctypes.c_int, [_vp, _u32p]),
        "svo_batch_destroy": (ctypes.c_int, [_vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


lib = _load()


def check(rc):
    if rc != SVO_OK:
        raise SvoError(rc, lib.svo_last_error().decode(errors="replace"))
    return rc


def _np_ptr(a):
    return a.ctypes.data_as(_vp) if a is not None else None


def _dev_ptr(x):
    """Device pointer of a torch CUDA tensor (or an int address)."""
    if x is None:
        return None
    if isinstance(x, int):
        return _vp(x)
    return _vp(x.data_ptr())


def _stream_ptr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return _vp(stream)
    return _vp(stream.cuda_stream)


def trim_memory():
    """Returns the builds' pooled scratch memory to the driver (svo_trim_memory)."""
    check(lib.svo_trim_memory())


def oct_read(path):
    """Decode a .oct file on the host: returns (words, center)."""
    p = _u32p()
    n = ctypes.c_uint64()
    c = np.zeros(3, np.float32)
    check(lib.svo_oct_read(os.fsencode(path), ctypes.byref(p), ctypes.byref(n), c.ctypes.data_as(_f32p)))
    words = np.ctypeslib.as_array(p, shape=(n.value,)).copy()
    lib.svo_free(ctypes.cast(p, _vp))
    return words, c


def oct_write(path, words, center):
    """Encode host words as a .oct file."""
    words = np.ascontiguousarray(words, dtype=np.uint32)
    c = np.ascontiguousarray(center, dtype=np.float32)
    check(lib.svo_oct_write(os.fsencode(path), _np_ptr(words), words.size, c.ctypes.data_as(_f32p)))


def ply_parse(path):
    """Host-only PLY parse (svo_ply_parse): dict with positions, normals (or
    None), colors (V x 3 float32), triangles (T x 3 int32), lower, upper."""
    pp, pn, pc, pt = _f32p(), _f32p(), _f32p(), ctypes.POINTER(ctypes.c_int32)()
    nv, nt = ctypes.c_uint64(), ctypes.c_uint64()
    lo, hi = np.zeros(3, np.float32), np.zeros(3, np.float32)
    check(lib.svo_ply_parse(os.fsencode(path), ctypes.byref(pp), ctypes.byref(pn), ctypes.byref(pc), ctypes.byref(nv),
                            ctypes.byref(pt), ctypes.byref(nt), lo.ctypes.data_as(_f32p), hi.ctypes.data_as(_f32p)))

    def take(p, n, k):
        if not p:
            return None
        a = np.ctypeslib.as_array(p, shape=(n * k,)).copy().reshape(n, k) if n else np.zeros((0, k), np.float32)
        lib.svo_free(ctypes.cast(p, _vp))
        return a

    V, T = nv.value, nt.value
    return {"positions": take(pp, V, 3), "normals": take(pn, V, 3), "colors": take(pc, V, 3),
            "triangles": take(pt, T, 3), "lower": lo, "upper": hi}


class PlyLoader:
    """A triangle mesh on the current device: PlyLoader(const char *path)
    (PlyLoader.cpp:66-79), or PlyLoader.from_arrays(positions, faces,
    normals=None, colors=None) for a mesh already in memory (faces: (F, k)
    array or a list of index lists; colours as floats, 255 when absent)."""

    def __init__(self, path=None, _handle=None):
        self._h = _vp()
        if _handle is not None:
            self._h = _handle
        else:
            check(lib.svo_mesh_load_ply(os.fsencode(path), ctypes.byref(self._h)))

    @classmethod
    def from_arrays(cls, positions, faces, normals=None, colors=None):
        pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
        nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        col = None if colors is None else np.ascontiguousarray(colors, dtype=np.float32).reshape(-1, 3)
        if isinstance(faces, np.ndarray) and faces.ndim == 2:
            f = np.asarray(faces, dtype=np.int32)
            flat = np.concatenate([np.full((f.shape[0], 1), f.shape[1], np.int32), f], 1).ravel()
        else:
            flat = np.asarray([x for fc in faces for x in (len(fc), *fc)], dtype=np.int32)
        flat = np.ascontiguousarray(flat, dtype=np.int32)
        h = _vp()
        check(lib.svo_mesh_from_arrays(_np_ptr(pos), _np_ptr(nrm), _np_ptr(col), pos.shape[0], _np_ptr(flat),
                                       flat.size, ctypes.byref(h)))
        return cls(_handle=h)

    @property
    def num_triangles(self):
        return int(lib.svo_mesh_num_triangles(self._h))

    def suggested_dimensions(self, side):
        """PlyLoader::suggestedDimensions (PlyLoader.cpp:499-504)."""
        dims = (ctypes.c_int * 3)()
        check(lib.svo_mesh_dimensions(self._h, int(side), dims))
        return tuple(dims)

    def convertToVolume(self, path, maxSize, memoryBudget=DEFAULT_MEM, threads=None):
        """PlyLoader::convertToVolume (PlyLoader.cpp:506-534): the .voxel file
        of this mesh at suggestedDimensions(maxSize), voxelized with a
        `threads`-thread pool's sub-block partition, in z-slabs of
        memoryBudget // (w*h) slices through one buffer that is never cleared
        between slabs (svo_mesh_write_voxel_file)."""
        threads = int(threads if threads is not None else (os.cpu_count() or 1))
        check(lib.svo_mesh_write_voxel_file(self._h, os.fsencode(path), int(maxSize), threads, int(memoryBudget),
                                            None))

    def to_volume(self, side, threads, mem=DEFAULT_MEM, stream=None, out=None):
        """The same volume as a (d, h, w) int32 CUDA tensor (svo_mesh_to_volume),
        written into `out` when given."""
        import torch
        w, h, d = self.suggested_dimensions(side)
        if out is None:
            out = torch.empty((d, h, w), dtype=torch.int32, device="cuda")
        if tuple(out.shape) != (d, h, w) or not out.is_contiguous() or str(out.dtype) != "torch.int32":
            raise ValueError("out must be a contiguous int32 CUDA tensor of shape %s" % ((d, h, w),))
        check(lib.svo_mesh_to_volume(self._h, int(side), int(threads), int(mem), _dev_ptr(out), _stream_ptr(stream)))
        return out

    def close(self):
        if self._h:
            lib.svo_mesh_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class VoxelData:
    """Input of the octree build: VoxelData(const char *path, size_t mem)
    (VoxelData.cpp:37-48), VoxelData(PlyLoader, side, mem, threads)
    (VoxelData.cpp:50-56; `threads` is the reference's thread-pool size,
    which its voxelization depends on), or an in-memory dense grid of shape
    (d, h, w), x fastest, 0 = empty (a numpy array or a CUDA tensor)."""

    def __init__(self, source, side=None, mem=DEFAULT_MEM, threads=None, slab_bytes=0):
        self.slab_bytes = int(slab_bytes)  # > 0: stream a .voxel file in slabs of about this many device bytes
        self.path = None
        self.grid = None
        self.loader = None
        if isinstance(source, PlyLoader):
            if side is None:
                raise TypeError("VoxelData(PlyLoader, side, mem, threads)")
            self.loader = source
            self.side = int(side)
            self.threads = int(threads if threads is not None else (os.cpu_count() or 1))
            self.mem = int(mem)
            return
        if side is not None:  # VoxelData(path_or_grid, mem)
            mem = side
        self.mem = int(mem)
        if isinstance(source, (str, bytes, os.PathLike)):
            self.path = os.fsdecode(source)
        else:
            self.grid = source

    @property
    def on_device(self):
        return self.grid is not None and hasattr(self.grid, "is_cuda") and self.grid.is_cuda


class VoxelOctree:
    """Resident GPU octree; see the module docstring for the reference mapping."""

    def __init__(self, source=None, stream=None, _handle=None):
        self._h = _vp()
        self._pending = []  # host arrays of asynchronous traces, kept alive until synchronize()
        if _handle is not None:
            self._h = _handle
        elif isinstance(source, (str, bytes, os.PathLike)):
            check(lib.svo_octree_load(os.fsencode(source), ctypes.byref(self._h)))
        elif isinstance(source, VoxelData):
            if source.loader is not None:
                check(lib.svo_octree_build_mesh(source.loader._h, source.side, source.threads, source.mem,
                                                _stream_ptr(stream), ctypes.byref(self._h)))
            elif source.path is not None and source.slab_bytes > 0:
                check(lib.svo_octree_build_voxel_file_streamed(os.fsencode(source.path), source.mem, source.slab_bytes,
                                                               _stream_ptr(stream), ctypes.byref(self._h)))
            elif source.path is not None:
                check(lib.svo_octree_build_voxel_file(os.fsencode(source.path), source.mem, _stream_ptr(stream),
                                                      ctypes.byref(self._h)))
            else:
                g = source.grid
                d, h, w = g.shape
                if source.on_device:
                    if str(g.dtype) not in ("torch.int32", "torch.uint32") or not g.is_contiguous():
                        raise ValueError("a device grid must be a contiguous int32 or uint32 tensor")
                    check(lib.svo_octree_build_dense(_dev_ptr(g), w, h, d, source.mem, 1, _stream_ptr(stream),
                                                     ctypes.byref(self._h)))
                else:
                    a = np.ascontiguousarray(g, dtype=np.uint32)
                    check(lib.svo_octree_build_dense(_np_ptr(a), w, h, d, source.mem, 0, _stream_ptr(stream),
                                                     ctypes.byref(self._h)))
        else:
            raise TypeError("VoxelOctree(path | VoxelData)")

    @classmethod
    def from_words(cls, words, center):
        words = np.ascontiguousarray(words, dtype=np.uint32)
        c = np.ascontiguousarray(center, dtype=np.float32)
        h = _vp()
        check(lib.svo_octree_from_words(_np_ptr(words), words.size, c.ctypes.data_as(_f32p), ctypes.byref(h)))
        return cls(_handle=h)

    def close(self):
        if self._h:
            lib.svo_octree_destroy(self._h)  # waits for queued host traces first
            self._h = _vp()
        self._pending = []

    def synchronize(self):
        """Waits for the host traces queued with wait=False (svo_octree_synchronize)."""
        try:
            check(lib.svo_octree_synchronize(self._h))
        finally:
            self._pending = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- VoxelOctree.hpp surface
    def save(self, path):
        check(lib.svo_octree_save(self._h, os.fsencode(path)))

    def center(self):
        c = np.zeros(3, np.float32)
        check(lib.svo_octree_center(self._h, c.ctypes.data_as(_f32p)))
        return c

    def raymarch(self, o, d, ray_scale=0.0):
        """One ray, as VoxelOctree::raymarch: returns (hit, normal, t).
        `normal` and `t` are None where the reference leaves them unset."""
        rays = np.array([list(o) + list(d)], dtype=np.float32)
        r = self.trace_host(rays, ray_scale=ray_scale, outputs=("hit", "t", "word"))
        hit = int(r["hit"][0])
        if hit == 0:
            return False, None, None
        return True, (int(r["word"][0]) if hit == 1 else None), float(r["t"][0])

    # -- words
    def num_words(self):
        n = ctypes.c_uint64()
        check(lib.svo_octree_num_words(self._h, ctypes.byref(n)))
        return n.value

    def set_index_width(self, bits):
        """32 or 64-bit word indices for trace()/trace_host(); octrees above
        2^32-1 words always use 64."""
        check(lib.svo_octree_set_index_width(self._h, int(bits)))

    def set_table(self, enable):
        """Walk the descriptor table (default) or the words directly."""
        check(lib.svo_octree_set_table(self._h, 1 if enable else 0))

    def table_size(self):
        """Entries of the descriptor table (built now if needed); 0 when the
        octree does not qualify for one."""
        n = ctypes.c_uint64()
        check(lib.svo_octree_table_size(self._h, ctypes.byref(n)))
        return n.value

    def words(self):
        n = self.num_words()
        out = np.empty(n, np.uint32)
        check(lib.svo_octree_copy_words(self._h, _np_ptr(out), n))
        return out

    def device_words_ptr(self):
        p = _vp()
        check(lib.svo_octree_device_words(self._h, ctypes.byref(p)))
        return p.value

    def validate(self):
        nd = ctypes.c_uint64()
        nl = ctypes.c_uint64()
        check(lib.svo_octree_validate(self._h, ctypes.byref(nd), ctypes.byref(nl)))
        return nd.value, nl.value

    def device_status(self):
        f = ctypes.c_uint32()
        check(lib.svo_octree_device_status(self._h, ctypes.byref(f)))
        return f.value

    # -- batched tracing
    def trace(self, rays, n=None, ray_scale=0.0, light=(0.0, 0.0, 1.0), out=None, stream=None):
        """Device form: rays is a CUDA tensor (R, 6) float32; out maps any of
        hit/t/leaf/word/rgb/rgba8 to preallocated CUDA tensors."""
        if n is None:
            n = rays.shape[0]
        o = TraceOut()
        for k in TRACE_OUTPUTS:
            v = (out or {}).get(k)
            setattr(o, k, _dev_ptr(v).value if v is not None else None)
        lt = np.ascontiguousarray(light, dtype=np.float32)
        check(lib.svo_trace(self._h, _dev_ptr(rays), int(n), float(ray_scale), lt.ctypes.data_as(_f32p),
                            ctypes.byref(o), _stream_ptr(stream)))

    def trace_host(self, rays, ray_scale=0.0, light=(0.0, 0.0, 1.0), outputs=("hit", "t", "leaf", "word", "rgb"),
                   out=None, wait=True):
        """Host form: rays is a numpy (R, 6) float32 array (pinned or not);
        returns a dict of numpy outputs (or fills `out`).  wait=False queues
        the work (svo_trace_host_async): the results are there after
        synchronize()."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        R = rays.shape[0]
        shapes = {"hit": ((R,), np.uint8), "t": ((R,), np.float32), "leaf": ((R,), np.uint32),
                  "word": ((R,), np.uint32), "rgb": ((R, 3), np.float32), "rgba8": ((R,), np.uint32)}
        res = out if out is not None else {k: np.empty(*shapes[k]) for k in outputs}
        o = TraceOut()
        for k in TRACE_OUTPUTS:
            v = res.get(k)
            setattr(o, k, v.ctypes.data if v is not None else None)
        lt = np.ascontiguousarray(light, dtype=np.float32)
        fn = lib.svo_trace_host if wait else lib.svo_trace_host_async
        check(fn(self._h, _np_ptr(rays), R, float(ray_scale), lt.ctypes.data_as(_f32p), ctypes.byref(o)))
        if not wait:
            self._pending.append((rays, res))
        return res

    def trace_image(self, rays, width, height, ray_scale=0.0, light=(0.0, 0.0, 1.0), out=None, stream=None):
        """Device form for row-major image rays (R = width*height)."""
        o = TraceOut()
        for k in TRACE_OUTPUTS:
            v = (out or {}).get(k)
            setattr(o, k, _dev_ptr(v).value if v is not None else None)
        lt = np.ascontiguousarray(light, dtype=np.float32)
        check(lib.svo_trace_image(self._h, _dev_ptr(rays), int(width), int(height), float(ray_scale),
                                  lt.ctypes.data_as(_f32p), ctypes.byref(o), _stream_ptr(stream)))

    def trace_image_host(self, rays, width, height, ray_scale=0.0, light=(0.0, 0.0, 1.0),
                         outputs=("hit", "t", "leaf", "word", "rgb"), out=None, wait=True):
        """svo_trace_image_host (or, with wait=False, its asynchronous form)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        R = rays.shape[0]
        if R != width * height:
            raise ValueError("%d rays for a %dx%d image" % (R, width, height))
        shapes = {"hit": ((R,), np.uint8), "t": ((R,), np.float32), "leaf": ((R,), np.uint32),
                  "word": ((R,), np.uint32), "rgb": ((R, 3), np.float32), "rgba8": ((R,), np.uint32)}
        res = out if out is not None else {k: np.empty(*shapes[k]) for k in outputs}
        o = TraceOut()
        for k in TRACE_OUTPUTS:
            v = res.get(k)
            setattr(o, k, v.ctypes.data if v is not None else None)
        lt = np.ascontiguousarray(light, dtype=np.float32)
        fn = lib.svo_trace_image_host if wait else lib.svo_trace_image_host_async
        check(fn(self._h, _np_ptr(rays), int(width), int(height), float(ray_scale), lt.ctypes.data_as(_f32p),
                 ctypes.byref(o)))
        if not wait:
            self._pending.append((rays, res))
        return res

    def diff_forward(self, rays, width, height, n_views, lights, leaf_rgb, leaf_normal, rgb, hit_leaf=None,
                     stream=None, param_stride=3):
        """Differentiable shading forward (all CUDA tensors); see svo_diff_forward.
        param_stride: floats from one leaf's parameters to the next (8 with
        leaf_normal = the record's floats 3..5: svo_diff_forward_stride)."""
        check(lib.svo_diff_forward_stride(self._h, _dev_ptr(rays), int(width), int(height), int(n_views),
                                          _dev_ptr(lights), _dev_ptr(leaf_rgb), _dev_ptr(leaf_normal),
                                          int(param_stride), _dev_ptr(hit_leaf), _dev_ptr(rgb), _stream_ptr(stream)))

    def diff_backward(self, rays, width, height, n_views, lights, leaf_rgb, leaf_normal, d_rgb, grad_rgb,
                      grad_normal, hit_leaf=None, stream=None, param_stride=3):
        """Adjoint: accumulates parameter gradients; hit_leaf=None re-traces."""
        check(lib.svo_diff_backward_stride(self._h, _dev_ptr(rays), int(width), int(height), int(n_views),
                                           _dev_ptr(lights), _dev_ptr(leaf_rgb), _dev_ptr(leaf_normal),
                                           int(param_stride), _dev_ptr(hit_leaf), _dev_ptr(d_rgb), _dev_ptr(grad_rgb),
                                           _dev_ptr(grad_normal), _stream_ptr(stream)))

    def diff_backward_l2(self, rays, width, height, n_views, lights, leaf_rgb, leaf_normal, rgb, target, loss_scale,
                         grad_rgb, grad_normal, hit_leaf=None, loss_sum=None, leaves=None, stream=None,
                         param_stride=3):
        """Adjoint of the L2 loss loss_scale/2 * sum (rgb - target)^2 with the
        loss gradient formed in the kernel (svo_diff_backward_l2); loss_sum
        (a float64 CUDA tensor) accumulates sum (rgb - target)^2, and
        `leaves` (a LeafSet) records the leaves that received a gradient."""
        tb = ll = lc = None
        cap = 0
        if leaves is not None:
            tb, ll, lc, cap = leaves.touched, leaves.list, leaves.count, leaves.list.numel()
        check(lib.svo_diff_backward_l2_stride(self._h, _dev_ptr(rays), int(width), int(height), int(n_views),
                                              _dev_ptr(lights), _dev_ptr(leaf_rgb), _dev_ptr(leaf_normal),
                                              int(param_stride), _dev_ptr(hit_leaf), _dev_ptr(rgb), _dev_ptr(target),
                                              float(loss_scale), _dev_ptr(grad_rgb), _dev_ptr(grad_normal),
                                              _dev_ptr(loss_sum), _dev_ptr(tb), _dev_ptr(ll), _dev_ptr(lc), int(cap),
                                              _stream_ptr(stream)))

    def render_frame(self, rot, pos, width=1280, height=720, n_strips=16, pixel_stride=1, out=None, stream=None):
        """The viewer's frame (svo_render_frame) into `out`, an int32 CUDA
        tensor of height*width RGBA8 words (allocated when None)."""
        import torch
        r = np.ascontiguousarray(rot, dtype=np.float32).reshape(9)
        p = np.ascontiguousarray(pos, dtype=np.float32).reshape(3)
        if out is None:
            out = torch.empty((height, width), dtype=torch.int32, device="cuda")
        if not (out.is_cuda and out.is_contiguous() and out.numel() == width * height):
            raise ValueError("out must be a contiguous CUDA tensor of width*height words")
        check(lib.svo_render_frame(self._h, r.ctypes.data_as(_f32p), p.ctypes.data_as(_f32p), width, height, n_strips,
                                   pixel_stride, _dev_ptr(out), _stream_ptr(stream)))
        return out

    def count_loads(self, rays, n=None, ray_scale=0.0, loads=None, stream=None):
        if n is None:
            n = rays.shape[0]
        check(lib.svo_trace_count_loads(self._h, _dev_ptr(rays), int(n), float(ray_scale), _dev_ptr(loads),
                                        _stream_ptr(stream)))


class LeafSet:
    """The leaves that have received a gradient (svo_diff_backward_l2's
    record): a bit per octree word, the leaves in order of first touch, and
    their count, all on the device and zeroed at creation."""

    def __init__(self, n_words, device="cuda"):
        import torch
        self.touched = torch.zeros((n_words + 31) // 32, dtype=torch.int32, device=device)
        self.list = torch.zeros(max(1, n_words), dtype=torch.int32, device=device)
        self.count = torch.zeros(1, dtype=torch.int32, device=device)

    def size(self):
        return int(self.count.item())


class LeafAdam:
    """Adam over per-leaf parameter tensors (CUDA float32, contiguous) with
    svo_adam_step: one fused pass per tensor that also zeroes the gradient
    (pass zero_grad=False to keep it).  step() reads each tensor's .grad.
    With `leaves` (a LeafSet kept by diff_backward_l2) only the listed
    leaves' `width` values per leaf are updated (svo_adam_step_leaves), with
    results identical to the dense pass."""

    def __init__(self, params, lr=1e-2, betas=(0.9, 0.999), eps=1e-8, zero_grad=True, leaves=None, width=3):
        import torch
        self.params = list(params)
        self.lr, self.betas, self.eps, self.zero_grad = float(lr), betas, float(eps), zero_grad
        self.state = [(torch.zeros_like(p), torch.zeros_like(p)) for p in self.params]
        self.leaves, self.width = leaves, int(width)
        self.t = 0

    def step(self, stream=None):
        self.t += 1
        for p, (m, v) in zip(self.params, self.state):
            g = p.grad
            if g is None or not (p.is_contiguous() and g.is_contiguous()):
                raise ValueError("LeafAdam needs contiguous parameters with gradients")
            if self.leaves is not None:
                L = self.leaves
                check(lib.svo_adam_step_leaves(_dev_ptr(p), _dev_ptr(g), _dev_ptr(m), _dev_ptr(v), p.numel(),
                                               self.width, _dev_ptr(L.list), _dev_ptr(L.count), L.list.numel(),
                                               self.lr, float(self.betas[0]), float(self.betas[1]), self.eps, self.t,
                                               1 if self.zero_grad else 0, _stream_ptr(stream)))
                continue
            check(lib.svo_adam_step(_dev_ptr(p), _dev_ptr(g), _dev_ptr(m), _dev_ptr(v), p.numel(), self.lr,
                                    float(self.betas[0]), float(self.betas[1]), self.eps, self.t,
                                    1 if self.zero_grad else 0, _stream_ptr(stream)))


def default_config(**overrides):
    c = TraceConfig()
    check(lib.svo_batch_default_config(ctypes.byref(c)))
    for k, v in overrides.items():
        setattr(c, k, int(v))
    return c


class Batch:
    """Many (octree, view) pairs traced by one persistent launch (svo_batch_*).

    views: list of dicts with keys octree (VoxelOctree), and either
      rays (CUDA tensor (R, 6)) [+ width, height for image order], or
      camera (17 floats, scenes.camera_constants) + width + height;
    optional ray_scale, light, and out: dict of CUDA tensors (hit/t/leaf/word/rgb).
    """

    def __init__(self, views):
        self._keep = views
        arr = (View * len(views))()
        for i, v in enumerate(views):
            cv = arr[i]
            cv.octree = v["octree"].handle.value
            rays = v.get("rays")
            cv.rays = _dev_ptr(rays).value if rays is not None else None
            cv.width = int(v.get("width", 0))
            cv.height = int(v.get("height", 0))
            cv.n_rays = int(v.get("n_rays", rays.shape[0] if (rays is not None and not cv.width) else 0))
            cam = v.get("camera")
            if cam is not None:
                for k in range(17):
                    cv.camera[k] = float(cam[k])
            cv.ray_scale = float(v.get("ray_scale", 0.0))
            lt = v.get("light", (0.0, 0.0, 1.0))
            for k in range(3):
                cv.light[k] = float(lt[k])
            out = v.get("out", {})
            for k in TRACE_OUTPUTS:
                t = out.get(k)
                setattr(cv.out, k, _dev_ptr(t).value if t is not None else None)
        self._h = _vp()
        check(lib.svo_batch_create(arr, len(views), ctypes.byref(self._h)))

    def close(self):
        if self._h:
            lib.svo_batch_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_slots(self):
        n = ctypes.c_uint64()
        check(lib.svo_batch_num_slots(self._h, ctypes.byref(n)))
        return n.value

    def trace(self, config=None, stream=None):
        check(lib.svo_batch_trace(self._h, ctypes.byref(config) if config is not None else None,
                                  _stream_ptr(stream)))

    def capture_graph(self, config=None):
        check(lib.svo_batch_capture_graph(self._h, ctypes.byref(config) if config is not None else None))

    def launch_graph(self, stream=None):
        check(lib.svo_batch_launch_graph(self._h, _stream_ptr(stream)))

    def autotune(self, stream=None):
        c = TraceConfig()
        ms = ctypes.c_float()
        check(lib.svo_batch_autotune(self._h, ctypes.byref(c), ctypes.byref(ms), _stream_ptr(stream)))
        return c, ms.value

    def status(self):
        f = ctypes.c_uint32()
        check(lib.svo_batch_status(self._h, ctypes.byref(f)))
        return f.value
