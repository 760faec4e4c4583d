"""Generate the committed golden fixtures from the reference compiled in place.

Run from the repository root where the reference sources exist:

    make -C oracle ref && python tests/golden/make_golden.py

Outputs (all produced by the reference's own code through oracle/_ref):
  dragon.npz   the shipped models/XYZRGB-Dragon.oct decoded by VoxelOctree(path)
               (words, center, file sha256) and VoxelOctree::raymarch results
               for seeded rays at rayScale 0 and 0.02 (hit, t, normal word)
  builds.npz   VoxelOctree(VoxelData(path, mem)) word streams for seeded small
               grids covering odd dimensions, small memory budgets (several
               cache blocks, an odd last slice, far pointers) and empty grids
  codec.npz    compressMaterial / decompressMaterial / invSqrt samples
  ply.npz      VoxelOctree(VoxelData(PlyLoader(path), side, mem)) word streams
               for a seeded edge-case mesh (displaced icosphere plus
               degenerate triangles and polygons; the mesh arrays are stored
               too) over thread counts, sides and memory budgets
  volumes.npz  PlyLoader::convertToVolume's volumes (the builder's --mode 1)
               for the same mesh, in one slab and in several, produced by the
               reference's own setupBlockProcessing / processBlock steps
               (oracle/ref_shim.cpp ref_ply_volume)
  frames.npz   the viewer's 1280 x 720 frames of the dragon by the reference's
               own renderBatch / renderTile (oracle/ref_render.cpp), full and
               half size, with the cameras' matrices

  python tests/golden/make_golden.py volumes   writes volumes.npz only
  python tests/golden/make_golden.py frames    writes frames.npz only
"""
import hashlib
import importlib.util
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from pyoracle import Oracle, Reference, write_voxel_file, REF_SRC  # noqa: E402

spec = importlib.util.spec_from_file_location("svo_scenes", os.path.join(ROOT, "sparse-voxel-octrees_gb300", "scenes.py"))
scenes = importlib.util.module_from_spec(spec)
spec.loader.exec_module(scenes)

OUT = os.path.dirname(os.path.abspath(__file__))

# (side, threads, mem, with_normals, binary): PLY builds of the edge-case mesh
PLY_CASES = [
    (64, 4, 1 << 30, False, True),
    (64, 16, 5 * 16 ** 3 + 3000, False, True),   # 16^3 cache blocks
    (96, 3, 5 * 32 ** 3 + 40000, True, True),    # file normals, 32^3 blocks
    (37, 8, 1 << 30, False, False),              # ascii, odd side
    (44, 8, 5 * 8 ** 3 + 2000, False, True),     # 8^3 blocks, odd depth (dropped slices)
    (65, 1, 5 * 16 ** 3 + 3000, True, False),
]

# (w, h, d, density, mem, seed)
BUILD_CASES = [
    (2, 2, 2, 0.5, 1 << 30, 1),
    (8, 8, 8, 0.3, 1 << 30, 2),
    (16, 16, 16, 0.0, 1 << 30, 3),
    (16, 16, 16, 1.0, 1 << 30, 4),
    (13, 7, 9, 0.4, 1 << 30, 5),      # odd depth: last slice dropped
    (33, 20, 17, 0.2, 3000, 6),       # 8^3 cache blocks, odd depth
    (40, 40, 41, 0.05, 4096, 7),      # several cache blocks
    (64, 64, 64, 0.1, 1 << 30, 8),    # far pointers at the root
    (48, 31, 25, 0.02, 20000, 9),     # 16^3 cache blocks
    (5, 40, 3, 0.9, 3000, 10),
    (70, 60, 50, 0.01, 1 << 30, 11),
    (29, 29, 29, 0.3, 100000, 12),
]


def golden_grid(shape, density, seed):
    """Seeded occupancy with small payloads (1..251) so the fixture compresses."""
    rng = np.random.default_rng(seed)
    occ = rng.random(shape) < density
    vals = (np.arange(occ.size, dtype=np.uint64) % 251 + 1).astype(np.uint32).reshape(shape)
    return np.where(occ, vals, 0).astype(np.uint32)


# (side, threads, mem) of volumes.npz: one slab, one slab, four slabs of 20 slices
VOLUME_CASES = [(48, 8, 1 << 30), (57, 16, 1 << 30), (64, 6, 62 * 62 * 20)]


def make_volumes(R):
    g = np.load(os.path.join(OUT, "ply.npz"))
    flat = g["faces"].tolist()
    faces, i = [], 0
    while i < len(flat):
        faces.append(flat[i + 1:i + 1 + flat[i]])
        i += 1 + flat[i]
    vols, meta = [], []
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "m.ply")
        scenes.write_ply(path, g["pos"], faces, colors=g["colors"])
        for (side, threads, mem) in VOLUME_CASES:
            v = R.ply_volume(path, side, mem, threads=threads)
            vols.append(v.ravel())
            meta.append((side, threads, mem) + tuple(reversed(v.shape)))
    np.savez_compressed(os.path.join(OUT, "volumes.npz"), meta=np.array(meta, np.uint64),
                        offsets=np.cumsum([0] + [v.size for v in vols]).astype(np.uint64),
                        words=np.concatenate(vols))
    print("volumes.npz", os.path.getsize(os.path.join(OUT, "volumes.npz")))


# (yaw, pitch, radius, half size): viewer frames of the dragon
FRAME_CASES = [(30.0, 20.0, 1.2, 0), (200.0, -35.0, 1.8, 0), (95.0, 60.0, 0.9, 1)]


def make_frames(R):
    g = np.load(os.path.join(OUT, "dragon.npz"))
    tree = R.tree_from_words(g["words"], g["center"])
    rots, transs, poss, halves, frames = [], [], [], [], []
    for (yaw, pitch, radius, half) in FRAME_CASES:
        rot, trans, pos = scenes.viewer_camera(yaw, pitch, radius, g["center"])
        frames.append(R.render_frame(tree, rot, trans, bool(half)))
        rots.append(rot)
        transs.append(trans)
        poss.append(pos)
        halves.append(half)
    R.free(tree)
    np.savez_compressed(os.path.join(OUT, "frames.npz"), rot=np.array(rots), trans=np.array(transs),
                        pos=np.array(poss), half=np.array(halves, np.int32), frames=np.array(frames))
    print("frames.npz", os.path.getsize(os.path.join(OUT, "frames.npz")))


def main():
    R = Reference()
    R.start_threads(4)
    if len(sys.argv) > 1 and sys.argv[1] == "volumes":
        make_volumes(R)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "frames":
        make_frames(R)
        return
    # ---- dragon
    path = os.path.join(REF_SRC, "models", "XYZRGB-Dragon.oct")
    raw = open(path, "rb").read()
    tree = R.load(path)
    words, center = R.words(tree)
    rays = scenes.random_rays(2048, 11, lo=0.0, hi=3.0)
    cams = scenes.orbit_cameras(2, 12, center, radius=1.6)
    cam_rays = np.concatenate([scenes.camera_rays(c, 48, 32) for c in cams])
    rays = np.concatenate([rays, cam_rays]).astype(np.float32)
    h0, t0, w0 = R.raymarch(tree, rays, 0.0)
    h1, t1, w1 = R.raymarch(tree, rays, 0.02)
    R.free(tree)
    np.savez_compressed(os.path.join(OUT, "dragon.npz"), words=words, center=center,
                        file_sha256=np.frombuffer(hashlib.sha256(raw).digest(), np.uint8),
                        rays=rays, hit=h0, t=t0, word=w0, lod_hit=h1, lod_t=t1)
    # ---- builds
    grids, wlist, centers, meta = [], [], [], []
    with tempfile.TemporaryDirectory() as tmp:
        vf = os.path.join(tmp, "g.voxel")
        for (w, h, d, dens, mem, seed) in BUILD_CASES:
            # the reference exits the process when no cache block fits `mem`
            assert Oracle().cache_block(w, h, d, mem) >= 2, (w, h, d, mem)
            g = golden_grid((d, h, w), dens, seed)
            write_voxel_file(vf, g)
            ws, c = R.build_voxel_file(vf, mem)
            grids.append(g.ravel())
            wlist.append(ws)
            centers.append(c)
            meta.append((w, h, d, mem))
    np.savez_compressed(os.path.join(OUT, "builds.npz"),
                        meta=np.array(meta, np.uint64),
                        grid_offsets=np.cumsum([0] + [g.size for g in grids]).astype(np.uint64),
                        grids=np.concatenate(grids),
                        word_offsets=np.cumsum([0] + [x.size for x in wlist]).astype(np.uint64),
                        words=np.concatenate(wlist), centers=np.array(centers, np.float32))
    # ---- codec
    rng = np.random.default_rng(5)
    n = rng.normal(size=(2048, 3)).astype(np.float32)
    n[:64] = np.round(n[:64] * 2)
    n[np.all(n == 0, axis=1)] = (0, 1, 0)
    shade = rng.random(2048).astype(np.float32)
    packed = np.array([R.compress_material(n[i], shade[i]) for i in range(2048)], np.uint32)
    wr = rng.integers(0, 2 ** 32, 2048, dtype=np.uint64).astype(np.uint32)
    wr &= np.uint32(0x9FFFFFFF)  # face bits 0..2 only (face 3 is outside the codec)
    wr |= (rng.integers(0, 3, 2048).astype(np.uint32) << np.uint32(29))
    dec = [R.decompress_material(int(x)) for x in wr]
    xs = (rng.random(2048) * 100).astype(np.float32)
    np.savez_compressed(os.path.join(OUT, "codec.npz"), normals=n, shade=shade, packed=packed, words=wr,
                        dec_n=np.array([d[0] for d in dec], np.float32),
                        dec_shade=np.array([d[1] for d in dec], np.float32),
                        isqrt_x=xs, isqrt_y=np.array([R.inv_sqrt(x) for x in xs], np.float32))
    # ---- PLY builds
    pos, faces, col = scenes.edge_case_mesh(3, 4)
    nrm = np.random.default_rng(17).normal(size=pos.shape).astype(np.float32)
    flat = np.asarray([x for fc in faces for x in (len(fc), *fc)], np.int32)
    wlist, centers, meta = [], [], []
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "m.ply")
        for (side, threads, mem, with_n, binary) in PLY_CASES:
            scenes.write_ply(path, pos, faces, colors=col, normals=nrm if with_n else None, binary=binary)
            ws, c = R.build_ply(path, side, mem, threads=threads)
            wlist.append(ws)
            centers.append(c)
            meta.append((side, threads, mem, int(with_n), int(binary)))
    np.savez_compressed(os.path.join(OUT, "ply.npz"), pos=pos, faces=flat, colors=col, normals=nrm,
                        meta=np.array(meta, np.uint64),
                        word_offsets=np.cumsum([0] + [x.size for x in wlist]).astype(np.uint64),
                        words=np.concatenate(wlist), centers=np.array(centers, np.float32))
    for f in ("dragon.npz", "builds.npz", "codec.npz", "ply.npz"):
        print(f, os.path.getsize(os.path.join(OUT, f)))
    make_volumes(R)
    make_frames(R)


if __name__ == "__main__":
    main()
