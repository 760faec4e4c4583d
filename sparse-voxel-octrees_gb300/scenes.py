"""Seeded synthetic scenes and camera rays for tests and benchmarks.

The reference ships no benchmark inputs, so the workloads are generated:

* sphere unions (union of solid spheres; voxel (x, y, z) is occupied when its
  centre (x+.5, y+.5, z+.5) lies within radius r of a sphere centre, tested
  in float32 as dx*dx + dy*dy + dz*dz <= r*r),
* a value-noise heightfield terrain (y up) with a shell of fixed thickness,
* voxel payload words as the reference's voxelizer would store them: a
  normal from the central difference of occupancy (outward, each component
  occ(-1) - occ(+1); (0, 1, 0) where it vanishes) and a shade equal to the
  Rec.709 luminance / 256 of an RGB8 colour taken from a 32-bit hash of the
  voxel coordinates (PlyLoader.cpp:315), packed by compressMaterial
  (Util.hpp:64-84); a word that packs to 0 (= empty) is stored as 1,
* camera rays by the reference viewer's formula (Main.cpp:149-176):
  pos = INV_MODELVIEW * 0 + center + 1, direction (dx*a11 + dy*a12 + zx, ...)
  with dx = -1 + x*2/W, dy = H/W - y*2/W, zx = a13/tan(pi/6), normalised with
  the Quake inverse square root.  INV_MODELVIEW is MODEL^-1 * VIEW with
  MODEL = rotXYZ(pitch, 0, 0) * rotXYZ(0, yaw, 0) and VIEW = translate(0, 0, -r).

All float arithmetic is float32 in the reference's operation order, so the
CUDA generators (when used) produce the same bits.
"""
import math

import numpy as np

F = np.float32


# ---------------------------------------------------------------- codec (numpy)

def inv_sqrt(x):
    """Util.hpp:47-58, vectorised."""
    x = np.asarray(x, dtype=np.float32)
    x2 = x * F(0.5)
    i = x.view(np.uint32)
    i = np.uint32(0x5F3759DF) - (i >> np.uint32(1))
    y = i.view(np.float32)
    return y * (F(1.5) - x2 * y * y)


def compress_material(nx, ny, nz, shade):
    """Util.hpp:64-84, vectorised over float32 arrays."""
    nx = np.asarray(nx, np.float32)
    ny = np.asarray(ny, np.float32)
    nz = np.asarray(nz, np.float32)
    shade = np.asarray(shade, np.float32)
    ax, ay, az = np.abs(nx), np.abs(ny), np.abs(nz)
    face = np.zeros(nx.shape, np.uint32)
    dom = ax.copy()
    m = ay > dom
    face[m] = 1
    dom[m] = ay[m]
    m = az > dom
    face[m] = 2
    dom[m] = az[m]
    n = np.stack([nx, ny, nz])
    idx = np.arange(nx.size).reshape(nx.shape)
    f1 = np.where(face == 2, 0, face + 1)
    f2 = np.where(face == 0, 2, face - 1)
    sel = n.reshape(3, -1)
    nf = sel[face.ravel(), idx.ravel()].reshape(nx.shape)
    n1 = sel[f1.ravel(), idx.ravel()].reshape(nx.shape) / dom
    n2 = sel[f2.ravel(), idx.ravel()].reshape(nx.shape) / dom
    sign = (nf < F(0)).astype(np.uint32)
    u = np.minimum(((n1 * F(0.5) + F(0.5)) * F(2047)).astype(np.int32), 0x7FF).astype(np.uint32)
    v = np.minimum(((n2 * F(0.5) + F(0.5)) * F(2047)).astype(np.int32), 0x7FF).astype(np.uint32)
    c = np.minimum((shade * F(127)).astype(np.int32), 0x7F).astype(np.uint32)
    return (sign << 31) | (face << 29) | (u << 18) | (v << 7) | c


def hash32(x, y, z):
    """32-bit coordinate hash (multiply-xor mix followed by a murmur3 finaliser)."""
    x = np.asarray(x, np.uint32)
    y = np.asarray(y, np.uint32)
    z = np.asarray(z, np.uint32)
    with np.errstate(over="ignore"):
        h = (x * np.uint32(0x8DA6B343)) ^ (y * np.uint32(0xD8163841)) ^ (z * np.uint32(0xCB1AB31F))
        h ^= h >> np.uint32(16)
        h *= np.uint32(0x85EBCA6B)
        h ^= h >> np.uint32(13)
        h *= np.uint32(0xC2B2AE35)
        h ^= h >> np.uint32(16)
    return h


def hash_shade(x, y, z):
    h = hash32(x, y, z)
    r = (h & np.uint32(255)).astype(np.float32)
    g = ((h >> np.uint32(8)) & np.uint32(255)).astype(np.float32)
    b = ((h >> np.uint32(16)) & np.uint32(255)).astype(np.float32)
    return (r * F(0.2126) + g * F(0.7152) + b * F(0.0722)) * F(1.0 / 256.0)


# ---------------------------------------------------------------- occupancy

def sphere_params(n, seed, lo, hi, rmin, rmax):
    rng = np.random.default_rng(seed)
    centers = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    radii = rng.uniform(rmin, rmax, n).astype(np.float32)
    return centers, radii


def sphere_boxes(shape, centers, radii):
    """Half-open, clipped voxel boxes (x0, x1, y0, y1, z0, z1) enclosing each sphere."""
    d, h, w = shape
    boxes = []
    for (cx, cy, cz), r in zip(centers, radii):
        boxes.append((max(0, int(math.floor(cx - r)) - 1), min(w, int(math.ceil(cx + r)) + 2),
                      max(0, int(math.floor(cy - r)) - 1), min(h, int(math.ceil(cy + r)) + 2),
                      max(0, int(math.floor(cz - r)) - 1), min(d, int(math.ceil(cz + r)) + 2)))
    return boxes


def occupancy_spheres(shape, centers, radii, occ=None):
    """shape = (d, h, w); returns bool occupancy (d, h, w)."""
    if occ is None:
        occ = np.zeros(shape, bool)
    for (cx, cy, cz), r, (x0, x1, y0, y1, z0, z1) in zip(centers, radii, sphere_boxes(shape, centers, radii)):
        if x0 >= x1 or y0 >= y1 or z0 >= z1:
            continue
        dx = (np.arange(x0, x1, dtype=np.float32) + F(0.5)) - F(cx)
        dy = (np.arange(y0, y1, dtype=np.float32) + F(0.5)) - F(cy)
        dz = (np.arange(z0, z1, dtype=np.float32) + F(0.5)) - F(cz)
        s = (dx[None, None, :] * dx[None, None, :] + dy[None, :, None] * dy[None, :, None]) + \
            dz[:, None, None] * dz[:, None, None]
        occ[z0:z1, y0:y1, x0:x1] |= s <= F(r) * F(r)
    return occ


def value_noise_fbm(n, seed, octaves, base_cells=4):
    """Seeded fractal value noise on an n x n lattice in [0, 1) (float64 math,
    returned as float32).  Octave k uses a (base_cells * 2^k + 1)^2 lattice of
    uniform values, smoothstep-interpolated, with amplitude 2^-k."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, n), np.float64)
    total = 0.0
    coords = (np.arange(n) + 0.5) / n
    for k in range(octaves):
        cells = base_cells << k
        lat = rng.random((cells + 1, cells + 1))
        p = coords * cells
        i = np.minimum(p.astype(np.int64), cells - 1)
        f = p - i
        s = f * f * (3 - 2 * f)
        a = lat[i[:, None], i[None, :]]
        b = lat[i[:, None], i[None, :] + 1]
        c = lat[i[:, None] + 1, i[None, :]]
        d = lat[i[:, None] + 1, i[None, :] + 1]
        top = a + (b - a) * s[None, :]
        bot = c + (d - c) * s[None, :]
        out += (top + (bot - top) * s[:, None]) * 0.5 ** k
        total += 0.5 ** k
    return (out / total).astype(np.float32)


def terrain_heights(n, seed, octaves=5, amplitude=0.3, base=0.1):
    """Heights (in voxels) per (z, x) column: n * (base + amplitude * fbm)."""
    f = value_noise_fbm(n, seed, octaves)
    return (F(n) * (F(base) + F(amplitude) * f)).astype(np.float32)


def occupancy_terrain(shape, heights, thickness=2.0, occ=None):
    """Voxel (x, y, z) is in the shell when h - thickness < y + 0.5 <= h,
    h = heights[z, x]."""
    d, h, w = shape
    if occ is None:
        occ = np.zeros(shape, bool)
    yc = np.arange(h, dtype=np.float32) + F(0.5)
    for z in range(d):
        hz = heights[z, :w]
        occ[z] |= (yc[:, None] <= hz[None, :]) & (yc[:, None] > hz[None, :] - F(thickness))
    return occ


def payload_from_occupancy(occ):
    """uint32 words (0 = empty) from a bool occupancy grid (d, h, w)."""
    d, h, w = occ.shape
    o = np.pad(occ.astype(np.int8), 1)
    nx = (o[1:-1, 1:-1, :-2] - o[1:-1, 1:-1, 2:]).astype(np.float32)
    ny = (o[1:-1, :-2, 1:-1] - o[1:-1, 2:, 1:-1]).astype(np.float32)
    nz = (o[:-2, 1:-1, 1:-1] - o[2:, 1:-1, 1:-1]).astype(np.float32)
    zi, yi, xi = np.nonzero(occ)
    gx, gy, gz = nx[zi, yi, xi], ny[zi, yi, xi], nz[zi, yi, xi]
    flat = (gx == 0) & (gy == 0) & (gz == 0)
    gy = np.where(flat, F(1), gy)
    words = compress_material(gx, gy, gz, hash_shade(xi, yi, zi))
    words[words == 0] = 1
    grid = np.zeros(occ.shape, np.uint32)
    grid[zi, yi, xi] = words
    return grid


# ---------------------------------------------------------------- scenes

def sphere_scene_params(side, n_spheres, seed):
    """The sphere-union scene: centres U[side/8, 7 side/8]^3, radii U[6, 32] * side/256."""
    s = side / 256.0
    return sphere_params(n_spheres, seed, 32 * s, 224 * s, 6 * s, 32 * s)


def terrain_scene_params(side, n_spheres, seed):
    """The terrain scene: 5-octave terrain (amplitude 0.3*side, 2-voxel shell)
    plus spheres with radii U[10, 120] * side/2048 and centres U[0.1, 0.9]*side."""
    heights = terrain_heights(side, seed)
    s = side / 2048.0
    centers, radii = sphere_params(n_spheres, seed + 1000003, 0.1 * side, 0.9 * side, 10 * s, 120 * s)
    return heights, centers, radii


def sphere_scene(side, n_spheres, seed, shape=None):
    centers, radii = sphere_scene_params(side, n_spheres, seed)
    occ = occupancy_spheres(shape or (side, side, side), centers, radii)
    return payload_from_occupancy(occ)


def terrain_scene(side, n_spheres, seed, shape=None):
    shape = shape or (side, side, side)
    heights, centers, radii = terrain_scene_params(side, n_spheres, seed)
    occ = occupancy_terrain(shape, heights)
    occupancy_spheres(shape, centers, radii, occ)
    return payload_from_occupancy(occ)


def random_grid(shape, density, seed):
    rng = np.random.default_rng(seed)
    occ = rng.random(shape) < density
    vals = rng.integers(1, 2 ** 32 - 1, shape, dtype=np.uint64).astype(np.uint32)
    return np.where(occ, vals, 0).astype(np.uint32)


# ---------------------------------------------------------------- cameras

def rot_xyz(rx, ry, rz):
    """Mat4::rotXYZ (math/Mat4.cpp:114-125) rotation block, degrees, float64."""
    r = np.radians([rx, ry, rz])
    c, s = np.cos(r), np.sin(r)
    return np.array([
        [c[1] * c[2], -c[0] * s[2] + s[0] * s[1] * c[2], s[0] * s[2] + c[0] * s[1] * c[2]],
        [c[1] * s[2], c[0] * c[2] + s[0] * s[1] * s[2], -s[0] * c[2] + c[0] * s[1] * s[2]],
        [-s[1], s[0] * c[1], c[0] * c[1]],
    ])


def camera(yaw, pitch, radius, center):
    """Returns the 12 float32 camera values (a11..a33 row-major, then pos)."""
    R = rot_xyz(pitch, 0, 0) @ rot_xyz(0, yaw, 0)
    Rt = R.T  # pseudoInvert of a pure rotation (Mat4.cpp:76-82)
    pos = Rt @ np.array([0.0, 0.0, -radius]) + np.asarray(center, np.float64) + 1.0
    return np.concatenate([Rt.reshape(9), pos]).astype(np.float32)


def viewer_camera(yaw, pitch, radius, center):
    """The orbit camera as the viewer's matrices give it: (rot (9,), trans
    (3,), pos (3,)) float32, with [rot | trans] the inverse model-view matrix
    and pos = (trans + center) + 1 formed in float32 as renderBatch forms its
    eye position (Main.cpp:145)."""
    cam = camera(yaw, pitch, radius, center)
    rot = cam[:9].astype(np.float32)
    trans = (rot.reshape(3, 3).astype(np.float64) @ np.array([0.0, 0.0, -radius])).astype(np.float32)
    pos = ((trans + np.asarray(center, np.float32)).astype(np.float32) + np.float32(1.0)).astype(np.float32)
    return rot, trans, pos


def headlight(cam):
    """Main.cpp:163: normalize(R^T * (-1, 1, -1)), float32."""
    a = cam[:9].reshape(3, 3).astype(np.float32)
    v = np.array([-1, 1, -1], np.float32)
    l = (a[:, 0] * v[0] + a[:, 1] * v[1]) + a[:, 2] * v[2]
    n = F(1) / np.sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2], dtype=np.float32)
    return (l * n).astype(np.float32)


PLANE_DIST = F(1.0) / F(math.tan(F(math.pi) / F(6.0)))


def camera_rays(cam, W, H, x0=0, y0=0, x1=None, y1=None):
    """(n, 6) float32 rays for pixels [x0, x1) x [y0, y1) in row-major order."""
    x1 = W if x1 is None else x1
    y1 = H if y1 is None else y1
    a = cam[:9].astype(np.float32)
    pos = cam[9:12].astype(np.float32)
    scale = F(2.0) / F(W)
    aspect = F(H) / F(W)
    zx, zy, zz = PLANE_DIST * a[2], PLANE_DIST * a[5], PLANE_DIST * a[8]
    xs = np.arange(x0, x1, dtype=np.float32)
    ys = np.arange(y0, y1, dtype=np.float32)
    dx = (F(-1.0) + xs * scale)[None, :]
    dy = (aspect - ys * scale)[:, None]
    vx = (dx * a[0] + dy * a[1]) + zx
    vy = (dx * a[3] + dy * a[4]) + zy
    vz = (dx * a[6] + dy * a[7]) + zz
    n = inv_sqrt((vx * vx + vy * vy) + vz * vz)
    rays = np.empty((y1 - y0, x1 - x0, 6), np.float32)
    rays[..., 0] = pos[0]
    rays[..., 1] = pos[1]
    rays[..., 2] = pos[2]
    rays[..., 3] = vx * n
    rays[..., 4] = vy * n
    rays[..., 5] = vz * n
    return rays.reshape(-1, 6)


def orbit_cameras(n, seed, center, radius=2.0, radius_hi=None, pitch=60.0):
    """n cameras with yaw U[0, 360), pitch U[-pitch, pitch] and radius r
    (or U[radius, radius_hi]) around `center`."""
    rng = np.random.default_rng(seed)
    cams = []
    for _ in range(n):
        yaw = rng.uniform(0, 360)
        pit = rng.uniform(-pitch, pitch)
        r = radius if radius_hi is None else rng.uniform(radius, radius_hi)
        cams.append(camera(yaw, pit, r, center))
    return cams


def batched_views(n_views, seed=3):
    """The batched workload's (octree, view) pairs as (index, side, generator,
    W, H): depth U{7..11}; even index -> sphere-union generator (48 spheres),
    odd -> terrain generator (200 spheres), scene seed = index; one view each,
    pixel count log-uniform in [256x256, 1920x1080] at 16:9, clipped to
    [256, 1920] x [256, 1080]."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(1, n_views + 1):
        depth = int(rng.integers(7, 12))
        pix = float(np.exp(rng.uniform(np.log(256 * 256), np.log(1920 * 1080))))
        W = int(min(1920, max(256, round((pix * 16 / 9) ** 0.5))))
        H = int(min(1080, max(256, round(pix / W))))
        specs.append((i, 1 << depth, "sphere" if i % 2 == 0 else "terrain", W, H))
    return specs


def scene_spec_params(side, generator, seed):
    """(heights or None, centres, radii) of one batched-workload octree."""
    if generator == "sphere":
        centers, radii = sphere_scene_params(side, 48, seed)
        return None, centers, radii
    return terrain_scene_params(side, 200, seed)


def random_rays(n, seed, lo=-1.0, hi=4.0):
    """Rays from U[lo, hi]^3 towards U[1, 2]^3 (unit directions), plus
    axis-aligned and grazing directions in the first rows."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    t = rng.uniform(1.0, 2.0, (n, 3)).astype(np.float32)
    d = t - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    k = n // 16
    d[:k, 0] = 0.0
    d[k:2 * k, 1] = 1e-5
    d[2 * k:3 * k, 2] = -3e-5
    o[3 * k:4 * k] = rng.uniform(1.0, 2.0, (k, 3)).astype(np.float32)  # origins inside the cube
    return np.concatenate([o, d], axis=1).astype(np.float32)


# ---------------------------------------------------------------- GPU generators

_SCENE_LIB = None


def _scene_lib():
    global _SCENE_LIB
    if _SCENE_LIB is None:
        import ctypes
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libsvo_scenes.so")
        if not os.path.exists(path):
            raise ImportError("libsvo_scenes.so is not built")
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.svo_scene_terrain.argtypes = [vp, ctypes.c_int, vp, ctypes.c_float, vp]
        L.svo_scene_spheres.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, vp]
        L.svo_scene_payload.argtypes = [vp, ctypes.c_int, vp, vp]
        L.svo_scene_camera_rays.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp]
        _SCENE_LIB = L
    return _SCENE_LIB


def _chk(rc):
    if rc != 0:
        raise RuntimeError("scene kernel launch failed (cudaError %d)" % rc)


def gpu_occupancy(side, heights=None, centers=None, radii=None, thickness=2.0):
    """Occupancy bitmap (int32 CUDA tensor, 32 voxels per word along x)."""
    import torch
    w32 = max(1, side // 32)
    bm = torch.zeros(w32 * side * side, dtype=torch.int32, device="cuda")
    L = _scene_lib()
    if heights is not None:
        ht = torch.from_numpy(np.ascontiguousarray(heights, np.float32)).cuda()
        _chk(L.svo_scene_terrain(bm.data_ptr(), side, ht.data_ptr(), float(thickness), None))
    if centers is not None and len(centers):
        boxes = np.array(sphere_boxes((side, side, side), centers, radii), np.int32)
        params = np.concatenate([np.asarray(centers, np.float32), np.asarray(radii, np.float32)[:, None]], 1)
        bt = torch.from_numpy(boxes).cuda()
        pt = torch.from_numpy(np.ascontiguousarray(params)).cuda()
        _chk(L.svo_scene_spheres(bm.data_ptr(), side, len(radii), bt.data_ptr(), pt.data_ptr(), None))
        torch.cuda.synchronize()
    return bm


def gpu_payload_grid(bm, side):
    """Dense (side, side, side) int32 CUDA tensor of payload words."""
    import torch
    grid = torch.empty((side, side, side), dtype=torch.int32, device="cuda")
    _chk(_scene_lib().svo_scene_payload(bm.data_ptr(), side, grid.data_ptr(), None))
    return grid


def gpu_sphere_scene(side, n_spheres, seed):
    centers, radii = sphere_scene_params(side, n_spheres, seed)
    return gpu_payload_grid(gpu_occupancy(side, centers=centers, radii=radii), side)


def gpu_terrain_scene(side, n_spheres, seed):
    heights, centers, radii = terrain_scene_params(side, n_spheres, seed)
    return gpu_payload_grid(gpu_occupancy(side, heights, centers, radii), side)


def camera_constants(cam, W, H):
    a = cam[:9].astype(np.float32)
    c = np.zeros(17, np.float32)
    c[:12] = cam[:12]
    c[12] = F(2.0) / F(W)
    c[13] = F(H) / F(W)
    c[14], c[15], c[16] = PLANE_DIST * a[2], PLANE_DIST * a[5], PLANE_DIST * a[8]
    return c


def gpu_camera_rays(cam, W, H, out=None):
    """(H*W, 6) float32 CUDA tensor of camera rays (same bits as camera_rays)."""
    import torch
    c = torch.from_numpy(camera_constants(cam, W, H)).cuda()
    if out is None:
        out = torch.empty((H * W, 6), dtype=torch.float32, device="cuda")
    _chk(_scene_lib().svo_scene_camera_rays(c.data_ptr(), 0, 0, W, H, out.data_ptr(), None))
    torch.cuda.synchronize()
    return out


# ---------------------------------------------------------------- colour field (torch)

def _lattice_value(ix, iy, iz, seed):
    """Hash of integer lattice points to [0, 1) (int64 tensors)."""
    import torch
    m = 0xFFFFFFFF
    h = (ix * 73856093) ^ (iy * 19349663) ^ (iz * 83492791) ^ (seed * 2654435761)
    h = h & m
    h = ((h ^ (h >> 16)) * 0x45D9F3B) & m
    h = ((h ^ (h >> 16)) * 0x45D9F3B) & m
    h = h ^ (h >> 16)
    return (h & 0xFFFFFF).to(torch.float32) / float(1 << 24)


def noise3(p, seed, octaves=3, freq=4.0):
    """Seeded 3-octave value noise in [0, 1) at points p (CUDA float tensor
    (N, 3) in the octree's [1, 2]^3 frame): trilinear smoothstep
    interpolation of hashed lattice values, octave k at frequency freq*2^k
    with amplitude 2^-k."""
    import torch
    total = torch.zeros(p.shape[0], dtype=torch.float32, device=p.device)
    norm = 0.0
    for k in range(octaves):
        q = (p - 1.0) * (freq * (2 ** k))
        qf = torch.floor(q)
        i = qf.to(torch.int64)
        f = q - qf
        s = f * f * (3.0 - 2.0 * f)
        v = 0.0
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    w = (s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1]) * \
                        (s[:, 2] if dz else 1 - s[:, 2])
                    v = v + w * _lattice_value(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed * 31 + k)
        total += v * (0.5 ** k)
        norm += 0.5 ** k
    return total / norm


def decompress_normal(word):
    """Leaf normal of packed words (Util.hpp:86-100 layout), exact
    normalisation; CUDA int64 tensor in, (N, 3) float tensor out."""
    import torch
    sign = ((word >> 31) & 1).to(torch.float32)
    face = (word >> 29) & 3
    u = ((word >> 18) & 0x7FF).to(torch.float32) * 4.8852e-4 * 2.0 - 1.0
    v = ((word >> 7) & 0x7FF).to(torch.float32) * 4.8852e-4 * 2.0 - 1.0
    s = 1.0 - 2.0 * sign
    n = torch.stack([s, u, v], 1)
    n = torch.where((face == 1)[:, None], torch.stack([v, s, u], 1), n)
    n = torch.where((face >= 2)[:, None], torch.stack([u, v, s], 1), n)
    return n / n.norm(dim=1, keepdim=True)


# ---------------------------------------------------------------- triangle meshes (PLY source)

def icosphere(level):
    """Unit icosphere: the icosahedron with every triangle split into four
    `level` times, new vertices pushed out to the sphere (float64).  Level 7
    has 163,842 vertices and 327,680 triangles."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.minimum(e[:, 0], e[:, 1]) * v.shape[0] + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // v.shape[0], uniq % v.shape[0]
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1) + v.shape[0]  # midpoints of edges 01, 12, 20
        v = np.concatenate([v, mid])
        f = np.concatenate([np.stack([f[:, 0], m[0], m[2]], 1), np.stack([f[:, 1], m[1], m[0]], 1),
                            np.stack([f[:, 2], m[2], m[1]], 1), np.stack([m[0], m[1], m[2]], 1)])
    return v, f.astype(np.int32)


def _hash_lattice(ix, iy, iz, seed):
    m = np.uint64(0xFFFFFFFF)
    h = ((ix.astype(np.uint64) * np.uint64(73856093)) ^ (iy.astype(np.uint64) * np.uint64(19349663)) ^
         (iz.astype(np.uint64) * np.uint64(83492791)) ^ np.uint64((seed * 2654435761) & 0xFFFFFFFF)) & m
    h = ((h ^ (h >> np.uint64(16))) * np.uint64(0x45D9F3B)) & m
    h = ((h ^ (h >> np.uint64(16))) * np.uint64(0x45D9F3B)) & m
    h = h ^ (h >> np.uint64(16))
    return (h & np.uint64(0xFFFFFF)).astype(np.float64) / float(1 << 24)


def value_noise3(p, seed, octaves=4, freq=2.0):
    """Seeded fractal value noise in [0, 1) at points p (N, 3) float64:
    smoothstep-trilinear hashed lattice values, octave k at frequency
    freq*2^k with amplitude 2^-k."""
    total = np.zeros(p.shape[0])
    norm = 0.0
    for k in range(octaves):
        q = (p + 4.0) * (freq * 2 ** k)
        i = np.floor(q).astype(np.int64)
        f = q - i
        s = f * f * (3.0 - 2.0 * f)
        v = 0.0
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    w = (s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1]) * \
                        (s[:, 2] if dz else 1 - s[:, 2])
                    v = v + w * _hash_lattice(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed * 31 + k)
        total += v * 0.5 ** k
        norm += 0.5 ** k
    return total / norm


def displaced_icosphere(level, seed, amplitude=0.15, octaves=4):
    """The PLY-build workload's mesh: a level-`level` icosphere radially
    displaced by `octaves`-octave seeded value noise (amplitude a fraction
    of the radius), per-vertex RGB uniform in [0, 255].  Returns
    (positions float32 (V, 3), faces int32 (F, 3), colours uint8 (V, 3))."""
    v, f = icosphere(level)
    r = 1.0 + amplitude * (2.0 * value_noise3(v, seed, octaves) - 1.0)
    pos = (v * r[:, None]).astype(np.float32)
    col = np.random.default_rng(seed).integers(0, 256, size=(v.shape[0], 3), dtype=np.uint8)
    return pos, f, col


def write_ply(path, pos, faces, colors=None, normals=None, binary=True, big_endian=False):
    """Write a PLY mesh: float x, y, z [, nx, ny, nz] [, uchar red, green,
    blue] per vertex and a `list uchar int vertex_indices` per face, as
    binary (little- or big-endian) or ASCII.  faces is (F, k) or a list of
    index lists."""
    pos = np.asarray(pos, np.float32)
    V = pos.shape[0]
    cols = [("x", "f4"), ("y", "f4"), ("z", "f4")]
    if normals is not None:
        cols += [("nx", "f4"), ("ny", "f4"), ("nz", "f4")]
    if colors is not None:
        cols += [("red", "u1"), ("green", "u1"), ("blue", "u1")]
    polys = [list(map(int, fc)) for fc in faces] if not isinstance(faces, np.ndarray) else None
    nf = len(polys) if polys is not None else faces.shape[0]
    fmt = ("binary_big_endian" if big_endian else "binary_little_endian") if binary else "ascii"
    bo = ">" if big_endian else "<"
    hdr = ["ply", "format %s 1.0" % fmt, "element vertex %d" % V]
    hdr += ["property %s %s" % ("float" if t == "f4" else "uchar", n) for n, t in cols]
    hdr += ["element face %d" % nf, "property list uchar int vertex_indices", "end_header"]
    rec = np.zeros(V, dtype=[(n, bo + t if t != "u1" else t) for n, t in cols])
    rec["x"], rec["y"], rec["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
    if normals is not None:
        nrm = np.asarray(normals, np.float32)
        rec["nx"], rec["ny"], rec["nz"] = nrm[:, 0], nrm[:, 1], nrm[:, 2]
    if colors is not None:
        c = np.asarray(colors, np.uint8)
        rec["red"], rec["green"], rec["blue"] = c[:, 0], c[:, 1], c[:, 2]
    with open(path, "wb") as fp:
        fp.write(("\n".join(hdr) + "\n").encode())
        if binary:
            fp.write(rec.tobytes())
            if polys is None:
                fr = np.zeros(nf, dtype=[("n", "u1"), ("i", bo + "i4", (faces.shape[1],))])
                fr["n"] = faces.shape[1]
                fr["i"] = faces
                fp.write(fr.tobytes())
            else:
                for fc in polys:
                    fp.write(np.uint8(len(fc)).tobytes() + np.asarray(fc, bo + "i4").tobytes())
        else:
            lines = []
            for i in range(V):
                lines.append(" ".join(repr(float(rec[n][i])) if t == "f4" else str(int(rec[n][i])) for n, t in cols))
            for fc in (polys if polys is not None else faces.tolist()):
                lines.append(" ".join([str(len(fc))] + [str(int(x)) for x in fc]))
            fp.write(("\n".join(lines) + "\n").encode())


def edge_case_mesh(level, seed):
    """A displaced icosphere plus the polygon cases PlyLoader meets: a
    triangle with a repeated vertex and a collinear triangle (zero area: NaN
    weights and normals), a quad and a pentagon (fan-triangulated), and
    faces with 1 and 2 indices (no triangles).  Returns (positions float32,
    faces as a list of index lists, colours uint8)."""
    pos, f, col = displaced_icosphere(level, seed)
    V = pos.shape[0]
    line = np.array([[0.05, 0.1, 0.2], [0.15, 0.2, 0.3], [0.35, 0.4, 0.5]], np.float32)
    pos = np.concatenate([pos, line])
    rng = np.random.default_rng(seed + 1)
    col = np.concatenate([col, rng.integers(0, 256, (3, 3), dtype=np.uint8)])
    faces = [list(map(int, t)) for t in f]
    faces += [[0, 0, 5], [V, V + 1, V + 2]]
    faces += [[int(f[7, 0]), int(f[7, 1]), int(f[7, 2]), int(f[9, 1])]]
    faces += [[int(f[11, 0]), int(f[11, 1]), int(f[11, 2]), int(f[13, 2]), int(f[15, 0])]]
    faces += [[3], [4, 6]]
    return pos, faces, col
