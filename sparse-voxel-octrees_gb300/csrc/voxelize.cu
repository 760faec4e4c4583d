// voxelize.cu — GPU mesh-to-octree build: PlyLoader + VoxelData(PlyLoader*,
// side, mem) + VoxelOctree(VoxelData*) (PlyLoader.cpp:226-504,
// VoxelData.cpp:50-56, 120-175, 262-289, VoxelOctree.cpp:125-205).
//
// The reference voxelizes one cache block at a time into a buffer that is
// never cleared between blocks: each block's triangles are taken from the
// lists of its sub-blocks (the cache block cut into one part per worker
// thread), every voxel of a triangle's clamped bounding box that passes the
// triangle/box test receives a running-average material write, and the
// octree walk then reads the block's voxels destructively, which leaves only
// voxels the walk never reaches (the dropped last z slice of an odd-depth
// block) behind for later blocks.  This file computes the same result:
//
//  1. Triangle setup (one thread per triangle): rescale to the unit cube,
//     gather the fan triangle's vertices, flat normal when the file has none,
//     bounds (PlyLoader.cpp:40-53, 167-224).
//  2. Sub-block lists (one thread per triangle): the cells of
//     iterateOverlappingBlocks (PlyLoader.cpp:233-270), culled by the same
//     triangle/box test with the same incrementally accumulated centres; each
//     member cell marks its cache block non-empty (isBlockEmpty) and emits
//     one (brick, triangle) pair per 8^3 brick (smaller when sub-blocks are)
//     of the cell that the triangle's clamped voxel box touches.
//  3. A stable radix sort of the pairs by brick (sort.cuh): each brick's
//     triangles in ascending index, the order a sub-block list holds them.
//  4. Cache blocks in the reference's visiting order (ascending Morton code
//     of the blocks the lists mark), each against the one persistent
//     buffer: one warp per brick folds the brick's triangles in order with
//     writeTriangleCell's blend (PlyLoader.cpp:296-336), its lanes covering
//     each triangle's clamped box inside the brick; voxel-box centres are
//     the reference's running sums (lo - 0.5) * h + h + ... + h, read from a
//     table of those sums.  Then the block's nonzero words are extracted in
//     Morton order and cleared, except a dropped odd last slice, from the
//     bricks that can hold any: the folded ones and those under earlier
//     blocks' dropped slices.
//  5. The octree from the Morton-ordered voxels and the block flags
//     (build_from_sorted_device).
#include <algorithm>
#include <memory>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mesh.h"
#include "morton.cuh"
#include "scan.cuh"
#include "sort.cuh"
#include "svo_device.cuh"
#include "svo_internal.h"

// Device-resident triangle mesh (after PlyLoader's rescale and
// triangulation).
struct svo_mesh {
    float *d_tris = nullptr;  // kTriFloats per triangle, see TriLayout
    uint64_t n_tris = 0;
    float lower[3] = {0, 0, 0}, upper[3] = {0, 0, 0};  // PlyLoader::_lower/_upper after rescale
    int has_normals = 0;
    int device = 0;
};

namespace svo {
namespace {

// Per triangle: p0 p1 p2 (9), n0 n1 n2 (9), c0 c1 c2 (9), lower (3),
// upper (3), padding (3).
constexpr int kTriFloats = 36;
constexpr int kTriP = 0, kTriN = 9, kTriC = 18, kTriLo = 27, kTriHi = 30;
constexpr int kStageFloats = 27;  // p, n, c: what the fold kernel stages

#define SVO_LAUNCH_OK(name)                                                    \
    do {                                                                       \
        cudaError_t _e = cudaGetLastError();                                   \
        if (_e != cudaSuccess) return ::svo::cuda_fail(_e, "launch of " name); \
    } while (0)

inline unsigned grid_for(uint64_t n, int t = 256) {
    uint64_t b = (n + t - 1) / t;
    if (b == 0) b = 1;
    return (unsigned)(b < (1u << 30) ? b : (1u << 30));
}

template <typename T>
struct Dev {
    T *p = nullptr;
    cudaStream_t st = nullptr;
    Dev() = default;
    Dev(const Dev &) = delete;
    Dev &operator=(const Dev &) = delete;
    cudaError_t alloc(uint64_t n, cudaStream_t s) {
        st = s;
        return scratch_alloc((void **)&p, (size_t)(n ? n : 1) * sizeof(T), s);
    }
    void release() {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
    }
    ~Dev() { release(); }
};

#define SVO_ALLOC(buf, n)                                                          \
    do {                                                                           \
        cudaError_t _e = (buf).alloc((n), st);                                     \
        if (_e != cudaSuccess) return ::svo::cuda_fail(_e, "device allocation in mesh build"); \
    } while (0)

// ---- triangle/box overlap ---------------------------------------------------

// Separating-axis triangle/box test of Akenine-Moller ("Fast 3D
// triangle-box overlap testing", 2001) in the form third-party/tribox3.c:
// 132-206 evaluates it: the nine edge-axis tests first (projections of two
// vertices per axis, with that code's choice of which vertex is tested
// first for the min), then the box axes, then the triangle's plane.
__device__ __forceinline__ bool axis_sep(float pa, float pb, bool a_first, float rad) {
    float mn, mx;
    if (a_first) {
        if (pa < pb) { mn = pa; mx = pb; } else { mn = pb; mx = pa; }
    } else {
        if (pb < pa) { mn = pb; mx = pa; } else { mn = pa; mx = pb; }
    }
    return mn > rad || mx < -rad;
}

__device__ __forceinline__ bool plane_box(const float n[3], const float v[3], const float h[3]) {
    float vmin[3], vmax[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
        if (n[q] > 0.0f) {
            vmin[q] = -h[q] - v[q];
            vmax[q] = h[q] - v[q];
        } else {
            vmin[q] = h[q] - v[q];
            vmax[q] = -h[q] - v[q];
        }
    }
    if (n[0] * vmin[0] + n[1] * vmin[1] + n[2] * vmin[2] > 0.0f) return false;
    if (n[0] * vmax[0] + n[1] * vmax[1] + n[2] * vmax[2] >= 0.0f) return true;
    return false;
}

__device__ __forceinline__ bool tri_box(float cx, float cy, float cz, const float h[3], const float *tv) {
    const float v0[3] = {tv[0] - cx, tv[1] - cy, tv[2] - cz};
    const float v1[3] = {tv[3] - cx, tv[4] - cy, tv[5] - cz};
    const float v2[3] = {tv[6] - cx, tv[7] - cy, tv[8] - cz};
    const float e0[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    const float e1[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
    const float e2[3] = {v0[0] - v2[0], v0[1] - v2[1], v0[2] - v2[2]};
    float fex, fey, fez, a, b;

    fex = fabsf(e0[0]); fey = fabsf(e0[1]); fez = fabsf(e0[2]);
    a = e0[2]; b = e0[1];
    if (axis_sep(a * v0[1] - b * v0[2], a * v2[1] - b * v2[2], true, fez * h[1] + fey * h[2])) return false;
    a = e0[2]; b = e0[0];
    if (axis_sep(-a * v0[0] + b * v0[2], -a * v2[0] + b * v2[2], true, fez * h[0] + fex * h[2])) return false;
    a = e0[1]; b = e0[0];
    if (axis_sep(a * v1[0] - b * v1[1], a * v2[0] - b * v2[1], false, fey * h[0] + fex * h[1])) return false;

    fex = fabsf(e1[0]); fey = fabsf(e1[1]); fez = fabsf(e1[2]);
    a = e1[2]; b = e1[1];
    if (axis_sep(a * v0[1] - b * v0[2], a * v2[1] - b * v2[2], true, fez * h[1] + fey * h[2])) return false;
    a = e1[2]; b = e1[0];
    if (axis_sep(-a * v0[0] + b * v0[2], -a * v2[0] + b * v2[2], true, fez * h[0] + fex * h[2])) return false;
    a = e1[1]; b = e1[0];
    if (axis_sep(a * v0[0] - b * v0[1], a * v1[0] - b * v1[1], true, fey * h[0] + fex * h[1])) return false;

    fex = fabsf(e2[0]); fey = fabsf(e2[1]); fez = fabsf(e2[2]);
    a = e2[2]; b = e2[1];
    if (axis_sep(a * v0[1] - b * v0[2], a * v1[1] - b * v1[2], true, fez * h[1] + fey * h[2])) return false;
    a = e2[2]; b = e2[0];
    if (axis_sep(-a * v0[0] + b * v0[2], -a * v1[0] + b * v1[2], true, fez * h[0] + fex * h[2])) return false;
    a = e2[1]; b = e2[0];
    if (axis_sep(a * v1[0] - b * v1[1], a * v2[0] - b * v2[1], false, fey * h[0] + fex * h[1])) return false;

    const float *vv[3] = {v0, v1, v2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float mn = vv[0][k], mx = vv[0][k];
        if (vv[1][k] < mn) mn = vv[1][k];
        if (vv[1][k] > mx) mx = vv[1][k];
        if (vv[2][k] < mn) mn = vv[2][k];
        if (vv[2][k] > mx) mx = vv[2][k];
        if (mn > h[k] || mx < -h[k]) return false;
    }
    const float n[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
    return plane_box(n, v0, h);
}

// ---- 1. triangle setup ---------------------------------------------------------

__global__ void k_mesh_setup(uint64_t n_tris, const int32_t *__restrict__ tri_idx, const float *__restrict__ pos,
                             const float *__restrict__ nrm, const float *__restrict__ col, float lx, float ly,
                             float lz, float factor, float *__restrict__ out) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tris) return;
    const float low[3] = {lx, ly, lz};
    float p[9], n[9], c[9];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        uint64_t v = (uint64_t)tri_idx[3 * t + j];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            p[3 * j + k] = (pos[3 * v + k] - low[k]) * factor;  // (pos - _lower) * factor
            c[3 * j + k] = col[3 * v + k];
            n[3 * j + k] = nrm ? nrm[3 * v + k] : 0.0f;
        }
    }
    if (!nrm) {  // (v1 - v0).cross(v2 - v0).normalize(), PlyLoader.cpp:213-218
        float ax = p[3] - p[0], ay = p[4] - p[1], az = p[5] - p[2];
        float bx = p[6] - p[0], by = p[7] - p[1], bz = p[8] - p[2];
        float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
        float inv = 1.0f / sqrtf(cx * cx + cy * cy + cz * cz);
        cx *= inv;
        cy *= inv;
        cz *= inv;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            n[3 * j] = cx;
            n[3 * j + 1] = cy;
            n[3 * j + 2] = cz;
        }
    }
    float *o = out + t * kTriFloats;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        o[kTriP + k] = p[k];
        o[kTriN + k] = n[k];
        o[kTriC + k] = c[k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        o[kTriLo + k] = smin(p[k], smin(p[3 + k], p[6 + k]));
        o[kTriHi + k] = smax(p[k], smax(p[3 + k], p[6 + k]));
    }
    o[33] = o[34] = o[35] = 0.0f;
}

// ---- 2. sub-block lists -> (brick, triangle) pairs -------------------------------

struct ListGeom {
    float grid_scale;        // float(sideLength - 2) of PlyLoader::pointToGrid
    float cell_h[3];         // _subBlock{W,H,D} / float(sideLength - 2)
    int sub[3];              // sub-block edges
    int part[3];             // partitions per cache block and axis
    int grid[3];             // _gridW/H/D
    int dims[3];             // volume W/H/D
    int log_e;               // brick edge 2^log_e
    int log_block;           // cache-block edge 2^log_block
    uint64_t n_blocks;       // Morton-indexed block flags (z-slabs in slab mode)
    int slab_mode;           // 1: blocks are z-slabs of part[2] cell layers (convertToVolume), block
                             // index = gz / part[2], and pair keys carry it above brick_bits
    int brick_bits;          // bits of a brick's Morton key
};

__device__ __forceinline__ int point_to_grid(float p, float s) { return (int)(p * s + 1.0f); }

// mode 0: count pairs per triangle (and store the triangle's voxel box,
// mark blocks); mode 1: emit pairs at out_off[t].
template <int kMode>
__global__ void k_tri_pairs(uint64_t n_tris, const float *__restrict__ tris, ListGeom g, int32_t *__restrict__ box,
                            uint8_t *__restrict__ block_flag, uint32_t *__restrict__ count,
                            const uint64_t *__restrict__ out_off, uint32_t *__restrict__ pair_key,
                            uint32_t *__restrict__ pair_tri, uint32_t *__restrict__ pair_cell,
                            uint32_t *__restrict__ err) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tris) return;
    const float *T = tris + t * kTriFloats;
    int lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = point_to_grid(T[kTriLo + k], g.grid_scale);
        hi[k] = point_to_grid(T[kTriHi + k], g.grid_scale);
    }
    if (kMode == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            box[6 * t + k] = lo[k];
            box[6 * t + 3 + k] = hi[k];
        }
    }
    float tv[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) tv[k] = T[kTriP + k];
    int lg[3], ug[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lg[k] = lo[k] / g.sub[k];
        ug[k] = (hi[k] + 1) / g.sub[k];
    }
    const int max_side = max(ug[0] - lg[0], max(ug[1] - lg[1], ug[2] - lg[2]));
    uint32_t n = 0;
    uint64_t o = kMode == 1 ? out_off[t] : 0;

    auto member = [&](int gx, int gy, int gz) {
        if (gx < 0 || gy < 0 || gz < 0 || gx >= g.grid[0] || gy >= g.grid[1] || gz >= g.grid[2]) {
            atomicOr(err, 1u);  // the reference would index past its block offsets
            return;
        }
        const uint32_t slab = g.slab_mode ? (uint32_t)(gz / g.part[2]) : 0u;
        if (kMode == 0) {
            uint64_t blk = g.slab_mode ? (uint64_t)slab
                                       : morton3((uint32_t)(gx / g.part[0]), (uint32_t)(gy / g.part[1]),
                                                 (uint32_t)(gz / g.part[2]));
            if (blk < g.n_blocks) block_flag[blk] = 1;
            else atomicOr(err, 2u);
        }
        const int c0[3] = {gx * g.sub[0], gy * g.sub[1], gz * g.sub[2]};
        int a[3], b[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            a[k] = max(lo[k], c0[k]);
            b[k] = min(hi[k], min(c0[k] + g.sub[k] - 1, g.dims[k] - 1));
        }
        if (a[0] > b[0] || a[1] > b[1] || a[2] > b[2]) return;
        for (int bz = a[2] >> g.log_e; bz <= (b[2] >> g.log_e); ++bz)
            for (int by = a[1] >> g.log_e; by <= (b[1] >> g.log_e); ++by)
                for (int bx = a[0] >> g.log_e; bx <= (b[0] >> g.log_e); ++bx) {
                    if (kMode == 1) {
                        pair_key[o + n] = (slab << g.brick_bits) | (uint32_t)morton3((uint32_t)bx, (uint32_t)by, (uint32_t)bz);
                        pair_tri[o + n] = (uint32_t)t;
                        pair_cell[o + n] = (uint32_t)gx + (uint32_t)g.grid[0] * ((uint32_t)gy + (uint32_t)g.grid[1] * (uint32_t)gz);
                    }
                    ++n;
                }
    };

    if (max_side > 0) {
        const float half[3] = {0.5f * g.cell_h[0], 0.5f * g.cell_h[1], 0.5f * g.cell_h[2]};
        float cz = ((float)lg[2] + 0.5f) * g.cell_h[2];
        for (int z = lg[2]; z <= ug[2]; ++z, cz += g.cell_h[2]) {
            float cy = ((float)lg[1] + 0.5f) * g.cell_h[1];
            for (int y = lg[1]; y <= ug[1]; ++y, cy += g.cell_h[1]) {
                float cx = ((float)lg[0] + 0.5f) * g.cell_h[0];
                for (int x = lg[0]; x <= ug[0]; ++x, cx += g.cell_h[0])
                    if (tri_box(cx, cy, cz, half, tv)) member(x, y, z);
            }
        }
    } else {
        member(lg[0], lg[1], lg[2]);
    }
    if (kMode == 0) count[t] = n;
}

__global__ void k_iota(uint32_t *__restrict__ v, uint64_t n) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (uint32_t)i;
}

__global__ void k_gather_pairs(const uint32_t *__restrict__ idx, uint64_t n, const uint32_t *__restrict__ tri,
                               const uint32_t *__restrict__ cell, uint32_t *__restrict__ stri,
                               uint32_t *__restrict__ scell) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t k = idx[i];
    stri[i] = tri[k];
    scell[i] = cell[k];
}

// Unique bricks of the sorted pairs.
__global__ void k_heads_u32(const uint32_t *__restrict__ key, uint64_t n, uint32_t *__restrict__ head) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) head[i] = (i == 0 || key[i] != key[i - 1]) ? 1u : 0u;
}

__global__ void k_brick_table(const uint32_t *__restrict__ key, uint64_t n, const uint32_t *__restrict__ head,
                              const uint32_t *__restrict__ hidx, uint32_t *__restrict__ bkey,
                              uint32_t *__restrict__ bstart) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !head[i]) return;
    bkey[hidx[i]] = key[i];
    bstart[hidx[i]] = (uint32_t)i;
}

// Per cache block: [first, last) of its bricks in the unique-brick table.
__global__ void k_block_ranges(const uint32_t *__restrict__ bkey, uint32_t nb, int shift, uint64_t n_blocks,
                               uint32_t *__restrict__ rfirst, uint32_t *__restrict__ rlast, uint32_t *__restrict__ err) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nb) return;
    uint32_t blk = bkey[j] >> shift;
    if (blk >= n_blocks) {
        atomicOr(err, 4u);
        return;
    }
    if (j == 0 || (bkey[j - 1] >> shift) != blk) rfirst[blk] = j;
    if (j == nb - 1 || (bkey[j + 1] >> shift) != blk) rlast[blk] = j + 1;
}

__global__ void k_flag_to_u32(const uint8_t *__restrict__ f, uint64_t n, uint32_t *__restrict__ out) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = f[i] ? 1u : 0u;
}

__global__ void k_gather_blocks(const uint8_t *__restrict__ flag, uint64_t n, const uint32_t *__restrict__ idx,
                                const uint32_t *__restrict__ rfirst, const uint32_t *__restrict__ rlast,
                                uint32_t *__restrict__ out) {
    uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n || !flag[b]) return;
    uint32_t k = idx[b];
    out[3 * k] = (uint32_t)b;
    out[3 * k + 1] = rfirst[b];
    out[3 * k + 2] = rlast[b];
}

// Running centres: acc[l * K + k] = ((l - 0.5) * h) + h + ... (k additions),
// the value the reference's loop holds at voxel l + k (PlyLoader.cpp:363-368).
__global__ void k_center_table(int n_l, int K, float h, float *__restrict__ acc) {
    int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n_l) return;
    float c = ((float)l - 0.5f) * h;
    float *row = acc + (uint64_t)l * K;
    for (int k = 0; k < K; ++k) {
        row[k] = c;
        c += h;
    }
}

// ---- 4. per-block brick fold ------------------------------------------------------

struct FoldArgs {
    const float *tris;
    const int32_t *box;
    const uint32_t *pair_tri;   // per sorted pair: triangle ...
    const uint32_t *pair_cell;  // ... and the sub-block cell whose list it came from
    const uint32_t *bkey;
    const uint32_t *bstart;  // nb + 1 entries
    uint32_t b_first, b_last;
    int log_e;
    int sub[3];
    int grid[3];  // sub-block cells per axis (PlyLoader::_gridW/H/D)
    int org[3];   // block origin
    int buf[3];   // clamped block dims (the buffer's W/H/D for this block)
    const float *acc;
    int K;
    float half;
    uint32_t *data;
    uint8_t *counts;
    uint32_t *next;  // work counter of this launch (zero at launch): bricks taken so far
    uint32_t brick_mask;  // the brick's Morton key within a pair key (slab mode keys carry the slab above it)
    // Optional: per brick of the block (Morton index of the brick relative to
    // org), nonzero where the buffer may hold a nonzero word before this
    // fold.  A brick marked 0 starts from zeros and is not read.
    const uint8_t *pre_dirty;
    uint64_t n_pre;
    // Optional (the octree build's blocks): per brick of the block, set to 2
    // (folded here) with the count of its nonzero words outside the dropped
    // last slice (drop_z, or -1), the voxels the extraction will emit.
    uint8_t *brick_flag;
    uint32_t *brick_count;
    uint32_t *brick_bits;  // and, 16 words per brick, which of its 512 cells those are
    int drop_z;
    // The direct fold (every brick starts from zeros): each brick's block
    // comes from its key (blocks of edge 2^log_block clamped to dims), and
    // brick j's voxels go to slot[j * E^3 ...] in Morton order, with their
    // count and cell bits at brick_count[j] and brick_bits[j * 16].
    int dims[3];
    int log_block;
    uint32_t *slot;
};

// PlyLoader::writeTriangleCell on a register copy of one buffer cell.
__device__ __forceinline__ void write_cell(uint32_t &w, uint32_t &cnt, float cx, float cy, float cz, const float *T) {
    const float *p = T + kTriP, *nv = T + kTriN, *cv = T + kTriC;
    // Triangle::barycentric (PlyLoader.cpp:55-64)
    float f1x = p[0] - cx, f1y = p[1] - cy, f1z = p[2] - cz;
    float f2x = p[3] - cx, f2y = p[4] - cy, f2z = p[5] - cz;
    float f3x = p[6] - cx, f3y = p[7] - cy, f3z = p[8] - cz;
    float ax = p[0] - p[3], ay = p[1] - p[4], az = p[2] - p[5];
    float bx = p[0] - p[6], by = p[1] - p[7], bz = p[2] - p[8];
    float qx = ay * bz - az * by, qy = az * bx - ax * bz, qz = ax * by - ay * bx;
    float area = sqrtf(qx * qx + qy * qy + qz * qz);
    qx = f2y * f3z - f2z * f3y;
    qy = f2z * f3x - f2x * f3z;
    qz = f2x * f3y - f2y * f3x;
    float l1 = sqrtf(qx * qx + qy * qy + qz * qz) / area;
    qx = f3y * f1z - f3z * f1y;
    qy = f3z * f1x - f3x * f1z;
    qz = f3x * f1y - f3y * f1x;
    float l2 = sqrtf(qx * qx + qy * qy + qz * qz) / area;
    if (!(l1 >= 0.0f && l2 >= 0.0f && l1 + l2 <= 1.0f)) {
        l1 = smin(smax(l1, 0.0f), 1.0f);
        l2 = smin(smax(l2, 0.0f), 1.0f);
        float tau = l1 + l2;
        if (tau > 1.0f) {
            l1 /= tau;
            l2 /= tau;
        }
    }
    float l3 = 1.0f - l1 - l2;
    float nx = nv[0] * l1 + nv[3] * l2 + nv[6] * l3;
    float ny = nv[1] * l1 + nv[4] * l2 + nv[7] * l3;
    float nz = nv[2] * l1 + nv[5] * l2 + nv[8] * l3;
    float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
    nx *= inv;
    ny *= inv;
    nz *= inv;
    float r = cv[0] * l1 + cv[3] * l2 + cv[6] * l3;
    float gg = cv[1] * l1 + cv[4] * l2 + cv[7] * l3;
    float b = cv[2] * l1 + cv[5] * l2 + cv[8] * l3;
    float shade = (r * 0.2126f + gg * 0.7152f + b * 0.0722f) * (1.0f / 256.0f);
    if (w == 0) {
        cnt = 1;
        w = compress_material(nx, ny, nz, shade);
    } else {
        float cur = (float)cnt / ((float)cnt + 1.0f);
        float nr = 1.0f - cur;
        float cnx, cny, cnz, cs;
        decompress_material(w, cnx, cny, cnz, cs);
        float mx = cnx * cur + nx * nr, my = cny * cur + ny * nr, mz = cnz * cur + nz * nr;
        float ms = cs * cur + shade * nr;
        if (mx * mx + my * my + mz * mz < 1e-3f) {
            mx = cnx;
            my = cny;
            mz = cnz;
        }
        w = compress_material(mx, my, mz, ms);
        cnt = cnt + 1 < 255 ? cnt + 1 : 255;
    }
}

constexpr int kFoldWarps = 4;   // warps per CTA of the fold kernel
constexpr int kFoldChunk = 8;   // pairs a warp stages per round (8-bit hit masks)

struct FoldSmem {
    float T[kFoldChunk][kStageFloats];  // p, n, c
    int lo[kFoldChunk][3];              // running-sum start: max(triangle box low, sub-block start)
    int box[kFoldChunk][6];             // brick-local inclusive range of the clamped box
    int pre[kFoldChunk + 1];            // prefix of the boxes' voxel counts
    float C[kFoldChunk][3][8];          // running centres of the brick's E coordinates per axis
    uint32_t w[512];                    // the brick's buffer words ...
    uint8_t cnt[512];                   // ... and counts (PlyLoader::_counts)
    uint32_t mask[128];                 // per voxel, 8 bits: which staged pairs hit it
    uint16_t list[512];                 // voxels with any hit in this round
    uint32_t touched[16];
};

// v / n and v % n for v < 1024, n <= 8 by a 16-bit fixed-point reciprocal
// (exact: the error v / 2^16 stays below 1/n minus the largest fraction).
__device__ __forceinline__ void divmod_small(int v, int n, int rcp, int &q, int &r) {
    q = (v * rcp) >> 16;
    r = v - q * n;
}

// One warp per brick.  The warp loads the brick's buffer cells, then takes
// the brick's (triangle, sub-block) pairs in list order, 16 per round:
//   1. every (pair, voxel of the pair's clamped box inside the brick) item of
//      the round is spread over the lanes and tested (triangleToVolume's loop
//      nest, PlyLoader.cpp:338-374), hits recorded as a per-voxel bit mask;
//   2. the voxels with hits are compacted and each lane folds one voxel's
//      hits in pair order with writeTriangleCell (PlyLoader.cpp:296-336).
// A voxel lies in exactly one sub-block, so only pairs of its own cell reach
// it, in ascending triangle order as that cell's list holds them.
template <bool kDirect>
__global__ void __launch_bounds__(kFoldWarps * 32, 8) k_fold_bricks(FoldArgs a) {
    __shared__ FoldSmem smem[kFoldWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    FoldSmem &sm = smem[wid];
    const int le = a.log_e, E = 1 << le, E3 = 1 << (3 * le);
    const float hv[3] = {a.half, a.half, a.half};
    int end0 = a.org[0] + a.buf[0], end1 = a.org[1] + a.buf[1], end2 = a.org[2] + a.buf[2];
    int drop_z = a.drop_z;
    const uint32_t lt = (1u << lane) - 1u;
    // Warps take bricks from a counter: a brick's cost grows with its
    // triangles, and a fixed stride left most warps idle behind the few that
    // drew the heaviest bricks.  Bricks own disjoint buffer cells, so the
    // order they are folded in does not change the result.
    for (;;) {
        uint32_t jt = 0;
        if (lane == 0) jt = atomicAdd(a.next, 1u);
        const uint32_t j = a.b_first + __shfl_sync(0xffffffffu, jt, 0);
        if (j >= a.b_last) break;
        const uint32_t key = a.bkey[j] & a.brick_mask;
        const int ox = (int)(compact3(key) << le), oy = (int)(compact3((uint64_t)key >> 1) << le),
                  oz = (int)(compact3((uint64_t)key >> 2) << le);
        // a brick the buffer holds only zeros for is not read (the extraction
        // cleared what earlier blocks left, except their dropped slices)
        bool clean = kDirect;
        uint64_t pm = ~0ull;  // the brick's Morton index within the block
        if (kDirect) {
            // the brick's block: its bounds and dropped slice (VoxelData.cpp:163-170)
            const int lb = a.log_block, B = 1 << lb;
            const uint64_t blk = (uint64_t)key >> (3 * (lb - le));
            const int bx = (int)(compact3(blk) << lb), by = (int)(compact3(blk >> 1) << lb),
                      bz = (int)(compact3(blk >> 2) << lb);
            end0 = min(bx + B, a.dims[0]);
            end1 = min(by + B, a.dims[1]);
            end2 = min(bz + B, a.dims[2]);
            drop_z = (((end2 - bz) & 1) && end2 > bz && lb >= 2) ? end2 - 1 : -1;
        } else {
            if (ox >= a.org[0] && oy >= a.org[1] && oz >= a.org[2])
                pm = morton3((uint32_t)((ox - a.org[0]) >> le), (uint32_t)((oy - a.org[1]) >> le),
                             (uint32_t)((oz - a.org[2]) >> le));
            if (a.pre_dirty) clean = pm < a.n_pre && a.pre_dirty[pm] == 0;
        }
        __syncwarp();
        for (int i = lane; i < E3; i += 32) {
            int x = ox + (i & (E - 1)), y = oy + ((i >> le) & (E - 1)), z = oz + (i >> (2 * le));
            uint32_t wv = 0, cv = 0;
            // a slab's bricks may start below its first slice (z-slabs need not be brick-aligned)
            if (!clean && x >= a.org[0] && y >= a.org[1] && z >= a.org[2] && x < end0 && y < end1 && z < end2) {
                uint64_t bi = (uint64_t)(x - a.org[0]) +
                              (uint64_t)a.buf[0] * ((uint64_t)(y - a.org[1]) + (uint64_t)a.buf[1] * (uint64_t)(z - a.org[2]));
                wv = a.data[bi];
                cv = a.counts[bi];
            }
            sm.w[i] = wv;
            sm.cnt[i] = (uint8_t)cv;
        }
        if (lane < 16) sm.touched[lane] = 0;
        const uint32_t s0 = a.bstart[j], s1 = a.bstart[j + 1];
        for (uint32_t c0 = s0; c0 < s1; c0 += kFoldChunk) {
            const int nc = (int)min((uint32_t)kFoldChunk, s1 - c0);
            __syncwarp();
            for (int i = lane; i < nc * kStageFloats; i += 32) {
                int q = i / kStageFloats, f = i - q * kStageFloats;
                sm.T[q][f] = a.tris[(uint64_t)a.pair_tri[c0 + q] * kTriFloats + f];
            }
            for (int i = lane; i < ((E3 + 3) >> 2); i += 32) sm.mask[i] = 0;
            int items = 0;
            if (lane < nc) {
                const int32_t *bx = a.box + (uint64_t)a.pair_tri[c0 + lane] * 6;
                const uint32_t cell = a.pair_cell[c0 + lane];
                const int g0 = (int)(cell % (uint32_t)a.grid[0]), g12 = (int)(cell / (uint32_t)a.grid[0]);
                const int g1 = g12 % a.grid[1], g2 = g12 / a.grid[1];
                const int o[3] = {ox, oy, oz}, st3[3] = {g0 * a.sub[0], g1 * a.sub[1], g2 * a.sub[2]};
                const int en[3] = {end0, end1, end2};
                items = 1;
#pragma unroll
                for (int ax = 0; ax < 3; ++ax) {
                    int lo = max(bx[ax], st3[ax]);                                // PlyLoader.cpp:344-346
                    int hi = min(bx[3 + ax], min(st3[ax] + a.sub[ax], en[ax]) - 1);  // :347-349
                    int b0 = max(lo, o[ax]) - o[ax], b1 = min(hi, o[ax] + E - 1) - o[ax];
                    sm.lo[lane][ax] = lo;
                    sm.box[lane][ax] = b0;
                    sm.box[lane][3 + ax] = b1;
                    items *= max(0, b1 - b0 + 1);
                }
            }
            // exclusive prefix of the items over the staged pairs
            int incl = items;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int n = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += n;
            }
            if (lane < nc) sm.pre[lane] = incl - items;
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            __syncwarp();
            for (int i = lane; i < nc * 3 * E; i += 32) {
                int q = i / (3 * E), r = i - q * 3 * E, ax = r / E, k = r - ax * E;
                int ov = ax == 0 ? ox : (ax == 1 ? oy : oz);
                int lo = sm.lo[q][ax];
                float c = 0.0f;
                if (k >= sm.box[q][ax] && k <= sm.box[q][3 + ax]) c = a.acc[(uint64_t)lo * a.K + (ov + k - lo)];
                sm.C[q][ax][k] = c;
            }
            __syncwarp();
            // 1. tests
            for (int it = lane; it < total; it += 32) {
                int q = 0;
#pragma unroll
                for (int step = kFoldChunk / 2; step; step >>= 1)
                    if (q + step < nc && sm.pre[q + step] <= it) q += step;
                const int v = it - sm.pre[q];
                const int bx0 = sm.box[q][0], by0 = sm.box[q][1], bz0 = sm.box[q][2];
                const int nx = sm.box[q][3] - bx0 + 1, ny = sm.box[q][4] - by0 + 1;
                int r, ix, iy, iz;
                divmod_small(v, nx, (65536 + nx - 1) / nx, r, ix);
                divmod_small(r, ny, (65536 + ny - 1) / ny, iz, iy);
                ix += bx0;
                iy += by0;
                iz += bz0;
                if (tri_box(sm.C[q][0][ix], sm.C[q][1][iy], sm.C[q][2][iz], hv, &sm.T[q][kTriP])) {
                    const int idx = ix + (iy << le) + (iz << (2 * le));
                    atomicOr(&sm.mask[idx >> 2], 1u << (q + ((idx & 3) << 3)));
                }
            }
            __syncwarp();
            // 2. compaction of the voxels with hits, then the ordered fold
            int nhit = 0;
            for (int b0 = 0; b0 < E3; b0 += 32) {
                const int idx = b0 + lane;
                const bool hit = idx < E3 && ((sm.mask[idx >> 2] >> ((idx & 3) << 3)) & 0xFFu) != 0;
                const uint32_t ball = __ballot_sync(0xffffffffu, hit);
                if (hit) sm.list[nhit + __popc(ball & lt)] = (uint16_t)idx;
                nhit += __popc(ball);
            }
            __syncwarp();
            for (int k = lane; k < nhit; k += 32) {
                const int idx = sm.list[k];
                uint32_t m = (sm.mask[idx >> 2] >> ((idx & 3) << 3)) & 0xFFu;
                const int ix = idx & (E - 1), iy = (idx >> le) & (E - 1), iz = idx >> (2 * le);
                uint32_t wv = sm.w[idx], cv = sm.cnt[idx];
                while (m) {
                    const int q = __ffs(m) - 1;
                    m &= m - 1;
                    write_cell(wv, cv, sm.C[q][0][ix], sm.C[q][1][iy], sm.C[q][2][iz], &sm.T[q][0]);
                }
                sm.w[idx] = wv;
                sm.cnt[idx] = (uint8_t)cv;
                atomicOr(&sm.touched[idx >> 5], 1u << (idx & 31));
            }
        }
        __syncwarp();
        if constexpr (kDirect) {
            // the brick's voxels outside the dropped slice, in Morton order
            // (shared memory is x-fastest), compacted into its slot
            uint32_t n = 0;
            uint32_t *dst = a.slot + (uint64_t)j * (uint32_t)E3;
            for (int m0 = 0; m0 < E3; m0 += 32) {
                const int m = m0 + lane;
                uint32_t wv = 0;
                if (m < E3) {
                    const int lx = (int)compact3((uint64_t)m), ly = (int)compact3((uint64_t)m >> 1),
                              lz = (int)compact3((uint64_t)m >> 2);
                    const int x = ox + lx, y = oy + ly, z = oz + lz;
                    if (x < end0 && y < end1 && z < end2 && z != drop_z) wv = sm.w[lx + (ly << le) + (lz << (2 * le))];
                }
                const uint32_t bits = __ballot_sync(0xffffffffu, wv != 0);
                if (wv) dst[n + __popc(bits & lt)] = wv;
                if (lane == 0) a.brick_bits[(uint64_t)j * 16 + (uint64_t)(m0 >> 5)] = bits;
                n += (uint32_t)__popc(bits);
            }
            if (lane == 0) a.brick_count[j] = n;
        } else {
            for (int i = lane; i < E3; i += 32) {
                if (!((sm.touched[i >> 5] >> (i & 31)) & 1u)) continue;
                int x = ox + (i & (E - 1)), y = oy + ((i >> le) & (E - 1)), z = oz + (i >> (2 * le));
                if (x < a.org[0] || y < a.org[1] || z < a.org[2] || x >= end0 || y >= end1 || z >= end2) continue;
                uint64_t bi = (uint64_t)(x - a.org[0]) +
                              (uint64_t)a.buf[0] * ((uint64_t)(y - a.org[1]) + (uint64_t)a.buf[1] * (uint64_t)(z - a.org[2]));
                a.data[bi] = sm.w[i];
                a.counts[bi] = sm.cnt[i];
            }
            if (a.brick_count && pm < a.n_pre) {
                // the brick's whole buffer state is in shared memory: words read
                // (or known zero) and folded.  The bits follow the extraction's
                // order, the brick-local Morton index m (shared memory is x-fastest).
                uint32_t n = 0;
                for (int m0 = 0; m0 < E3; m0 += 32) {
                    const int m = m0 + lane;
                    bool on = false;
                    if (m < E3) {
                        const int lx = (int)compact3((uint64_t)m), ly = (int)compact3((uint64_t)m >> 1),
                                  lz = (int)compact3((uint64_t)m >> 2);
                        const int x = ox + lx, y = oy + ly, z = oz + lz;
                        on = x < end0 && y < end1 && z < end2 && z != drop_z && sm.w[lx + (ly << le) + (lz << (2 * le))] != 0;
                    }
                    const uint32_t bits = __ballot_sync(0xffffffffu, on);
                    if (lane == 0) a.brick_bits[pm * 16 + (uint64_t)(m0 >> 5)] = bits;
                    n += (uint32_t)__popc(bits);
                }
                if (lane == 0) {
                    a.brick_count[pm] = n;
                    a.brick_flag[pm] = 2;
                }
            }
        }
    }
}

// Bricks of the block (edge E, Morton-indexed within the block) that may
// hold a nonzero buffer word before the fold: those holding a buffer index of
// an earlier block's dropped slice ([s0, s1) flat), read in this block's
// w x h x d layout.
__global__ void k_mark_range(uint64_t s0, uint64_t s1, int w, int h, int d, int log_e, uint8_t *__restrict__ dirty,
                             uint64_t n_dirty) {
    uint64_t i = s0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s1) return;
    uint64_t x = i % (uint64_t)w, y = (i / (uint64_t)w) % (uint64_t)h, z = i / ((uint64_t)w * (uint64_t)h);
    if (z >= (uint64_t)d) return;
    uint64_t m = morton3((uint32_t)(x >> log_e), (uint32_t)(y >> log_e), (uint32_t)(z >> log_e));
    if (m < n_dirty) dirty[m] = 1;
}

struct ExtractArgs {
    const uint8_t *flag;   // per brick of the block: 0 holds nothing, 1 earlier dropped-slice words only, 2 folded
    uint64_t n_bricks;
    int log_e;
    int buf[3];
    int drop;              // the z == buf[2]-1 slice is never read (VoxelData.cpp:163-170)
    uint64_t key_base;     // Morton key of the block's first voxel
    uint32_t *data;
};

// Voxel m (local Morton index) of brick c: buffer index, or ~0 when the
// voxel lies outside the block or in a dropped slice.
__device__ __forceinline__ uint64_t cand_cell(const ExtractArgs &a, uint32_t c, uint32_t m) {
    const int le = a.log_e;
    int x = (int)((compact3(c) << le) + compact3(m)), y = (int)((compact3((uint64_t)c >> 1) << le) + compact3((uint64_t)m >> 1));
    int z = (int)((compact3((uint64_t)c >> 2) << le) + compact3((uint64_t)m >> 2));
    if (x >= a.buf[0] || y >= a.buf[1] || z >= a.buf[2] || (a.drop && z == a.buf[2] - 1)) return ~0ull;
    return (uint64_t)x + (uint64_t)a.buf[0] * ((uint64_t)y + (uint64_t)a.buf[1] * (uint64_t)z);
}

// Warp w of nw handles bricks w, w + nw, w + 2 nw, ...: every lane reads one
// of those bricks' flags, and the whole warp then runs body(c) for each
// brick c whose flag passes, one after another.  The interleaving spreads
// the flagged bricks, which cluster along the surface, over all warps.
template <typename Pred, typename Body>
__device__ __forceinline__ void for_flagged_bricks(const ExtractArgs &a, Pred pred, Body body) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (uint64_t j0 = 0; w + j0 * nw < a.n_bricks; j0 += 32) {
        const uint64_t mine = w + (j0 + lane) * nw;
        unsigned ball = __ballot_sync(0xffffffffu, mine < a.n_bricks && pred(a.flag[mine]));
        for (; ball; ball &= ball - 1) body(w + (j0 + (unsigned)(__ffs(ball) - 1)) * nw);
    }
}

// One warp per brick flagged 1 (dropped-slice words of earlier blocks, not
// folded here, so the fold has not counted them): its occupied voxels.
__global__ void k_ghost_count(ExtractArgs a, uint32_t *__restrict__ count) {
    const int lane = threadIdx.x & 31;
    const uint32_t E3 = 1u << (3 * a.log_e);
    for_flagged_bricks(a, [](uint8_t f) { return f == 1; }, [&](uint64_t c) {
        uint32_t n = 0;
        for (uint32_t m = lane; m < E3; m += 32) {
            uint64_t bi = cand_cell(a, (uint32_t)c, m);
            if (bi != ~0ull && a.data[bi]) ++n;
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
        if (lane == 0) count[c] = n;
    });
}

// One warp per flagged brick: (key, word) of its occupied voxels in Morton
// order at *base + off[c] (at most cap), and the emitted cells cleared (the
// walk reads them with getVoxelDestructive).
__global__ void k_cand_emit(ExtractArgs a, const uint32_t *__restrict__ bits, const uint32_t *__restrict__ count,
                            const uint64_t *__restrict__ off, const uint64_t *__restrict__ base_p, uint64_t cap,
                            uint64_t *__restrict__ keys, uint32_t *__restrict__ payload, uint32_t *__restrict__ err) {
    const int lane = threadIdx.x & 31;
    const uint32_t E3 = 1u << (3 * a.log_e);
    const uint32_t lt = (1u << lane) - 1u;
    for_flagged_bricks(a, [](uint8_t f) { return f != 0; }, [&](uint64_t c) {
        uint64_t base = *base_p + off[c];
        // a brick the fold counted comes with the positions of its voxels:
        // only those cells are read
        const bool folded = a.flag[c] == 2;
        for (uint32_t m0 = 0; m0 < E3; m0 += 32) {
            const uint32_t m = m0 + lane;
            uint32_t on = 1u;
            if (folded) {
                const uint32_t word = bits[c * 16 + (m0 >> 5)];
                if (word == 0) continue;
                on = (word >> lane) & 1u;
            }
            uint64_t bi = m < E3 && on ? cand_cell(a, (uint32_t)c, m) : ~0ull;
            uint32_t v = bi != ~0ull ? a.data[bi] : 0u;
            uint32_t ball = __ballot_sync(0xffffffffu, v != 0);
            if (v) {
                uint64_t o = base + __popc(ball & lt);
                if (o < cap) {
                    keys[o] = a.key_base + ((uint64_t)c << (3 * a.log_e)) + m;
                    payload[o] = v;
                    a.data[bi] = 0;
                } else {
                    atomicOr(err, 8u);
                }
            }
            base += __popc(ball);
        }
        // the counted voxels are exactly those emitted, or the key array has a
        // gap the level build must not read: report it instead
        if (lane == 0 && base != *base_p + off[c] + count[c]) atomicOr(err, 16u);
    });
}

// One warp per brick j of the direct fold: its voxels' (key, word) pairs
// at off[j], keys in Morton order from the brick's cell bits, words from its
// slot (at most cap).
__global__ void k_direct_emit(uint64_t nb, int log_e, const uint32_t *__restrict__ bkey,
                              const uint32_t *__restrict__ bits, const uint32_t *__restrict__ slot,
                              const uint64_t *__restrict__ off, uint64_t cap, uint64_t *__restrict__ keys,
                              uint32_t *__restrict__ payload, uint32_t *__restrict__ err) {
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t E3 = 1u << (3 * log_e);
    const int chunks = (int)((E3 + 31) >> 5);
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t j = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < nb; j += nw) {
        const uint32_t mine = lane < chunks ? bits[j * 16 + (uint64_t)lane] : 0u;
        const uint64_t key0 = (uint64_t)bkey[j] << (3 * log_e), base = off[j];
        const uint32_t *src = slot + j * E3;
        uint32_t rank = 0;
        for (int c = 0; c < chunks; ++c) {
            const uint32_t b = __shfl_sync(0xffffffffu, mine, c);
            if ((b >> lane) & 1u) {
                const uint32_t r = rank + (uint32_t)__popc(b & lt);
                if (base + r < cap) {
                    keys[base + r] = key0 + (uint64_t)(c * 32 + lane);
                    payload[base + r] = src[r];
                } else {
                    atomicOr(err, 8u);
                }
            }
            rank += (uint32_t)__popc(b);
        }
    }
}

__global__ void k_add_u64(uint64_t *__restrict__ acc, const uint64_t *__restrict__ add) { *acc += *add; }

// findBestBlockPartition (PlyLoader.cpp:381-405).
void best_partition(int &w, int &h, int &d, int threads) {
    auto maximum = [&]() -> int & { if (w > h && w > d) return w; else if (h > d) return h; else return d; };
    auto median = [&]() -> int & {
        int mx = std::max(w, std::max(h, d)), mn = std::min(w, std::min(h, d));
        if (w != mn && w != mx) return w; else if (h != mn && h != mx) return h; else return d;
    };
    auto minimum = [&]() -> int & { if (w < h && w < d) return w; else if (h < d) return h; else return d; };
    int used = 1;
    while (used < threads) {
        if ((maximum() % 2) == 0) maximum() /= 2;
        else if ((median() % 2) == 0) median() /= 2;
        else if ((minimum() % 2) == 0) minimum() /= 2;
        else break;
        used *= 2;
    }
}

template <typename TI, typename TO>
int scan_total(const TI *in, TO *out, uint64_t n, TO *total_host, cudaStream_t st) {
    Dev<TO> scratch, tot;
    SVO_ALLOC(scratch, scan_scratch_elems(n));
    SVO_ALLOC(tot, 1);
    SVO_CUDA_TRY((exclusive_scan<TI, TO>(in, out, n, tot.p, scratch.p, st)));
    SVO_CUDA_TRY(cudaMemcpyAsync(total_host, tot.p, sizeof(TO), cudaMemcpyDeviceToHost, st));
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    return SVO_OK;
}

int log2_floor(uint64_t v) {
    int r = -1;
    while (v) {
        v >>= 1;
        ++r;
    }
    return r;
}

uint64_t round_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

struct BlockJob {
    uint32_t morton, first, last;
};

}  // namespace

// Mesh dimensions for a side length: PlyLoader::suggestedDimensions
// (PlyLoader.cpp:499-504).
static void mesh_dims(const svo_mesh *m, int side, int dims[3]) {
    const float s = (float)(side - 2);
    for (int k = 0; k < 3; ++k) dims[k] = (int)((m->upper[k] - m->lower[k]) * s) + 2;
}

int mesh_upload(const MeshHost &h, svo_mesh **out) {
    *out = nullptr;
    const uint64_t nv = h.pos.size() / 3, nt = h.tris.size() / 3;
    if (nv == 0) return set_error(SVO_ERR_FORMAT, "mesh has no vertices");
    std::unique_ptr<svo_mesh> m(new svo_mesh());
    SVO_CUDA_TRY(cudaGetDevice(&m->device));
    // PlyLoader::rescaleVertices (PlyLoader.cpp:167-181)
    float diff[3] = {h.upper[0] - h.lower[0], h.upper[1] - h.lower[1], h.upper[2] - h.lower[2]};
    int largest = 2;
    if (diff[0] > diff[1] && diff[0] > diff[2]) largest = 0;
    else if (diff[1] > diff[2]) largest = 1;
    const float factor = 1.0f / diff[largest];
    for (int k = 0; k < 3; ++k) {
        m->upper[k] = h.upper[k] * factor;
        m->lower[k] = h.lower[k] * factor;
    }
    m->has_normals = h.nrm.empty() ? 0 : 1;
    m->n_tris = nt;
    if (nt == 0) {
        *out = m.release();
        return SVO_OK;
    }
    cudaStream_t st = nullptr;
    SVO_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{st};
    Dev<float> pos, nrm, col;
    Dev<int32_t> idx;
    SVO_ALLOC(pos, nv * 3);
    SVO_ALLOC(col, nv * 3);
    SVO_ALLOC(idx, nt * 3);
    if (m->has_normals) SVO_ALLOC(nrm, nv * 3);
    SVO_CUDA_TRY(cudaMemcpyAsync(pos.p, h.pos.data(), nv * 3 * sizeof(float), cudaMemcpyHostToDevice, st));
    SVO_CUDA_TRY(cudaMemcpyAsync(col.p, h.col.data(), nv * 3 * sizeof(float), cudaMemcpyHostToDevice, st));
    SVO_CUDA_TRY(cudaMemcpyAsync(idx.p, h.tris.data(), nt * 3 * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    if (m->has_normals)
        SVO_CUDA_TRY(cudaMemcpyAsync(nrm.p, h.nrm.data(), nv * 3 * sizeof(float), cudaMemcpyHostToDevice, st));
    SVO_CUDA_TRY(cudaMalloc((void **)&m->d_tris, nt * kTriFloats * sizeof(float)));
    k_mesh_setup<<<grid_for(nt), 256, 0, st>>>(nt, idx.p, pos.p, m->has_normals ? nrm.p : nullptr, col.p, h.lower[0],
                                               h.lower[1], h.lower[2], factor, m->d_tris);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(m->d_tris);
        m->d_tris = nullptr;
        return cuda_fail(e, "mesh setup");
    }
    *out = m.release();
    return SVO_OK;
}

// The mesh build.  With d_volume == nullptr: VoxelData(PlyLoader*, side,
// mem) + VoxelOctree, words out.  With d_volume: PlyLoader::convertToVolume
// (PlyLoader.cpp:506-534, the builder's --mode 1), the w*h*d voxel words (x
// fastest) out in d_volume.  Its blocks are z-slabs of S = mem / (w*h)
// slices, partitioned from (w, h, S) and folded one after another with the
// reference's never-cleared buffer (it reuses `data` and the counts), the
// words folded in place in each slab's output region; no extraction, no
// octree.
int build_mesh_device(const svo_mesh *m, int side, int threads, uint64_t mem, cudaStream_t st, uint32_t **d_words,
                      uint64_t *n_words, float center[3], uint32_t *d_volume) {
    if (side < 5 || side > (1 << 20)) return set_error(SVO_ERR_INVALID, "side %d outside [5, 2^20]", side);
    if (threads < 1) return set_error(SVO_ERR_INVALID, "threads must be >= 1");
    const bool volume = d_volume != nullptr;
    int dims[3];
    mesh_dims(m, side, dims);
    const uint64_t V = round_pow2((uint64_t)std::max(dims[0], std::max(dims[1], dims[2])));
    const int D = log2_floor(V);
    int lb;
    int slab = 0, n_slabs = 0;  // volume mode: slices per slab, slabs
    if (volume) {
        // convertToVolume's slab height: the budget over one byte per cell of a w x h slice
        const uint64_t slice_cost = (uint64_t)dims[0] * (uint64_t)dims[1];
        const uint64_t slice = std::min<uint64_t>(mem / slice_cost, (uint64_t)dims[2]);
        if (slice == 0)
            return set_error(SVO_ERR_MEMORY, "memory budget %llu holds no %dx%d slice", (unsigned long long)mem,
                             dims[0], dims[1]);
        slab = (int)slice;
        n_slabs = (dims[2] + slab - 1) / slab;
        lb = D;  // bricks are keyed over the whole power-of-two volume
    } else {
        // VoxelData::init (VoxelData.cpp:211-262) with the loader's cell cost 4 + 1
        lb = cache_block_log2(dims[0], dims[1], dims[2], mem, 5);
        if (lb < 1)
            return set_error(SVO_ERR_MEMORY, "memory budget %llu too small for a %dx%dx%d volume",
                             (unsigned long long)mem, dims[0], dims[1], dims[2]);
    }
    const int B = 1 << lb;
    // VoxelData::getCenter (VoxelData.cpp:297-303)
    for (int k = 0; k < 3; ++k) center[k] = (float)dims[k] * 0.5f / (float)V;

    // PlyLoader::setupBlockProcessing (PlyLoader.cpp:407-437)
    ListGeom g;
    // block edges: the cubic cache block, or convertToVolume's w x h x S slab
    // (setupBlockProcessing(maxSize, w, h, S, w, h, d))
    const int blk[3] = {volume ? dims[0] : B, volume ? dims[1] : B, volume ? slab : B};
    int sub[3] = {blk[0], blk[1], blk[2]};
    best_partition(sub[0], sub[1], sub[2], threads);
    for (int k = 0; k < 3; ++k) {
        g.sub[k] = sub[k];
        g.part[k] = blk[k] / sub[k];
        g.grid[k] = g.part[k] * (dims[k] + blk[k] - 1) / blk[k];  // the reference's order: multiply, then divide
        g.dims[k] = dims[k];
        g.cell_h[k] = (float)sub[k] / (float)(side - 4);
    }
    g.grid_scale = (float)(side - 4);
    g.log_e = std::min(3, lb);  // 8^3 bricks (the block edge when smaller); pairs carry their sub-block
    g.log_block = lb;
    g.slab_mode = volume ? 1 : 0;
    g.brick_bits = 3 * (D - g.log_e);
    const int lbv = D - lb;  // log2 of blocks per axis
    g.n_blocks = volume ? (uint64_t)n_slabs : 1ull << (3 * lbv);
    if (g.n_blocks > (1ull << 27))
        return set_error(SVO_ERR_LIMIT, "memory budget gives %llu cache blocks; the GPU build supports at most 2^27",
                         (unsigned long long)g.n_blocks);
    const int key_bits = g.brick_bits + (volume ? log2_floor(round_pow2((uint64_t)n_slabs)) : 0);
    if (key_bits > 32)
        return set_error(SVO_ERR_LIMIT, "side %d with %d^3 bricks%s needs more than 32-bit brick keys", side,
                         1 << g.log_e, volume && n_slabs > 1 ? " and this many slabs" : "");
    const int K = std::max(sub[0], std::max(sub[1], sub[2]));
    const int n_l = std::max(dims[0], std::max(dims[1], dims[2])) + 1;
    if ((uint64_t)n_l * (uint64_t)K > (1ull << 28))
        return set_error(SVO_ERR_LIMIT, "voxel-centre table of %d x %d entries is too large", n_l, K);

    const uint64_t nt = m->n_tris;
    Dev<uint32_t> err;
    SVO_ALLOC(err, 1);
    SVO_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(uint32_t), st));
    Dev<uint8_t> bflag;
    SVO_ALLOC(bflag, g.n_blocks);
    SVO_CUDA_TRY(cudaMemsetAsync(bflag.p, 0, g.n_blocks, st));

    // 2. pairs: count, offsets, emit (triangle-major order)
    Dev<int32_t> box;
    Dev<uint32_t> pcount;
    Dev<uint64_t> poff;
    SVO_ALLOC(box, nt * 6);
    SVO_ALLOC(pcount, nt);
    SVO_ALLOC(poff, nt);
    uint64_t n_pairs = 0;
    if (nt) {
        k_tri_pairs<0><<<grid_for(nt, 128), 128, 0, st>>>(nt, m->d_tris, g, box.p, bflag.p, pcount.p, nullptr,
                                                          nullptr, nullptr, nullptr, err.p);
        SVO_LAUNCH_OK("k_tri_pairs<count>");
        int rc = scan_total<uint32_t, uint64_t>(pcount.p, poff.p, nt, &n_pairs, st);
        if (rc) return rc;
    }
    if (n_pairs >= 0xFFFFFFFFull)
        return set_error(SVO_ERR_LIMIT, "%llu brick/triangle pairs exceed 2^32-1", (unsigned long long)n_pairs);
    Dev<uint32_t> pk, pt, pc, pi, pk2, pi2, stri_buf, scell_buf, sort_scratch;
    SVO_ALLOC(pk, n_pairs);
    SVO_ALLOC(pt, n_pairs);
    SVO_ALLOC(pc, n_pairs);
    SVO_ALLOC(pi, n_pairs);
    SVO_ALLOC(pk2, n_pairs);
    SVO_ALLOC(pi2, n_pairs);
    if (n_pairs) {
        k_tri_pairs<1><<<grid_for(nt, 128), 128, 0, st>>>(nt, m->d_tris, g, box.p, bflag.p, pcount.p, poff.p, pk.p,
                                                          pt.p, pc.p, err.p);
        SVO_LAUNCH_OK("k_tri_pairs<emit>");
        k_iota<<<grid_for(n_pairs), 256, 0, st>>>(pi.p, n_pairs);
        SVO_LAUNCH_OK("k_iota");
    }
    pcount.release();
    poff.release();

    // 3. stable sort by brick, then the pairs' triangles and cells in that order
    SVO_ALLOC(sort_scratch, radix_scratch_elems(n_pairs));
    bool in_alt = false;
    SVO_CUDA_TRY(radix_sort_pairs(pk.p, pi.p, pk2.p, pi2.p, n_pairs, key_bits, sort_scratch.p, st, &in_alt));
    sort_scratch.release();
    const uint32_t *skey = in_alt ? pk2.p : pk.p;
    const uint32_t *sidx = in_alt ? pi2.p : pi.p;
    SVO_ALLOC(stri_buf, n_pairs);
    SVO_ALLOC(scell_buf, n_pairs);
    if (n_pairs) {
        k_gather_pairs<<<grid_for(n_pairs), 256, 0, st>>>(sidx, n_pairs, pt.p, pc.p, stri_buf.p, scell_buf.p);
        SVO_LAUNCH_OK("k_gather_pairs");
    }
    const uint32_t *stri = stri_buf.p;
    const uint32_t *scell = scell_buf.p;

    // unique bricks and per-block brick ranges
    Dev<uint32_t> head, hidx, bkey, bstart, rfirst, rlast;
    SVO_ALLOC(head, n_pairs);
    SVO_ALLOC(hidx, n_pairs);
    uint32_t nb = 0;
    if (n_pairs) {
        k_heads_u32<<<grid_for(n_pairs), 256, 0, st>>>(skey, n_pairs, head.p);
        SVO_LAUNCH_OK("k_heads_u32");
        int rc = scan_total<uint32_t, uint32_t>(head.p, hidx.p, n_pairs, &nb, st);
        if (rc) return rc;
    }
    SVO_ALLOC(bkey, nb);
    SVO_ALLOC(bstart, (uint64_t)nb + 1);
    SVO_ALLOC(rfirst, g.n_blocks);
    SVO_ALLOC(rlast, g.n_blocks);
    SVO_CUDA_TRY(cudaMemsetAsync(rfirst.p, 0, g.n_blocks * sizeof(uint32_t), st));
    SVO_CUDA_TRY(cudaMemsetAsync(rlast.p, 0, g.n_blocks * sizeof(uint32_t), st));
    {
        uint32_t np32 = (uint32_t)n_pairs;
        SVO_CUDA_TRY(cudaMemcpyAsync(bstart.p + nb, &np32, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    }
    if (nb) {
        k_brick_table<<<grid_for(n_pairs), 256, 0, st>>>(skey, n_pairs, head.p, hidx.p, bkey.p, bstart.p);
        k_block_ranges<<<grid_for(nb), 256, 0, st>>>(bkey.p, nb, 3 * (lb - g.log_e), g.n_blocks, rfirst.p, rlast.p,
                                                    err.p);
        SVO_LAUNCH_OK("k_block_ranges");
    }
    head.release();
    hidx.release();

    // cache blocks the lists mark, in Morton (visiting) order
    std::vector<BlockJob> jobs;
    {
        Dev<uint32_t> f32, fidx, packed;
        SVO_ALLOC(f32, g.n_blocks);
        SVO_ALLOC(fidx, g.n_blocks);
        k_flag_to_u32<<<grid_for(g.n_blocks), 256, 0, st>>>(bflag.p, g.n_blocks, f32.p);
        SVO_LAUNCH_OK("k_flag_to_u32");
        uint32_t n_jobs = 0;
        int rc = scan_total<uint32_t, uint32_t>(f32.p, fidx.p, g.n_blocks, &n_jobs, st);
        if (rc) return rc;
        SVO_ALLOC(packed, (uint64_t)n_jobs * 3);
        if (n_jobs) {
            k_gather_blocks<<<grid_for(g.n_blocks), 256, 0, st>>>(bflag.p, g.n_blocks, fidx.p, rfirst.p, rlast.p,
                                                                 packed.p);
            SVO_LAUNCH_OK("k_gather_blocks");
        }
        jobs.resize(n_jobs);
        if (n_jobs)
            SVO_CUDA_TRY(cudaMemcpyAsync(jobs.data(), packed.p, (size_t)n_jobs * 3 * sizeof(uint32_t),
                                         cudaMemcpyDeviceToHost, st));
        uint32_t e_h = 0;
        SVO_CUDA_TRY(cudaMemcpyAsync(&e_h, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        SVO_CUDA_TRY(cudaStreamSynchronize(st));
        if (e_h) return set_error(SVO_ERR_DEVICE, "mesh build: sub-block lists out of range (flags %u)", e_h);
    }
    rfirst.release();
    rlast.release();

    // The direct fold.  The extraction leaves the block buffer zero except
    // for each block's dropped last slice (VoxelData.cpp:163-170).  When no
    // such slice lies inside the volume of a block visited after it, every
    // brick is folded from zeros and the blocks need no shared buffer: one
    // fold over all bricks writes each brick's voxels to a slot of its own,
    // and one scan places them.  Bricks are sorted by key and blocks are
    // visited in Morton order, so the bricks of consecutive blocks follow
    // one another and the result is in Morton order.
    bool direct = !volume && nb > 0;
    if (direct) {
        uint32_t next = 0;
        std::vector<std::pair<uint64_t, uint64_t>> gs;  // flat ranges of the dropped slices so far
        for (const BlockJob &j : jobs) {
            if (j.last > j.first) {
                if (j.first != next) direct = false;
                next = j.last;
            }
            int o[3] = {(int)(compact3(j.morton) << lb), (int)(compact3((uint64_t)j.morton >> 1) << lb),
                        (int)(compact3((uint64_t)j.morton >> 2) << lb)};
            int bb[3];
            bool inside = true;
            for (int k = 0; k < 3; ++k) {
                bb[k] = std::min(B, dims[k] - o[k]);
                if (bb[k] <= 0) inside = false;
            }
            if (!inside) continue;
            const uint64_t vol = (uint64_t)bb[0] * bb[1] * bb[2];
            for (const auto &r : gs)
                if (std::min(r.second, vol) > r.first) direct = false;
            if ((bb[2] & 1) && lb >= 2) {
                const uint64_t plane = (uint64_t)bb[0] * bb[1];
                gs.emplace_back(plane * (uint64_t)(bb[2] - 1), plane * (uint64_t)bb[2]);
            }
        }
        if (next != nb) direct = false;
        // the direct fold's scratch (a slot of E^3 words per brick, besides
        // the keys and words both paths hold) must fit comfortably
        size_t free_b = 0, total_b = 0;
        if (direct && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
            (uint64_t)nb * (1ull << (3 * g.log_e)) * 16ull > (uint64_t)free_b / 2)
            direct = false;
        // SVO_MESH_BLOCK_BUFFER=1 keeps the per-block buffer path (same words)
        const char *env = std::getenv("SVO_MESH_BLOCK_BUFFER");
        if (env && *env && *env != '0') direct = false;
    }

    // the persistent block buffer (VoxelData::_bufferedData, zeroed) and the
    // loader's per-cell counts, sized for the largest block volume (a whole
    // w x h x S slab in the conversion)
    uint64_t buf_cells = volume ? (uint64_t)dims[0] * (uint64_t)dims[1] * (uint64_t)slab : 1;
    for (const BlockJob &j : jobs) {
        if (volume) break;
        int o[3] = {(int)(compact3(j.morton) << lb), (int)(compact3((uint64_t)j.morton >> 1) << lb),
                    (int)(compact3((uint64_t)j.morton >> 2) << lb)};
        uint64_t v = 1;
        for (int k = 0; k < 3; ++k) v *= (uint64_t)std::max(0, std::min(B, dims[k] - o[k]));
        buf_cells = std::max(buf_cells, v);
    }
    Dev<uint32_t> data;
    Dev<uint8_t> counts;
    Dev<float> acc;
    // the conversion folds every slab in place in its output (region 0 zeroed here)
    if (!volume && !direct) SVO_ALLOC(data, buf_cells);
    uint32_t *const data_p = volume ? d_volume : data.p;
    if (!direct) {
        SVO_ALLOC(counts, buf_cells);
        SVO_CUDA_TRY(cudaMemsetAsync(data_p, 0, buf_cells * sizeof(uint32_t), st));
        SVO_CUDA_TRY(cudaMemsetAsync(counts.p, 0, buf_cells, st));
    }
    SVO_ALLOC(acc, (uint64_t)n_l * K);
    const float hx = 1.0f / (float)(side - 4);
    k_center_table<<<grid_for(n_l), 256, 0, st>>>(n_l, K, hx, acc.p);
    SVO_LAUNCH_OK("k_center_table");

    int dev = 0, sms = 0;
    SVO_CUDA_TRY(cudaGetDevice(&dev));
    SVO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned fold_grid = (unsigned)sms * 8, warp_grid = (unsigned)sms * 16;
    Dev<uint32_t> fold_next;  // one work counter per fold launch
    const size_t n_next = std::max<size_t>(jobs.size(), 1);
    SVO_ALLOC(fold_next, n_next);
    SVO_CUDA_TRY(cudaMemsetAsync(fold_next.p, 0, n_next * sizeof(uint32_t), st));
    const uint32_t brick_mask = g.slab_mode ? (uint32_t)((1ull << g.brick_bits) - 1) : 0xFFFFFFFFu;
    // what every fold launch shares
    auto fold_args = [&]() -> FoldArgs {
        FoldArgs fa{};
        for (int k = 0; k < 3; ++k) {
            fa.sub[k] = sub[k];
            fa.grid[k] = g.grid[k];
            fa.dims[k] = dims[k];
        }
        fa.tris = m->d_tris;
        fa.box = box.p;
        fa.pair_tri = stri;
        fa.pair_cell = scell;
        fa.bkey = bkey.p;
        fa.bstart = bstart.p;
        fa.log_e = g.log_e;
        fa.log_block = lb;
        fa.acc = acc.p;
        fa.K = K;
        fa.half = 0.5f * hx;
        fa.brick_mask = brick_mask;
        fa.drop_z = -1;
        return fa;
    };

    if (direct) {
        // PlyLoader::processBlock (PlyLoader.cpp:439-458) of every block at
        // once, then the walk's voxels (VoxelOctree.cpp:66-103) from the slots
        const uint32_t E3 = 1u << (3 * g.log_e);
        const uint64_t cap = (uint64_t)nb * E3;
        Dev<uint32_t> slot, ccount, cbits, pay;
        Dev<uint64_t> coff, dN, sc64, keys;
        SVO_ALLOC(slot, cap);
        SVO_ALLOC(ccount, nb);
        SVO_ALLOC(cbits, (uint64_t)nb * 16);
        SVO_ALLOC(coff, nb);
        SVO_ALLOC(dN, 1);
        SVO_ALLOC(sc64, scan_scratch_elems(nb));
        SVO_ALLOC(keys, cap);
        SVO_ALLOC(pay, cap);
        FoldArgs fa = fold_args();
        fa.b_first = 0;
        fa.b_last = nb;
        fa.next = fold_next.p;
        fa.slot = slot.p;
        fa.brick_count = ccount.p;
        fa.brick_bits = cbits.p;
        const unsigned grid = (unsigned)std::min<uint64_t>((nb + kFoldWarps - 1) / kFoldWarps, fold_grid);
        k_fold_bricks<true><<<grid, kFoldWarps * 32, 0, st>>>(fa);
        SVO_LAUNCH_OK("k_fold_bricks<direct>");
        SVO_CUDA_TRY((exclusive_scan<uint32_t, uint64_t>(ccount.p, coff.p, nb, dN.p, sc64.p, st)));
        k_direct_emit<<<warp_grid, 256, 0, st>>>(nb, g.log_e, bkey.p, cbits.p, slot.p, coff.p, cap, keys.p, pay.p,
                                                err.p);
        SVO_LAUNCH_OK("k_direct_emit");
        uint64_t N = 0;
        uint32_t e_h = 0;
        SVO_CUDA_TRY(cudaMemcpyAsync(&N, dN.p, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
        SVO_CUDA_TRY(cudaMemcpyAsync(&e_h, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        SVO_CUDA_TRY(cudaStreamSynchronize(st));
        if (e_h) return set_error(SVO_ERR_DEVICE, "mesh build: voxel extraction check failed (flags %u)", e_h);
        slot.release();
        acc.release();
        if (N >= 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "%llu voxels exceed 2^32-1", (unsigned long long)N);
        return build_from_sorted_device(keys.p, pay.p, N, D, lb, lb < D ? bflag.p : nullptr, st, d_words, n_words);
    }

    // PlyLoader::processBlock (PlyLoader.cpp:439-458) of job ji, whose buffer
    // `data` starts at org with edges buf: its bricks' pairs folded into it
    auto fold_block = [&](size_t ji, const int org[3], const int buf[3], uint32_t *data, const uint8_t *pre_dirty,
                          uint64_t n_pre, uint8_t *brick_flag, uint32_t *brick_count, uint32_t *brick_bits,
                          int drop_z) -> int {
        const BlockJob &j = jobs[ji];
        if (j.last <= j.first) return SVO_OK;
        FoldArgs fa = fold_args();
        for (int k = 0; k < 3; ++k) {
            fa.org[k] = org[k];
            fa.buf[k] = buf[k];
        }
        fa.b_first = j.first;
        fa.b_last = j.last;
        fa.data = data;
        fa.counts = counts.p;
        fa.next = fold_next.p + ji;
        fa.pre_dirty = pre_dirty;
        fa.n_pre = n_pre;
        fa.brick_flag = brick_flag;
        fa.brick_count = brick_count;
        fa.brick_bits = brick_bits;
        fa.drop_z = drop_z;
        unsigned grid = (unsigned)std::min<uint64_t>((j.last - j.first + kFoldWarps - 1) / kFoldWarps, fold_grid);
        k_fold_bricks<false><<<grid, kFoldWarps * 32, 0, st>>>(fa);
        SVO_LAUNCH_OK("k_fold_bricks");
        return SVO_OK;
    };

    if (volume) {
        // convertToVolume (PlyLoader.cpp:506-534): every slab in order through
        // a buffer (words and counts) the reference never clears, so slab s
        // starts from what slab s - 1 left and a slab with no triangles
        // repeats it.  Here slab s is folded in place in its own output
        // region, which first receives a copy of region s - 1 (the buffer
        // after slab s - 1).  The last slab's region holds only its d - z
        // slices; no triangle reaches a cell at z >= d (their voxel boxes end
        // at d - 1), so the shorter buffer changes no output cell.
        const uint64_t plane = (uint64_t)dims[0] * (uint64_t)dims[1];
        size_t ji = 0;
        for (int s = 0; s < n_slabs; ++s) {
            const int nz = std::min(slab, dims[2] - s * slab);
            uint32_t *region = d_volume + plane * (uint64_t)(s * slab);
            if (s > 0)
                SVO_CUDA_TRY(cudaMemcpyAsync(region, region - plane * (uint64_t)slab, plane * (uint64_t)nz * sizeof(uint32_t),
                                             cudaMemcpyDeviceToDevice, st));
            const int org[3] = {0, 0, s * slab}, buf[3] = {dims[0], dims[1], nz};
            if (ji < jobs.size() && jobs[ji].morton == (uint32_t)s) {
                int rc = fold_block(ji, org, buf, region, nullptr, 0, nullptr, nullptr, nullptr, -1);
                if (rc) return rc;
                ++ji;
            }
        }
        uint32_t e_v = 0;
        SVO_CUDA_TRY(cudaMemcpyAsync(&e_v, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        SVO_CUDA_TRY(cudaStreamSynchronize(st));
        if (e_v) return set_error(SVO_ERR_DEVICE, "mesh conversion check failed (flags %u)", e_v);
        if (ji != jobs.size()) return set_error(SVO_ERR_DEVICE, "mesh conversion: slab jobs out of order");
        return SVO_OK;
    }

    // 4. blocks in order: fold, then extract (and clear) the block's voxels.
    // Counts stay on the device, so the loop queues its work without waiting.
    const uint64_t n_e = 1ull << (3 * (lb - g.log_e));  // bricks per block
    Dev<uint8_t> flag;    // per brick of the block: 0 nothing, 1 earlier dropped-slice words, 2 folded here
    Dev<uint32_t> ccount;  // per brick: the voxels the extraction emits
    Dev<uint32_t> cbits;   // per folded brick: which cells those are (16 words)
    Dev<uint64_t> coff, bn, dN, sc64;
    SVO_ALLOC(flag, n_e);
    SVO_ALLOC(ccount, n_e);
    SVO_ALLOC(cbits, n_e * 16);
    SVO_ALLOC(coff, n_e);
    SVO_ALLOC(bn, 1);
    SVO_ALLOC(dN, 1);
    SVO_ALLOC(sc64, scan_scratch_elems(n_e));
    SVO_CUDA_TRY(cudaMemsetAsync(dN.p, 0, sizeof(uint64_t), st));
    // Every emitted voxel lies in a brick folded by its block or is a word an
    // earlier block's dropped slice left behind (each emitted once).
    uint64_t cap = (uint64_t)nb << (3 * g.log_e);
    for (const BlockJob &j : jobs) {
        int oz = (int)(compact3((uint64_t)j.morton >> 2) << lb);
        int bd = std::min(B, dims[2] - oz);
        if (bd > 0 && (bd & 1) && lb >= 2) cap += (uint64_t)B * B;
    }
    Dev<uint64_t> keys;
    Dev<uint32_t> pay;
    SVO_ALLOC(keys, cap);
    SVO_ALLOC(pay, cap);
    std::vector<std::pair<uint64_t, uint64_t>> ghosts;  // flat ranges of the dropped slices so far
    uint64_t ghost_len = 0;
    for (const BlockJob &j : jobs) {
        FoldArgs fa;
        fa.org[0] = (int)(compact3(j.morton) << lb);
        fa.org[1] = (int)(compact3((uint64_t)j.morton >> 1) << lb);
        fa.org[2] = (int)(compact3((uint64_t)j.morton >> 2) << lb);
        bool inside = true;
        for (int k = 0; k < 3; ++k) {
            fa.buf[k] = std::min(B, dims[k] - fa.org[k]);
            if (fa.buf[k] <= 0) inside = false;
        }
        if (!inside) continue;  // VoxelData::prepareDataAccess returns early
        // Bricks under an earlier block's dropped slice may hold nonzero words
        // before this fold (flag 1); every other buffer cell is zero (the
        // extraction cleared it).  When those slices are large, every brick
        // is flagged.  The fold flags the bricks it folds 2 and counts their
        // voxels.
        const uint64_t vol = (uint64_t)fa.buf[0] * fa.buf[1] * fa.buf[2];
        const bool all_dirty = ghost_len * 4 > vol;
        if (all_dirty) {
            SVO_CUDA_TRY(cudaMemsetAsync(flag.p, 1, n_e, st));
        } else {
            SVO_CUDA_TRY(cudaMemsetAsync(flag.p, 0, n_e, st));
            for (const auto &r : ghosts) {
                uint64_t s1 = std::min(r.second, vol);
                if (r.first >= s1) continue;
                k_mark_range<<<grid_for(s1 - r.first), 256, 0, st>>>(r.first, s1, fa.buf[0], fa.buf[1], fa.buf[2],
                                                                    g.log_e, flag.p, n_e);
                SVO_LAUNCH_OK("k_mark_range");
            }
        }
        SVO_CUDA_TRY(cudaMemsetAsync(ccount.p, 0, n_e * sizeof(uint32_t), st));
        const int drop = ((fa.buf[2] & 1) && lb >= 2) ? 1 : 0;
        const int drop_z = drop ? fa.org[2] + fa.buf[2] - 1 : -1;
        int rc = fold_block((size_t)(&j - jobs.data()), fa.org, fa.buf, data_p, all_dirty ? nullptr : flag.p, n_e,
                            flag.p, ccount.p, cbits.p, drop_z);
        if (rc) return rc;
        ExtractArgs ea;
        ea.flag = flag.p;
        ea.n_bricks = n_e;
        ea.log_e = g.log_e;
        for (int k = 0; k < 3; ++k) ea.buf[k] = fa.buf[k];
        ea.drop = drop;
        ea.key_base = (uint64_t)j.morton << (3 * lb);
        ea.data = data.p;
        if (all_dirty || !ghosts.empty()) {
            k_ghost_count<<<warp_grid, 256, 0, st>>>(ea, ccount.p);
            SVO_LAUNCH_OK("k_ghost_count");
        }
        SVO_CUDA_TRY((exclusive_scan<uint32_t, uint64_t>(ccount.p, coff.p, n_e, bn.p, sc64.p, st)));
        k_cand_emit<<<warp_grid, 256, 0, st>>>(ea, cbits.p, ccount.p, coff.p, dN.p, cap, keys.p, pay.p, err.p);
        SVO_LAUNCH_OK("k_cand_emit");
        k_add_u64<<<1, 1, 0, st>>>(dN.p, bn.p);
        if (drop) {  // the walk never reads this slice; it stays in the buffer
            uint64_t plane = (uint64_t)fa.buf[0] * fa.buf[1];
            ghosts.emplace_back(plane * (uint64_t)(fa.buf[2] - 1), plane * (uint64_t)fa.buf[2]);
            ghost_len += plane;
        }
    }
    uint64_t N = 0;
    uint32_t e_h = 0;
    SVO_CUDA_TRY(cudaMemcpyAsync(&N, dN.p, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    SVO_CUDA_TRY(cudaMemcpyAsync(&e_h, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    if (e_h) return set_error(SVO_ERR_DEVICE, "mesh build: voxel extraction check failed (flags %u)", e_h);
    data.release();
    counts.release();
    acc.release();
    if (N >= 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "%llu voxels exceed 2^32-1", (unsigned long long)N);

    // 5. octree from the (already Morton-ordered) voxels
    return build_from_sorted_device(keys.p, pay.p, N, D, lb, lb < D ? bflag.p : nullptr, st, d_words, n_words);
}

}  // namespace svo

// ---- C ABI ---------------------------------------------------------------------

using namespace svo;

extern "C" int svo_mesh_load_ply(const char *path, svo_mesh **out) {
    clear_error();
    if (!path || !out) return set_error(SVO_ERR_INVALID, "null argument");
    *out = nullptr;
    MeshHost h;
    int rc = ply_read(path, h);
    if (rc) return rc;
    return mesh_upload(h, out);
}

extern "C" int svo_mesh_from_arrays(const float *positions, const float *normals, const float *colors,
                                    uint64_t n_vertices, const int32_t *faces, uint64_t n_face_ints, svo_mesh **out) {
    clear_error();
    if (!positions || !out || (!faces && n_face_ints)) return set_error(SVO_ERR_INVALID, "null argument");
    *out = nullptr;
    MeshHost h;
    h.pos.reserve(n_vertices * 3);
    h.col.reserve(n_vertices * 3);
    const float white[3] = {255.0f, 255.0f, 255.0f};
    for (uint64_t v = 0; v < n_vertices; ++v) {
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(positions[3 * v + k]))
                return set_error(SVO_ERR_FORMAT, "vertex %llu has a non-finite coordinate", (unsigned long long)v);
        mesh_add_vertex(h, positions + 3 * v, normals ? normals + 3 * v : nullptr, colors ? colors + 3 * v : white);
    }
    for (uint64_t o = 0; o < n_face_ints;) {
        int32_t c = faces[o];
        if (c < 0 || o + 1 + (uint64_t)c > n_face_ints) return set_error(SVO_ERR_FORMAT, "face list truncated");
        int rc = mesh_add_face(h, faces + o + 1, c, n_vertices);
        if (rc) return rc;
        o += 1 + (uint64_t)c;
    }
    return mesh_upload(h, out);
}

extern "C" int svo_ply_parse(const char *path, float **positions, float **normals, float **colors,
                             uint64_t *n_vertices, int32_t **triangles, uint64_t *n_triangles, float lower[3],
                             float upper[3]) {
    clear_error();
    if (!path || !positions || !normals || !colors || !n_vertices || !triangles || !n_triangles || !lower || !upper)
        return set_error(SVO_ERR_INVALID, "null argument");
    *positions = *normals = *colors = nullptr;
    *triangles = nullptr;
    MeshHost h;
    int rc = ply_read(path, h);
    if (rc) return rc;
    auto dup = [](const void *src, size_t bytes) -> void * {
        void *d = std::malloc(bytes ? bytes : 1);
        if (d && bytes) std::memcpy(d, src, bytes);
        return d;
    };
    *positions = (float *)dup(h.pos.data(), h.pos.size() * sizeof(float));
    *colors = (float *)dup(h.col.data(), h.col.size() * sizeof(float));
    *normals = h.nrm.empty() ? nullptr : (float *)dup(h.nrm.data(), h.nrm.size() * sizeof(float));
    *triangles = (int32_t *)dup(h.tris.data(), h.tris.size() * sizeof(int32_t));
    if (!*positions || !*colors || !*triangles || (!h.nrm.empty() && !*normals)) {
        std::free(*positions);
        std::free(*colors);
        std::free(*normals);
        std::free(*triangles);
        *positions = *normals = *colors = nullptr;
        *triangles = nullptr;
        return set_error(SVO_ERR_MEMORY, "host allocation for the parsed mesh");
    }
    *n_vertices = h.pos.size() / 3;
    *n_triangles = h.tris.size() / 3;
    for (int k = 0; k < 3; ++k) {
        lower[k] = h.lower[k];
        upper[k] = h.upper[k];
    }
    return SVO_OK;
}

extern "C" uint64_t svo_mesh_num_triangles(const svo_mesh *m) { return m ? m->n_tris : 0; }

extern "C" int svo_mesh_dimensions(const svo_mesh *m, int side, int dims[3]) {
    clear_error();
    if (!m || !dims) return set_error(SVO_ERR_INVALID, "null argument");
    mesh_dims(m, side, dims);
    return SVO_OK;
}

extern "C" void svo_mesh_destroy(svo_mesh *m) {
    if (!m) return;
    if (m->d_tris) cudaFree(m->d_tris);
    delete m;
}

extern "C" int svo_octree_build_mesh(const svo_mesh *m, int side, int threads, uint64_t mem, svo_stream stream,
                                     svo_octree **out) {
    clear_error();
    if (!m || !out) return set_error(SVO_ERR_INVALID, "null argument");
    *out = nullptr;
    int cur = 0;
    SVO_CUDA_TRY(cudaGetDevice(&cur));
    if (cur != m->device) return set_error(SVO_ERR_INVALID, "mesh lives on device %d, current device is %d", m->device, cur);
    uint32_t *dw = nullptr;
    uint64_t nw = 0;
    float center[3];
    int rc = build_mesh_device(m, side, threads, mem, (cudaStream_t)stream, &dw, &nw, center, nullptr);
    if (rc) return rc;
    return make_handle(dw, nw, center, out);
}

extern "C" int svo_mesh_to_volume(const svo_mesh *m, int side, int threads, uint64_t mem, uint32_t *d_volume,
                                  svo_stream stream) {
    clear_error();
    if (!m || !d_volume) return set_error(SVO_ERR_INVALID, "null argument");
    int cur = 0;
    SVO_CUDA_TRY(cudaGetDevice(&cur));
    if (cur != m->device) return set_error(SVO_ERR_INVALID, "mesh lives on device %d, current device is %d", m->device, cur);
    uint32_t *dw = nullptr;
    uint64_t nw = 0;
    float center[3];
    return build_mesh_device(m, side, threads, mem, (cudaStream_t)stream, &dw, &nw, center, d_volume);
}

extern "C" int svo_mesh_write_voxel_file(const svo_mesh *m, const char *path, int side, int threads, uint64_t mem,
                                         svo_stream stream) {
    clear_error();
    if (!m || !path) return set_error(SVO_ERR_INVALID, "null argument");
    int dims[3];
    int rc = svo_mesh_dimensions(m, side, dims);
    if (rc) return rc;
    const uint64_t cells = (uint64_t)dims[0] * dims[1] * dims[2];
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t *dv = nullptr;
    SVO_CUDA_TRY(cudaMalloc((void **)&dv, cells * sizeof(uint32_t)));
    std::unique_ptr<uint32_t, cudaError_t (*)(void *)> dguard(dv, cudaFree);
    rc = svo_mesh_to_volume(m, side, threads, mem, dv, stream);
    if (rc) return rc;
    FILE *fp = fopen(path, "wb");
    if (!fp) return set_error(SVO_ERR_IO, "cannot open %s", path);
    std::unique_ptr<FILE, int (*)(FILE *)> fguard(fp, fclose);
    // the .voxel layout VoxelData reads (VoxelData.cpp:37-48): int32 w, h, d, then the words, x fastest
    if (fwrite(dims, 4, 3, fp) != 3) return set_error(SVO_ERR_IO, "%s: write failed", path);
    const uint64_t chunk = 16ull << 20;  // words per staged copy (64 MB)
    uint32_t *pin = nullptr;
    SVO_CUDA_TRY(cudaMallocHost((void **)&pin, std::min(chunk, cells) * sizeof(uint32_t)));
    std::unique_ptr<uint32_t, cudaError_t (*)(void *)> pguard(pin, cudaFreeHost);
    for (uint64_t c0 = 0; c0 < cells; c0 += chunk) {
        const uint64_t n = std::min(chunk, cells - c0);
        SVO_CUDA_TRY(cudaMemcpyAsync(pin, dv + c0, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        SVO_CUDA_TRY(cudaStreamSynchronize(st));
        if (fwrite(pin, sizeof(uint32_t), n, fp) != n) return set_error(SVO_ERR_IO, "%s: write failed", path);
    }
    return SVO_OK;
}

extern "C" int svo_octree_build_ply(const char *path, int side, int threads, uint64_t mem, svo_stream stream,
                                    svo_octree **out) {
    svo_mesh *m = nullptr;
    int rc = svo_mesh_load_ply(path, &m);
    if (rc) return rc;
    rc = svo_octree_build_mesh(m, side, threads, mem, stream, out);
    svo_mesh_destroy(m);
    return rc;
}
