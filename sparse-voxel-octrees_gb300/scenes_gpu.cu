// scenes_gpu.cu — GPU generators for the synthetic benchmark inputs
// (libsvo_scenes.so).  Harness code, not part of the octree path: it
// produces the same voxel grids and camera rays as scenes.py, bit for bit
// (float32 in the same operation order, built with -fmad=false), at sizes
// where numpy is too slow (2048^3).
//
// Occupancy is a bitmap of 32-voxel words along x: word (xw, y, z) at
// xw + W32 * (y + side * z), W32 = max(1, side / 32), bit b = voxel 32*xw + b.
#include <cstdint>
#include <cuda_runtime.h>

#include "csrc/svo_device.cuh"

namespace {

__device__ __forceinline__ uint64_t bm_index(int xw, int y, int z, int w32, int side) {
    return (uint64_t)xw + (uint64_t)w32 * ((uint64_t)y + (uint64_t)side * (uint64_t)z);
}

__device__ __forceinline__ int bm_get(const uint32_t *bm, int x, int y, int z, int w32, int side) {
    if (x < 0 || y < 0 || z < 0 || x >= side || y >= side || z >= side) return 0;
    return (bm[bm_index(x >> 5, y, z, w32, side)] >> (x & 31)) & 1;
}

// Terrain shell: h - thickness < y + 0.5 <= h for h = heights[z * side + x].
__global__ void k_terrain(uint32_t *bm, int side, int w32, const float *heights, float thickness) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)side * side) return;
    int x = (int)(i % side), z = (int)(i / side);
    float h = heights[i];
    float lo = h - thickness;
    int y0 = (int)floorf(lo) - 1, y1 = (int)ceilf(h) + 1;
    if (y0 < 0) y0 = 0;
    if (y1 > side - 1) y1 = side - 1;
    for (int y = y0; y <= y1; ++y) {
        float yc = (float)y + 0.5f;
        if (yc <= h && yc > lo) atomicOr(bm + bm_index(x >> 5, y, z, w32, side), 1u << (x & 31));
    }
}

// One sphere per blockIdx.y; threads enumerate (xw, y, z) items of its box.
// box[s] = {x0, x1, y0, y1, z0, z1} (half-open, clipped), params[s] = {cx, cy, cz, r}.
__global__ void k_spheres(uint32_t *bm, int side, int w32, const int *box, const float *params) {
    int s = blockIdx.y;
    const int *b = box + 6 * s;
    int x0 = b[0], x1 = b[1], y0 = b[2], y1 = b[3], z0 = b[4], z1 = b[5];
    if (x0 >= x1 || y0 >= y1 || z0 >= z1) return;
    int xw0 = x0 >> 5, xw1 = (x1 - 1) >> 5;
    int nxw = xw1 - xw0 + 1, ny = y1 - y0;
    uint64_t items = (uint64_t)nxw * ny * (z1 - z0);
    float cx = params[4 * s], cy = params[4 * s + 1], cz = params[4 * s + 2], r = params[4 * s + 3];
    float rr = r * r;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < items; i += (uint64_t)gridDim.x * blockDim.x) {
        int xw = xw0 + (int)(i % nxw);
        int y = y0 + (int)((i / nxw) % ny);
        int z = z0 + (int)(i / ((uint64_t)nxw * ny));
        float dy = ((float)y + 0.5f) - cy;
        float dz = ((float)z + 0.5f) - cz;
        float dyy = dy * dy, dzz = dz * dz;
        uint32_t bits = 0;
        for (int k = 0; k < 32; ++k) {
            int x = xw * 32 + k;
            if (x < x0 || x >= x1) continue;
            float dx = ((float)x + 0.5f) - cx;
            if ((dx * dx + dyy) + dzz <= rr) bits |= 1u << k;
        }
        if (bits) atomicOr(bm + bm_index(xw, y, z, w32, side), bits);
    }
}

__device__ __forceinline__ uint32_t hash32(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t h = (x * 0x8DA6B343u) ^ (y * 0xD8163841u) ^ (z * 0xCB1AB31Fu);
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

// Dense payload grid (x fastest, side^3 words) from the bitmap.
__global__ void k_payload(const uint32_t *bm, int side, int w32, uint32_t *grid) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t nwords = (uint64_t)w32 * side * side;
    if (i >= nwords) return;
    int xw = (int)(i % w32);
    int y = (int)((i / w32) % side);
    int z = (int)(i / ((uint64_t)w32 * side));
    uint32_t occ = bm[i];
    int xbase = xw * 32;
    int nx = side - xbase < 32 ? side - xbase : 32;
    uint32_t *row = grid + (uint64_t)xbase + (uint64_t)side * ((uint64_t)y + (uint64_t)side * z);
    for (int k = 0; k < nx; ++k) {
        uint32_t word = 0;
        if ((occ >> k) & 1) {
            int x = xbase + k;
            float gx = (float)(bm_get(bm, x - 1, y, z, w32, side) - bm_get(bm, x + 1, y, z, w32, side));
            float gy = (float)(bm_get(bm, x, y - 1, z, w32, side) - bm_get(bm, x, y + 1, z, w32, side));
            float gz = (float)(bm_get(bm, x, y, z - 1, w32, side) - bm_get(bm, x, y, z + 1, w32, side));
            if (gx == 0.0f && gy == 0.0f && gz == 0.0f) gy = 1.0f;
            uint32_t h = hash32((uint32_t)x, (uint32_t)y, (uint32_t)z);
            float r = (float)(h & 255u), g = (float)((h >> 8) & 255u), b = (float)((h >> 16) & 255u);
            float shade = (r * 0.2126f + g * 0.7152f + b * 0.0722f) * (1.0f / 256.0f);
            word = svo::compress_material(gx, gy, gz, shade);
            if (word == 0) word = 1;
        }
        row[k] = word;
    }
}

// Camera rays, row-major over [x0, x1) x [y0, y1); c = {a11..a33, px, py, pz,
// scale, aspect, zx, zy, zz}.
__global__ void k_camera(const float *c, int x0, int y0, int nx, int ny, float *rays) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)nx * ny) return;
    int px = x0 + (int)(i % nx), py = y0 + (int)(i / nx);
    float dx = -1.0f + (float)px * c[12];
    float dy = c[13] - (float)py * c[12];
    float vx = (dx * c[0] + dy * c[1]) + c[14];
    float vy = (dx * c[3] + dy * c[4]) + c[15];
    float vz = (dx * c[6] + dy * c[7]) + c[16];
    float n = svo::inv_sqrt((vx * vx + vy * vy) + vz * vz);
    float *r = rays + 6 * i;
    r[0] = c[9];
    r[1] = c[10];
    r[2] = c[11];
    r[3] = vx * n;
    r[4] = vy * n;
    r[5] = vz * n;
}

inline unsigned nblk(uint64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

extern "C" {

int svo_scene_terrain(uint32_t *bm, int side, const float *heights, float thickness, void *stream) {
    int w32 = side >= 32 ? side / 32 : 1;
    k_terrain<<<nblk((uint64_t)side * side), 256, 0, (cudaStream_t)stream>>>(bm, side, w32, heights, thickness);
    return (int)cudaGetLastError();
}

int svo_scene_spheres(uint32_t *bm, int side, int n, const int *box, const float *params, void *stream) {
    if (n <= 0) return 0;
    int w32 = side >= 32 ? side / 32 : 1;
    dim3 grid(512, (unsigned)n);
    k_spheres<<<grid, 256, 0, (cudaStream_t)stream>>>(bm, side, w32, box, params);
    return (int)cudaGetLastError();
}

int svo_scene_payload(const uint32_t *bm, int side, uint32_t *grid, void *stream) {
    int w32 = side >= 32 ? side / 32 : 1;
    k_payload<<<nblk((uint64_t)w32 * side * side), 256, 0, (cudaStream_t)stream>>>(bm, side, w32, grid);
    return (int)cudaGetLastError();
}

int svo_scene_camera_rays(const float *cam17, int x0, int y0, int nx, int ny, float *rays, void *stream) {
    k_camera<<<nblk((uint64_t)nx * ny), 256, 0, (cudaStream_t)stream>>>(cam17, x0, y0, nx, ny, rays);
    return (int)cudaGetLastError();
}

}  // extern "C"
