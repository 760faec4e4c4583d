// render.cu — the viewer's frame on the GPU: renderBatch + renderTile
// (Main.cpp:92-202) with the beam prepass, headless.
//
// The frame is cut into n_strips horizontal strips as Main.cpp:349-361 cuts
// it over its threads; each strip has its own corner grid (a corner every 8
// pixels, one tile row and column past the strip) and its own running
// dx/dy sums, so pixel values depend on that layout, which is a parameter.
//   1. k_corners: one thread per corner; the level-of-detail raymarch from
//      the camera with coarseScale = 16 / (planeDist * H) gives t or a miss
//      depth of 1e10 (Main.cpp:166-185).
//   2. k_tiles: one warp per 8x4 half of an 8x8 tile.  A tile whose four
//      corner depths are all misses stays 0 (the strip's memset, :160);
//      otherwise each pixel rebuilds its direction from the same running
//      sums as renderTile (dx = -1 + x0*scale, then += scale per pixel),
//      normalises it with invSqrt, traces from pos + dir*max(minT - 0.03, 0)
//      (:187-198) and packs shade() as RGBA8 with the reference's
//      double-precision scale (:116-128).  With pixel_stride > 1 (the
//      viewer's half-size mode) a pixel takes the colour of its stride
//      corner, which is computed the same way.
#include <algorithm>
#include <cmath>

#include "svo_device.cuh"
#include "svo_internal.h"

namespace svo {
namespace {

constexpr int kTile = 8;
constexpr float kTreeMiss = 1e10f;

struct FrameArgs {
    const uint32_t *oct;
    const uint4 *tab;  // descriptor table (kernels instantiated with kTab)
    uint32_t n_words;
    float a[9];
    float pos[3];
    float light[3];
    float zx, zy, zz, scale, tile_scale, aspect, coarse;
    int W, H, strip_rows, n_strips, tiles_x, tiles_y_max, pixel_stride;
    float *dx_corner;   // tiles_x running sums (x0 = 0 for every strip)
    float *dy_corner;   // n_strips x tiles_y_max running sums
    int *tile_start;    // n_strips + 1 prefix of (tiles_y - 1) * (tiles_x - 1)
    float *depth;       // n_strips x tiles_y_max x tiles_x
    uint32_t *out;
    uint32_t *status;
};

__device__ __forceinline__ void view_dir(const FrameArgs &f, float dx, float dy, float &x, float &y, float &z) {
    x = dx * f.a[0] + dy * f.a[1] + f.zx;
    y = dx * f.a[3] + dy * f.a[4] + f.zy;
    z = dx * f.a[6] + dy * f.a[7] + f.zz;
    float s = inv_sqrt(x * x + y * y + z * z);
    x *= s;
    y *= s;
    z *= s;
}

__device__ __forceinline__ int strip_rows_of(const FrameArgs &f, int s, int &y0) {
    y0 = s * f.strip_rows;
    int y1 = min((s + 1) * f.strip_rows, f.H);
    return y1 - y0;
}

// The corner loop's running sums (Main.cpp:166-168): dx from -1 + x0*scale
// (x0 = 0), dy per strip from AspectRatio - y0*scale, stepping by tileScale;
// and the strips' tile prefix.  One warp.
__global__ void k_frame_setup(FrameArgs f) {
    const int lane = threadIdx.x;
    if (lane == 0) {
        float dx = -1.0f + 0.0f * f.scale;
        for (int x = 0; x < f.tiles_x; ++x, dx += f.tile_scale) f.dx_corner[x] = dx;
        int acc = 0;
        f.tile_start[0] = 0;
        for (int s = 0; s < f.n_strips; ++s) {
            int y0;
            int rows = strip_rows_of(f, s, y0);
            int tiles_y = (rows - 1) / kTile + 2;
            acc += max(0, tiles_y - 1) * (f.tiles_x - 1);
            f.tile_start[s + 1] = acc;
        }
    }
    for (int s = lane; s < f.n_strips; s += 32) {
        float dy = f.aspect - (float)(s * f.strip_rows) * f.scale;
        for (int y = 0; y < f.tiles_y_max; ++y, dy -= f.tile_scale) f.dy_corner[s * f.tiles_y_max + y] = dy;
    }
}

template <bool kTab>
__global__ void k_corners(FrameArgs f) {
    const int tx = blockIdx.x * blockDim.x + threadIdx.x;
    const int ty = blockIdx.y, s = blockIdx.z;
    if (tx >= f.tiles_x) return;
    int y0;
    const int rows = strip_rows_of(f, s, y0);
    const int tiles_y = (rows - 1) / kTile + 2;  // Main.cpp:360 (C division)
    if (ty >= tiles_y) return;
    float x, y, z;
    view_dir(f, f.dx_corner[tx], f.dy_corner[s * f.tiles_y_max + ty], x, y, z);
    RayResult r = trace_ray<kTab>(f.oct, f.tab, f.n_words, f.pos[0], f.pos[1], f.pos[2], x, y, z, f.coarse);
    if (r.status == kFault) atomicOr(f.status, 1u);
    f.depth[((size_t)s * f.tiles_y_max + ty) * f.tiles_x + tx] = (r.status == kLeafHit || r.status == kLodHit) ? r.t : kTreeMiss;
}

template <bool kTab>
__global__ void k_tiles(FrameArgs f, int total_tiles) {
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int tile = w >> 1, half = w & 1;
    if (tile >= total_tiles) return;
    int s = 0;
    while (s + 1 < f.n_strips && f.tile_start[s + 1] <= tile) ++s;
    const int k = tile - f.tile_start[s];
    const int c = k % (f.tiles_x - 1), r = k / (f.tiles_x - 1);
    int y0;
    const int rows = strip_rows_of(f, s, y0);
    const int y1 = y0 + rows;
    const int tx0 = c * kTile, ty0 = r * kTile + y0;
    const int px = tx0 + (lane & 7), py = ty0 + half * 4 + (lane >> 3);
    if (px >= f.W || py >= y1) return;
    const float *d = f.depth + (size_t)s * f.tiles_y_max * f.tiles_x;
    const int idx = (r + 1) * f.tiles_x + (c + 1);
    const float minT = smin(smin(d[idx], d[idx - 1]), smin(d[idx - f.tiles_x], d[idx - f.tiles_x - 1]));
    uint32_t color = 0;
    if (minT != kTreeMiss) {
        const int cx = px - ((px - tx0) % f.pixel_stride), cy = py - ((py - ty0) % f.pixel_stride);
        float dx = -1.0f + (float)tx0 * f.scale;
        for (int i = tx0; i < cx; ++i) dx += f.scale;
        float dy = f.aspect - (float)ty0 * f.scale;
        for (int i = ty0; i < cy; ++i) dy -= f.scale;
        float x, y, z;
        view_dir(f, dx, dy, x, y, z);
        const float t0 = smax(minT - 0.03f, 0.0f);
        RayResult res = trace_ray<kTab>(f.oct, f.tab, f.n_words, f.pos[0] + x * t0, f.pos[1] + y * t0,
                                        f.pos[2] + z * t0, x, y, z, 0.0f);
        if (res.status == kFault) atomicOr(f.status, 1u);
        float col = 0.0f;
        if (res.status == kLeafHit) col = shade_grey(res.word, x, y, z, f.light[0], f.light[1], f.light[2]);
        uint32_t c8 = (uint32_t)((double)smin(col, 1.0f) * 255.0);
        color = c8 | (c8 << 8) | (c8 << 16) | 0xFF000000u;
    }
    f.out[(size_t)py * f.W + px] = color;
}

}  // namespace
}  // namespace svo

using namespace svo;

extern "C" int svo_render_frame(const svo_octree *oct, const float rot[9], const float pos[3], uint32_t width,
                                uint32_t height, uint32_t n_strips, uint32_t pixel_stride, uint32_t *rgba,
                                svo_stream stream) {
    clear_error();
    if (!oct || !rot || !pos || !rgba) return set_error(SVO_ERR_INVALID, "null argument");
    if (width < 1 || height < 1 || width > 32768 || height > 32768)
        return set_error(SVO_ERR_INVALID, "frame size %ux%u outside [1, 32768]", width, height);
    if (n_strips < 1 || n_strips > height) return set_error(SVO_ERR_INVALID, "n_strips must lie in [1, height]");
    if (pixel_stride < 1 || pixel_stride > kTile) return set_error(SVO_ERR_INVALID, "pixel_stride must lie in [1, 8]");
    if (wide_octree(oct)) return set_error(SVO_ERR_LIMIT, "frame rendering takes octrees of up to 2^32-1 words");
    cudaStream_t st = (cudaStream_t)stream;
    FrameArgs f;
    f.oct = oct->d_words;
    f.tab = octree_table(oct, (cudaStream_t)stream);
    f.n_words = (uint32_t)oct->n_words;
    for (int i = 0; i < 9; ++i) f.a[i] = rot[i];
    for (int i = 0; i < 3; ++i) f.pos[i] = pos[i];
    const int W = (int)width, H = (int)height, S = (int)n_strips;
    // Main.cpp:150-158, 62
    const float plane_dist = 1.0f / std::tan(3.14159265358979323846f / 6.0f);
    f.scale = 2.0f / (float)W;
    const float tile_scale = (float)kTile * f.scale;
    f.aspect = (float)H / (float)W;
    f.zx = plane_dist * rot[2];
    f.zy = plane_dist * rot[5];
    f.zz = plane_dist * rot[8];
    f.coarse = 2.0f * (float)kTile / (plane_dist * (float)H);
    float l[3] = {rot[0] * -1.0f + rot[1] * 1.0f + rot[2] * -1.0f + 0.0f,
                  rot[3] * -1.0f + rot[4] * 1.0f + rot[5] * -1.0f + 0.0f,
                  rot[6] * -1.0f + rot[7] * 1.0f + rot[8] * -1.0f + 0.0f};
    const float inv = 1.0f / std::sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
    for (int i = 0; i < 3; ++i) f.light[i] = l[i] * inv;
    f.W = W;
    f.H = H;
    f.n_strips = S;
    f.strip_rows = (H - 1) / S + 1;  // Main.cpp:349
    f.tiles_x = (W - 1) / kTile + 2;
    f.tiles_y_max = (f.strip_rows - 1) / kTile + 2;
    f.pixel_stride = (int)pixel_stride;
    f.tile_scale = tile_scale;
    int total_tiles = 0;  // the same prefix as k_frame_setup's, for the launch size
    for (int s = 0; s < S; ++s) {
        int y0 = s * f.strip_rows, y1 = std::min((s + 1) * f.strip_rows, H);
        total_tiles += std::max(0, (y1 - y0 - 1) / kTile + 1) * (f.tiles_x - 1);
    }
    void *scratch = nullptr;
    const size_t n_f = (size_t)f.tiles_x + (size_t)S * f.tiles_y_max, n_depth = (size_t)S * f.tiles_y_max * f.tiles_x;
    const size_t bytes = (n_f + n_depth) * sizeof(float) + (S + 1) * sizeof(int);
    SVO_CUDA_TRY(scratch_alloc(&scratch, bytes, st));
    float *sf = (float *)scratch;
    f.dx_corner = sf;
    f.dy_corner = sf + f.tiles_x;
    f.depth = sf + n_f;
    f.tile_start = (int *)(sf + n_f + n_depth);
    f.out = rgba;
    f.status = oct->d_status;
    k_frame_setup<<<1, 32, 0, st>>>(f);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        dim3 g1((unsigned)((f.tiles_x + 127) / 128), (unsigned)f.tiles_y_max, (unsigned)S);
        if (f.tab)
            k_corners<true><<<g1, 128, 0, st>>>(f);
        else
            k_corners<false><<<g1, 128, 0, st>>>(f);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && total_tiles > 0) {
        uint64_t threads = (uint64_t)total_tiles * 64;
        if (f.tab)
            k_tiles<true><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(f, total_tiles);
        else
            k_tiles<false><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(f, total_tiles);
        e = cudaGetLastError();
    }
    cudaFreeAsync(scratch, st);
    if (e != cudaSuccess) return cuda_fail(e, "svo_render_frame");
    return SVO_OK;
}
