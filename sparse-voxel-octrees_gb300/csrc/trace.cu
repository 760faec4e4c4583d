// trace.cu — ray traversal kernels over the resident octree.
//
// k_trace_plain: one thread per ray, the drop-in for a loop of
// VoxelOctree::raymarch (VoxelOctree.cpp:207-346) plus the viewer's shade()
// (Main.cpp:81-90).  Rays are 24-byte records (o, d) read as three float2;
// outputs are structure-of-arrays so every store is coalesced.  It is
// instantiated for 32-bit word indices (octrees of up to 2^32-1 words) and
// 64-bit ones (larger octrees, whose far offsets exceed 32 bits);
// k_trace_plain_tab walks the handle's descriptor table instead, where it
// has one.
#include <algorithm>

#include "svo_device.cuh"
#include "svo_internal.h"

namespace svo {
namespace {

struct TraceArgs {
    const uint32_t *oct;
    const uint4 *tab;  // descriptor table (the table kernel only)
    uint64_t n_words;
    const float *rays;
    uint64_t n;
    float ray_scale;
    float lx, ly, lz;
    uint8_t *hit;
    float *t;
    uint32_t *leaf;
    uint32_t *word;
    float *rgb;
    uint32_t *rgba8;
    uint32_t *status;
};

__device__ __forceinline__ void load_ray(const float *rays, uint64_t i, float &ox, float &oy, float &oz, float &dx,
                                         float &dy, float &dz) {
    const float2 *r = reinterpret_cast<const float2 *>(rays) + 3 * i;
    float2 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
    ox = a.x; oy = a.y; oz = b.x;
    dx = b.y; dy = c.x; dz = c.y;
}

template <typename Idx>
__device__ __forceinline__ void store_result(const TraceArgs &a, uint64_t i, const RayResultT<Idx> &r, float dx,
                                             float dy, float dz) {
    if (r.status == kFault) atomicOr(a.status, 1u);
    uint8_t hs = r.status == kFault ? 0 : (uint8_t)r.status;
    if (a.hit) a.hit[i] = hs;
    if (a.t) a.t[i] = (hs == 0) ? __int_as_float(0x7f800000) : r.t;
    bool leaf = r.status == kLeafHit;
    if (a.leaf) a.leaf[i] = leaf ? (uint32_t)r.leaf : 0xFFFFFFFFu;  // the host admits it only below 2^32
    if (a.word) a.word[i] = leaf ? r.word : 0u;
    if (a.rgb || a.rgba8) {
        float g = leaf ? shade_grey(r.word, dx, dy, dz, a.lx, a.ly, a.lz) : 0.0f;
        if (a.rgb) {
            a.rgb[3 * i + 0] = g;
            a.rgb[3 * i + 1] = g;
            a.rgb[3 * i + 2] = g;
        }
        if (a.rgba8) a.rgba8[i] = pack_rgba8(g);
    }
}

template <typename Idx>
__global__ void __launch_bounds__(256) k_trace_plain(TraceArgs a) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    float ox, oy, oz, dx, dy, dz;
    load_ray(a.rays, i, ox, oy, oz, dx, dy, dz);
    RayResultT<Idx> r = raymarch<false, Idx>(a.oct, (Idx)a.n_words, ox, oy, oz, dx, dy, dz, a.ray_scale, nullptr);
    store_result<Idx>(a, i, r, dx, dy, dz);
}

// The same over the handle's descriptor table.
__global__ void __launch_bounds__(256) k_trace_plain_tab(TraceArgs a) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    float ox, oy, oz, dx, dy, dz;
    load_ray(a.rays, i, ox, oy, oz, dx, dy, dz);
    RayResult r = trace_ray<true>(a.oct, a.tab, 0u, ox, oy, oz, dx, dy, dz, a.ray_scale);
    store_result<uint32_t>(a, i, r, dx, dy, dz);
}

// The table kernel as a persistent grid: each warp takes the next
// kQueueChunk rays from a per-launch counter (32 at a time), so a warp that
// finishes early starts new rays instead of leaving its slot idle until the
// slowest warp of its CTA is done.
constexpr int kQueueChunk = 32;

__global__ void __launch_bounds__(256) k_trace_queue_tab(TraceArgs a, unsigned long long *queue) {
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0, end = 0;
    while (true) {
        if (base >= end) {
            if (lane == 0) base = atomicAdd(queue, (unsigned long long)kQueueChunk);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= a.n) break;
            end = min(base + (unsigned long long)kQueueChunk, (unsigned long long)a.n);
        }
        const uint64_t i = base + lane;
        base += 32;
        if (i >= end) continue;
        float ox, oy, oz, dx, dy, dz;
        load_ray(a.rays, i, ox, oy, oz, dx, dy, dz);
        RayResult r = trace_ray<true>(a.oct, a.tab, 0u, ox, oy, oz, dx, dy, dz, a.ray_scale);
        store_result<uint32_t>(a, i, r, dx, dy, dz);
    }
}

// svo_trace's table kernel: the persistent queue form, or one thread per ray.
constexpr bool kPlainQueue = true;

__global__ void __launch_bounds__(256) k_count_loads(const uint32_t *oct, uint32_t n_words, const float *rays,
                                                    uint64_t n, float ray_scale, uint32_t *loads,
                                                    uint32_t *status) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float ox, oy, oz, dx, dy, dz;
    load_ray(rays, i, ox, oy, oz, dx, dy, dz);
    uint32_t nl = 0;
    RayResult r = raymarch<true>(oct, n_words, ox, oy, oz, dx, dy, dz, ray_scale, &nl);
    if (r.status == kFault) atomicOr(status, 1u);
    loads[i] = nl;
}

}  // namespace

int launch_trace(const svo_octree *oct, const float *d_rays, uint64_t n, float ray_scale, const float light[3],
                 const svo_trace_out &out, cudaStream_t st) {
    if (n == 0) return SVO_OK;
    if (out.leaf && wide_octree(oct))
        return set_error(SVO_ERR_LIMIT, "leaf indices of an octree of %llu words do not fit the 32-bit leaf output",
                         (unsigned long long)oct->n_words);
    TraceArgs a;
    a.oct = oct->d_words;
    a.n_words = oct->n_words;
    a.rays = d_rays;
    a.n = n;
    a.ray_scale = ray_scale;
    a.lx = light ? light[0] : 0.0f;
    a.ly = light ? light[1] : 0.0f;
    a.lz = light ? light[2] : 0.0f;
    a.hit = out.hit;
    a.t = out.t;
    a.leaf = out.leaf;
    a.word = out.word;
    a.rgb = out.rgb;
    a.rgba8 = out.rgba8;
    a.status = oct->d_status;
    a.tab = nullptr;
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (wide_octree(oct) || oct->index_bits == 64)
        k_trace_plain<uint64_t><<<grid, 256, 0, st>>>(a);
    else if ((a.tab = octree_table(oct, st)) != nullptr) {
        if (kPlainQueue) {
            int dev = 0, sms = 0, resident = 0;
            SVO_CUDA_TRY(cudaGetDevice(&dev));
            SVO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_trace_queue_tab, 256, 0));
            void *q = nullptr;
            SVO_CUDA_TRY(scratch_alloc(&q, sizeof(unsigned long long), st));
            cudaError_t e = cudaMemsetAsync(q, 0, sizeof(unsigned long long), st);
            const uint64_t warps = (n + 31) / 32;
            const uint64_t ctas = std::min<uint64_t>((uint64_t)sms * std::max(1, resident), (warps + 7) / 8);
            if (e == cudaSuccess) {
                k_trace_queue_tab<<<(unsigned)ctas, 256, 0, st>>>(a, (unsigned long long *)q);
                e = cudaGetLastError();
            }
            cudaFreeAsync(q, st);
            if (e != cudaSuccess) return cuda_fail(e, "svo_trace");
            return SVO_OK;
        }
        k_trace_plain_tab<<<grid, 256, 0, st>>>(a);
    } else
        k_trace_plain<uint32_t><<<grid, 256, 0, st>>>(a);
    SVO_CUDA_TRY(cudaGetLastError());
    return SVO_OK;
}

int launch_count_loads(const svo_octree *oct, const float *d_rays, uint64_t n, float ray_scale, uint32_t *loads,
                       cudaStream_t st) {
    if (n == 0) return SVO_OK;
    if (wide_octree(oct)) return set_error(SVO_ERR_LIMIT, "load counting takes octrees of up to 2^32-1 words");
    k_count_loads<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(oct->d_words, (uint32_t)oct->n_words, d_rays, n,
                                                               ray_scale, loads, oct->d_status);
    SVO_CUDA_TRY(cudaGetLastError());
    return SVO_OK;
}

}  // namespace svo
