// batch.cu — persistent, queue-driven traversal over many (octree, view)
// pairs in one launch, its CUDA-graph capture and its autotuner.
//
// Work is a global space of ray slots: each view contributes either one slot
// per ray (linear views) or 32 slots per tile_w x tile_h pixel tile (image
// views, so a warp's lanes start on neighbouring pixels).  A persistent grid
// of SMs x blocks_per_sm CTAs drains the space: each warp takes `chunk`
// consecutive slots from one device counter with a single atomicAdd and hands
// them to its idle lanes in ballot-rank order.  Lanes whose ray finishes go
// idle; once at least `refill_idle` lanes of a warp are idle the warp refills
// them, so lanes keep doing traversal steps instead of waiting for the
// slowest ray of a fixed 32-ray batch.  Nothing waits on another warp or CTA.
//
// Optionally (plain-tile schedule) each warp keeps the first `cache_entries`
// descriptor-table entries (the top levels: the table is stored breadth
// first) of one octree in its own slice of shared memory, reloaded when the
// octree of the warp's next 32 slots changes; lanes tracing another octree
// read the global table.  The cached entries are copies of the global ones,
// so results do not depend on the cache.  The autotuner picks the depth.
//
// Each ray runs the same ray_init / ray_step as svo_trace (VoxelOctree.cpp:
// 207-346), so results are bit-identical to the plain kernel's.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "svo_device.cuh"
#include "svo_internal.h"

namespace svo {
namespace {

constexpr int kMaxSmemJobs = 2048;  // views whose slot offsets are staged in shared memory

struct JobDev {
    const uint32_t *oct;
    const uint4 *tab;  // the octree's descriptor table (kernels instantiated with kTab)
    uint32_t n_tab;
    uint32_t n_words;
    uint32_t width, height, tiles_x;
    const float *rays;
    float cam[17];
    float ray_scale, lx, ly, lz;
    uint8_t *hit;
    float *t;
    uint32_t *leaf;
    uint32_t *word;
    float *rgb;
    uint32_t *rgba8;
};

struct BatchArgs {
    const JobDev *jobs;
    const uint64_t *begin;  // n_jobs + 1 slot offsets
    int n_jobs;
    uint64_t total;
    unsigned long long *queue;
    uint32_t *status;
    int refill_idle;
    int steps_per_round;
    int log_tile_w;
    int chunk;
    int cache_entries;      // per-warp table cache (0 = none)
    uint32_t cache_offset;  // byte offset of the warp caches in dynamic shared memory
};

constexpr int kMaxCacheEntries = 512;
constexpr int kMaxCacheBytes = 64 * 1024;  // per CTA

// Fills a warp's table cache with the first entries of job j's table and
// returns how many it holds.  Called by all 32 lanes with no lane still
// reading the cache.
__device__ __forceinline__ uint32_t load_warp_cache(const JobDev *jobs, int j, uint4 *wc, int cap, int lane) {
    const uint4 *tab = jobs[j].tab;
    const uint32_t n = min((uint32_t)cap, jobs[j].n_tab);
    __syncwarp();
    for (uint32_t i = lane; i < n; i += 32) wc[i] = __ldg(tab + i);
    __syncwarp();
    return n;
}

// The table step, reading the warp's cache for rays of the cached octree.
template <bool kTab, bool kLod, bool kCache>
__device__ __forceinline__ bool batch_step(RayState &s, RayStackFor<kTab> &stk, const uint32_t *__restrict__ words,
                                           const uint4 *__restrict__ tab, uint32_t n_words, float rayScale,
                                           RayResult &res, const uint4 *wc, uint32_t wc_n) {
    if constexpr (kTab && kCache)
        return ray_step_tab<kLod, true>(s, stk, words, tab, rayScale, res, wc, wc_n);
    else
        return ray_step_any<kTab, kLod>(s, stk, words, tab, n_words, rayScale, res);
}

__device__ __forceinline__ int find_job(const uint64_t *beg, int n_jobs, uint64_t slot) {
    int lo = 0, hi = n_jobs;  // beg[lo] <= slot < beg[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (beg[mid] <= slot) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Maps a work slot to its view and ray, initialises the traversal state and
// returns false for the padding slots of partial pixel tiles.
template <bool kTab>
__device__ __forceinline__ bool setup_slot(const BatchArgs &a, const uint64_t *beg, uint64_t slot, RayState &st,
                                           int &job, uint32_t &out_idx, const uint32_t *&oct, const uint4 *&tab,
                                           uint32_t &nw, float &rs, float &rdx, float &rdy, float &rdz) {
    int j = find_job(beg, a.n_jobs, slot);
    const JobDev &J = a.jobs[j];
    uint64_t local = slot - beg[j];
    uint32_t px = 0, py = 0;
    if (J.width) {
        // tile < 2^27 (a view has at most 2^32 pixels): 32-bit division
        const uint32_t tile = (uint32_t)(local >> 5), r = (uint32_t)(local & 31);
        const uint32_t ty = tile / J.tiles_x, tx = tile - ty * J.tiles_x;
        px = tx * (1u << a.log_tile_w) + (r & ((1u << a.log_tile_w) - 1u));
        py = ty * (32u >> a.log_tile_w) + (r >> a.log_tile_w);
        if (px >= J.width || py >= J.height) return false;
        out_idx = py * J.width + px;
    } else {
        out_idx = (uint32_t)local;
    }
    float ox, oy, oz, dx, dy, dz;
    if (J.rays) {
        const float2 *r2 = reinterpret_cast<const float2 *>(J.rays) + 3 * (uint64_t)out_idx;
        float2 p0 = __ldg(r2), p1 = __ldg(r2 + 1), p2 = __ldg(r2 + 2);
        ox = p0.x; oy = p0.y; oz = p1.x;
        dx = p1.y; dy = p2.x; dz = p2.y;
    } else {
        // The viewer's camera ray (Main.cpp:167-176), as scenes.camera_rays.
        const float *c = J.cam;
        float sx = -1.0f + (float)px * c[12];
        float sy = c[13] - (float)py * c[12];
        float vx = (sx * c[0] + sy * c[1]) + c[14];
        float vy = (sx * c[3] + sy * c[4]) + c[15];
        float vz = (sx * c[6] + sy * c[7]) + c[16];
        float n = inv_sqrt((vx * vx + vy * vy) + vz * vz);
        ox = c[9]; oy = c[10]; oz = c[11];
        dx = vx * n; dy = vy * n; dz = vz * n;
    }
    ray_init_any<kTab>(st, J.oct, J.tab, ox, oy, oz, dx, dy, dz);
    rdx = dx; rdy = dy; rdz = dz;
    job = j;
    oct = J.oct;
    tab = J.tab;
    nw = J.n_words;
    rs = J.ray_scale;
    return true;
}

__device__ __forceinline__ void write_result(const BatchArgs &a, int job, uint32_t out_idx, const RayResult &res,
                                             float rdx, float rdy, float rdz) {
    const JobDev &J = a.jobs[job];
    if (res.status == kFault) atomicOr(a.status, 1u);
    uint8_t hs = res.status == kFault ? 0 : (uint8_t)res.status;
    bool leaf = res.status == kLeafHit;
    if (J.hit) J.hit[out_idx] = hs;
    if (J.t) J.t[out_idx] = hs == 0 ? __int_as_float(0x7f800000) : res.t;
    if (J.leaf) J.leaf[out_idx] = leaf ? res.leaf : 0xFFFFFFFFu;
    if (J.word) J.word[out_idx] = leaf ? res.word : 0u;
    if (J.rgb || J.rgba8) {
        float g = leaf ? shade_grey(res.word, rdx, rdy, rdz, J.lx, J.ly, J.lz) : 0.0f;
        if (J.rgb) {
            J.rgb[3 * (uint64_t)out_idx + 0] = g;
            J.rgb[3 * (uint64_t)out_idx + 1] = g;
            J.rgb[3 * (uint64_t)out_idx + 2] = g;
        }
        if (J.rgba8) J.rgba8[out_idx] = pack_rgba8(g);
    }
}

// refill_idle == 0: a warp takes `chunk` slots at once and runs them 32 at a
// time, each lane to completion, before it takes the next chunk.
template <bool kTab, bool kLod, bool kCache>
__device__ __forceinline__ void trace_tiles(const BatchArgs &a, unsigned char *s_dyn) {
    uint64_t *s_begin = reinterpret_cast<uint64_t *>(s_dyn);
    const bool staged = a.n_jobs + 1 <= kMaxSmemJobs;
    if (staged)
        for (int i = threadIdx.x; i <= a.n_jobs; i += blockDim.x) s_begin[i] = a.begin[i];
    __syncthreads();
    const uint64_t *beg = staged ? s_begin : a.begin;
    const int lane = threadIdx.x & 31;
    uint4 *wc = nullptr;
    if (kCache) wc = reinterpret_cast<uint4 *>(s_dyn + a.cache_offset) + (threadIdx.x >> 5) * a.cache_entries;
    int cjob = -1;
    uint32_t cn = 0;
    RayStackFor<kTab> stk;
    while (true) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.queue, (unsigned long long)a.chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= a.total) break;
        unsigned long long end = min(base + (unsigned long long)a.chunk, (unsigned long long)a.total);
        for (unsigned long long s0 = base; s0 < end; s0 += 32) {
            if constexpr (kCache) {
                // The octree of the group's first slot (a group spans two
                // views only at the end of one), loaded before any ray state
                // is live.  s0 is the same in every lane.
                const int want = find_job(beg, a.n_jobs, s0);
                if (want != cjob) {
                    cn = load_warp_cache(a.jobs, want, wc, a.cache_entries, lane);
                    cjob = want;
                }
            }
            uint64_t slot = s0 + lane;
            if (slot >= end) continue;
            RayState st;
            int job;
            uint32_t out_idx, nw;
            const uint32_t *oct;
            const uint4 *tab;
            float rs, rdx, rdy, rdz;
            if (!setup_slot<kTab>(a, beg, slot, st, job, out_idx, oct, tab, nw, rs, rdx, rdy, rdz)) continue;
            const uint32_t my_n = (kCache && job == cjob) ? cn : 0u;
            RayResult res;
            while (!batch_step<kTab, kLod, kCache>(st, stk, oct, tab, nw, rs, res, wc, my_n)) {
            }
            write_result(a, job, out_idx, res, rdx, rdy, rdz);
        }
    }
}

template <bool kTab, bool kLod>
__global__ void k_trace_tiles(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    trace_tiles<kTab, kLod, false>(a, s_dyn);
}

// With the table cache: capped at 48 registers (5 CTAs of 256 threads per
// SM, as the uncached kernel); uncapped it takes 60.
template <bool kLod>
__global__ void __maxnreg__(48) k_trace_tiles_cached(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    trace_tiles<true, kLod, true>(a, s_dyn);
}

template <bool kTab, bool kLod>
__device__ __forceinline__ void trace_refill(const BatchArgs &a, unsigned char *s_dyn) {
    uint64_t *s_begin = reinterpret_cast<uint64_t *>(s_dyn);
    const bool staged = a.n_jobs + 1 <= kMaxSmemJobs;
    if (staged)
        for (int i = threadIdx.x; i <= a.n_jobs; i += blockDim.x) s_begin[i] = a.begin[i];
    __syncthreads();
    const uint64_t *beg = staged ? s_begin : a.begin;

    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    RayState st;
    RayStackFor<kTab> stk;
    bool active = false;
    int job = 0;
    uint32_t out_idx = 0, nw = 0;
    const uint32_t *oct = nullptr;
    const uint4 *tab = nullptr;
    float rdx = 0.f, rdy = 0.f, rdz = 0.f, rs = 0.f;
    uint64_t pool_next = 0, pool_end = 0;
    bool exhausted = false;

    while (true) {
        unsigned idle = ~__ballot_sync(FULL, active);
        if (__popc(idle) >= a.refill_idle) {
            while (idle) {
                if (pool_next >= pool_end) {
                    if (exhausted) break;
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(a.queue, (unsigned long long)a.chunk);
                    base = __shfl_sync(FULL, base, 0);
                    if (base >= a.total) {
                        exhausted = true;
                        break;
                    }
                    pool_next = base;
                    pool_end = min(base + (unsigned long long)a.chunk, (unsigned long long)a.total);
                }
                uint32_t avail = (uint32_t)(pool_end - pool_next);
                uint32_t rank = __popc(idle & lt_mask);
                bool mine = ((idle >> lane) & 1u) && rank < avail;
                if (mine)
                    active = setup_slot<kTab>(a, beg, pool_next + rank, st, job, out_idx, oct, tab, nw, rs, rdx, rdy,
                                              rdz);
                unsigned taken = __ballot_sync(FULL, mine);
                pool_next += __popc(taken);
                idle &= ~taken;
            }
        }
        if (!__any_sync(FULL, active)) {
            if (exhausted && pool_next >= pool_end) break;
            continue;
        }
        if (active) {
            for (int k = 0; k < a.steps_per_round; ++k) {
                RayResult res;
                if (ray_step_any<kTab, kLod>(st, stk, oct, tab, nw, rs, res)) {
                    write_result(a, job, out_idx, res, rdx, rdy, rdz);
                    active = false;
                    break;
                }
            }
        }
    }
}

template <bool kTab, bool kLod>
__global__ void k_trace_persistent(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    trace_refill<kTab, kLod>(a, s_dyn);
}

// The same kernel built with at most 48 registers per thread (reg_cap 48):
// 5 resident CTAs of 256 threads per SM instead of 4, for a few spilled
// registers.
template <bool kTab, bool kLod>
__global__ void __maxnreg__(48) k_trace_persistent_r48(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    trace_refill<kTab, kLod>(a, s_dyn);
}

// Table entries (the top levels) each CTA of the image kernel copies into
// shared memory.
constexpr int kImageStage = 0;

// One image view, passed by value (svo_trace_image): the tile kernel's loop
// without a job table.
template <bool kTab, bool kLod, int kStage>
__global__ void k_trace_single(JobDev J, uint64_t total, unsigned long long *queue, uint32_t *status, int log_tile_w,
                               int chunk) {
    const int lane = threadIdx.x & 31;
    __shared__ uint4 s_tab[kStage > 0 ? kStage : 1];
    if (kTab && kStage > 0) {
        const uint32_t m = min((uint32_t)kStage, J.n_tab);
        for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) s_tab[i] = __ldg(J.tab + i);
        __syncthreads();
    }
    RayStackFor<kTab> stk;
    BatchArgs a;  // only the fields write_result reads
    a.jobs = &J;
    a.status = status;
    while (true) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(queue, (unsigned long long)chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        unsigned long long end = min(base + (unsigned long long)chunk, (unsigned long long)total);
        for (unsigned long long s0 = base; s0 < end; s0 += 32) {
            uint64_t local = s0 + lane;
            if (local >= end) continue;
            const uint32_t tile = (uint32_t)(local >> 5), r = (uint32_t)(local & 31);  // tile < 2^27
            const uint32_t ty = tile / J.tiles_x, tx = tile - ty * J.tiles_x;
            uint32_t px = tx * (1u << log_tile_w) + (r & ((1u << log_tile_w) - 1u));
            uint32_t py = ty * (32u >> log_tile_w) + (r >> log_tile_w);
            if (px >= J.width || py >= J.height) continue;
            uint32_t out_idx = py * J.width + px;
            const float2 *r2 = reinterpret_cast<const float2 *>(J.rays) + 3 * (uint64_t)out_idx;
            float2 p0 = __ldg(r2), p1 = __ldg(r2 + 1), p2 = __ldg(r2 + 2);
            RayState st;
            ray_init_any<kTab>(st, J.oct, J.tab, p0.x, p0.y, p1.x, p1.y, p2.x, p2.y);
            RayResult res;
            if constexpr (kTab && kStage > 0) {
                const uint32_t m = min((uint32_t)kStage, J.n_tab);
                while (!ray_step_tab<kLod, true>(st, stk, J.oct, J.tab, J.ray_scale, res, s_tab, m)) {
                }
            } else {
                while (!ray_step_any<kTab, kLod>(st, stk, J.oct, J.tab, J.n_words, J.ray_scale, res)) {
                }
            }
            write_result(a, 0, out_idx, res, p1.y, p2.x, p2.y);
        }
    }
}

int log2_of(int v) {
    int r = 0;
    while ((1 << r) < v) ++r;
    return r;
}

bool config_ok(const svo_trace_config &c) {
    return c.block_threads >= 32 && c.block_threads <= 1024 && c.block_threads % 32 == 0 && c.blocks_per_sm >= 1 &&
           c.blocks_per_sm <= 32 && c.refill_idle >= 0 && c.refill_idle <= 32 && c.steps_per_round >= 1 &&
           c.steps_per_round <= 4096 && (c.tile_w == 4 || c.tile_w == 8 || c.tile_w == 16 || c.tile_w == 32) &&
           c.chunk >= 32 && c.chunk <= 8192 && c.chunk % 32 == 0 && c.cache_entries >= 0 &&
           c.cache_entries <= kMaxCacheEntries && c.cache_entries % 32 == 0 &&
           (c.cache_entries == 0 || c.refill_idle == 0) && (c.reg_cap == 0 || c.reg_cap == 48) &&
           (c.block_threads / 32) * c.cache_entries * (int)sizeof(uint4) <= kMaxCacheBytes;
}

}  // namespace

// svo_trace_image: rays in row-major image order, traced in tile_w x (32 /
// tile_w) pixel tiles by one persistent launch.
int launch_trace_image(const svo_octree *oct, const float *d_rays, uint32_t width, uint32_t height, float ray_scale,
                       const float light[3], const svo_trace_out &out, cudaStream_t st, int queue) {
    if (width == 0 || height == 0) return SVO_OK;
    if (wide_octree(oct)) return set_error(SVO_ERR_LIMIT, "image tracing takes octrees of up to 2^32-1 words");
    const int tile_w = 8, log_tw = 3, chunk = 32, threads = 256;
    JobDev J;
    std::memset(&J, 0, sizeof(J));
    J.oct = oct->d_words;
    J.n_words = (uint32_t)oct->n_words;
    J.width = width;
    J.height = height;
    J.tiles_x = (width + tile_w - 1) / tile_w;
    J.rays = d_rays;
    J.ray_scale = ray_scale;
    J.lx = light ? light[0] : 0.0f;
    J.ly = light ? light[1] : 0.0f;
    J.lz = light ? light[2] : 0.0f;
    J.hit = out.hit;
    J.t = out.t;
    J.leaf = out.leaf;
    J.word = out.word;
    J.rgb = out.rgb;
    J.rgba8 = out.rgba8;
    uint64_t total = (uint64_t)J.tiles_x * ((height + (32 / tile_w) - 1) / (32 / tile_w)) * 32;
    J.tab = octree_table(oct, st);
    J.n_tab = J.tab ? (uint32_t)oct->n_tab : 0u;
    constexpr int S = kImageStage;
    void (*kern)(JobDev, uint64_t, unsigned long long *, uint32_t *, int, int) =
        J.tab ? (ray_scale != 0.0f ? k_trace_single<true, true, S> : k_trace_single<true, false, S>)
              : (ray_scale != 0.0f ? k_trace_single<false, true, 0> : k_trace_single<false, false, 0>);
    int dev = 0, sms = 0, resident = 0;
    SVO_CUDA_TRY(cudaGetDevice(&dev));
    SVO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, threads, 0));
    unsigned long long *q = oct->d_queue + queue;
    SVO_CUDA_TRY(cudaMemsetAsync(q, 0, sizeof(unsigned long long), st));
    kern<<<(unsigned)(sms * std::max(1, resident)), threads, 0, st>>>(J, total, q, oct->d_status, log_tw, chunk);
    SVO_CUDA_TRY(cudaGetLastError());
    return SVO_OK;
}

}  // namespace svo

struct svo_batch {
    std::vector<svo_view> views;
    std::vector<uint64_t> begin_h;  // slot offsets for the tile width of begin_tile_w
    int begin_tile_w = 0;
    svo::JobDev *jobs_d = nullptr;
    uint64_t *begin_d = nullptr;
    unsigned long long *queue_d = nullptr;
    uint32_t *status_d = nullptr;
    uint64_t total = 0;
    bool any_lod = false;
    bool all_tab = false;  // every view's octree has a descriptor table
    int device = 0, num_sms = 0;
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace svo {
namespace {

// Uploads the job table and slot offsets for tile width `tile_w`.
int prepare_jobs(svo_batch *b, int tile_w) {
    if (b->begin_tile_w == tile_w) return SVO_OK;
    const int n = (int)b->views.size();
    const int th = 32 / tile_w;
    std::vector<JobDev> jobs(n);
    std::vector<uint64_t> beg(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        const svo_view &v = b->views[i];
        JobDev &J = jobs[i];
        std::memset(&J, 0, sizeof(J));
        J.oct = v.octree->d_words;
        J.tab = b->all_tab ? v.octree->d_tab : nullptr;
        J.n_tab = b->all_tab ? (uint32_t)v.octree->n_tab : 0u;
        J.n_words = (uint32_t)v.octree->n_words;
        J.width = v.width;
        J.height = v.height;
        J.tiles_x = v.width ? (v.width + tile_w - 1) / tile_w : 0;
        J.rays = v.rays;
        std::memcpy(J.cam, v.camera, sizeof(J.cam));
        J.ray_scale = v.ray_scale;
        J.lx = v.light[0];
        J.ly = v.light[1];
        J.lz = v.light[2];
        J.hit = v.out.hit;
        J.t = v.out.t;
        J.leaf = v.out.leaf;
        J.word = v.out.word;
        J.rgb = v.out.rgb;
        J.rgba8 = v.out.rgba8;
        uint64_t slots = v.width ? (uint64_t)J.tiles_x * ((v.height + th - 1) / th) * 32 : v.n_rays;
        beg[i + 1] = beg[i] + slots;
    }
    SVO_CUDA_TRY(cudaMemcpy(b->jobs_d, jobs.data(), n * sizeof(JobDev), cudaMemcpyHostToDevice));
    SVO_CUDA_TRY(cudaMemcpy(b->begin_d, beg.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice));
    b->begin_h = beg;
    b->total = beg[n];
    b->begin_tile_w = tile_w;
    return SVO_OK;
}

using BatchKernel = void (*)(BatchArgs);

// The kernel for a launch shape: plain tiles or lane refill (default or
// 48-register build), table or word traversal, level-of-detail exit,
// per-warp table cache (tiles over tables only).
BatchKernel batch_kernel(bool tab, bool lod, bool refill, bool cache, bool r48 = false) {
    if (refill && r48) {
        if (tab) return lod ? k_trace_persistent_r48<true, true> : k_trace_persistent_r48<true, false>;
        return lod ? k_trace_persistent_r48<false, true> : k_trace_persistent_r48<false, false>;
    }
    if (refill) {
        if (tab) return lod ? k_trace_persistent<true, true> : k_trace_persistent<true, false>;
        return lod ? k_trace_persistent<false, true> : k_trace_persistent<false, false>;
    }
    if (tab) {
        if (cache) return lod ? k_trace_tiles_cached<true> : k_trace_tiles_cached<false>;
        return lod ? k_trace_tiles<true, true> : k_trace_tiles<true, false>;
    }
    return lod ? k_trace_tiles<false, true> : k_trace_tiles<false, false>;
}

// Dynamic shared memory above the default 48 KB needs an opt-in per kernel;
// it is set outside any stream capture, when a batch is created.
int allow_large_smem() {
    const int bytes = (int)(((kMaxSmemJobs * sizeof(uint64_t)) + 15) / 16 * 16) + kMaxCacheBytes;
    for (int tab = 0; tab < 2; ++tab)
        for (int lod = 0; lod < 2; ++lod)
            for (int refill = 0; refill < 2; ++refill)
                for (int cache = 0; cache <= (tab && !refill); ++cache)
                    for (int r48 = 0; r48 <= refill; ++r48)
                        SVO_CUDA_TRY(cudaFuncSetAttribute(batch_kernel(tab, lod, refill, cache, r48),
                                                          cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    return SVO_OK;
}

int enqueue_trace(svo_batch *b, const svo_trace_config &c, cudaStream_t st) {
    BatchArgs a;
    a.jobs = b->jobs_d;
    a.begin = b->begin_d;
    a.n_jobs = (int)b->views.size();
    a.total = b->total;
    a.queue = b->queue_d;
    a.status = b->status_d;
    a.refill_idle = c.refill_idle;
    a.steps_per_round = c.steps_per_round;
    a.log_tile_w = log2_of(c.tile_w);
    a.chunk = c.chunk;
    // [slot offsets (when staged)][one table cache per warp]
    size_t smem = (a.n_jobs + 1 <= kMaxSmemJobs) ? (size_t)(a.n_jobs + 1) * sizeof(uint64_t) : 0;
    const bool cache = b->all_tab && c.cache_entries > 0;
    a.cache_entries = cache ? c.cache_entries : 0;
    a.cache_offset = (uint32_t)((smem + 15) / 16 * 16);
    if (cache) smem = a.cache_offset + (size_t)(c.block_threads / 32) * c.cache_entries * sizeof(uint4);
    // A persistent grid larger than what is resident only adds CTAs that
    // start after the queue is drained: clamp to the occupancy limit.
    BatchKernel kern = batch_kernel(b->all_tab, b->any_lod, c.refill_idle != 0, cache, c.reg_cap == 48);
    int resident = 0;
    SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, c.block_threads, smem));
    int per_sm = std::max(1, std::min(c.blocks_per_sm, resident));
    SVO_CUDA_TRY(cudaMemsetAsync(b->queue_d, 0, sizeof(unsigned long long), st));
    dim3 grid((unsigned)(b->num_sms * per_sm));
    kern<<<grid, c.block_threads, smem, st>>>(a);
    SVO_CUDA_TRY(cudaGetLastError());
    return SVO_OK;
}

// ---- autotuner cache: one JSON object per line, keyed by device and workload.
std::string cache_path() {
    const char *p = getenv("SVO_AUTOTUNE_CACHE");
    if (p && *p) return p;
    const char *home = getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/svo_gb300_autotune.jsonl";
}

std::string workload_key(const svo_batch *b) {
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, b->device);
    uint64_t words = 0, rays = 0;
    int images = 0;
    for (const auto &v : b->views) {
        words += v.octree->n_words;
        rays += v.width ? (uint64_t)v.width * v.height : v.n_rays;
        images += v.width != 0;
    }
    char key[512];
    snprintf(key, sizeof(key), "%s|views=%zu|images=%d|rays_log2=%d|words_log2=%d", prop.name, b->views.size(),
             images, log2_of((int)std::min<uint64_t>(rays, 1u << 30)),
             log2_of((int)std::min<uint64_t>(words, 1u << 30)));
    for (char *c = key; *c; ++c)
        if (*c == '"') *c = '\'';
    return key;
}

bool cache_lookup(const std::string &key, svo_trace_config *c) {
    FILE *fp = fopen(cache_path().c_str(), "r");
    if (!fp) return false;
    char line[1024];
    bool found = false;
    while (fgets(line, sizeof(line), fp)) {
        std::string s(line);
        std::string tag = "\"key\": \"" + key + "\"";
        if (s.find(tag) == std::string::npos) continue;
        svo_trace_config t;
        const char *q = strstr(line, "\"block_threads\":");
        t.cache_entries = 0;
        t.reg_cap = 0;
        const char *ce = strstr(line, "\"cache_entries\":");
        const char *rc = strstr(line, "\"reg_cap\":");
        if (q && sscanf(q, "\"block_threads\": %d, \"blocks_per_sm\": %d, \"refill_idle\": %d, \"steps_per_round\": %d, "
                           "\"tile_w\": %d, \"chunk\": %d",
                        &t.block_threads, &t.blocks_per_sm, &t.refill_idle, &t.steps_per_round, &t.tile_w,
                        &t.chunk) == 6 &&
            (!ce || sscanf(ce, "\"cache_entries\": %d", &t.cache_entries) == 1) &&
            (!rc || sscanf(rc, "\"reg_cap\": %d", &t.reg_cap) == 1) && config_ok(t)) {
            *c = t;
            found = true;  // the last matching line wins
        }
    }
    fclose(fp);
    return found;
}

// Creates every missing directory of `dir` (mkdir -p, without a shell).
bool make_dirs(const std::string &dir) {
    for (size_t i = 1; i <= dir.size(); ++i) {
        if (i < dir.size() && dir[i] != '/') continue;
        const std::string part = dir.substr(0, i);
        if (mkdir(part.c_str(), 0755) != 0 && errno != EEXIST) return false;
    }
    return true;
}

void cache_store(const std::string &key, const svo_trace_config &c, float ms) {
    std::string path = cache_path();
    size_t slash = path.rfind('/');
    if (slash != std::string::npos && slash > 0 && !make_dirs(path.substr(0, slash))) return;
    FILE *fp = fopen(path.c_str(), "a");
    if (!fp) return;
    fprintf(fp,
            "{\"key\": \"%s\", \"block_threads\": %d, \"blocks_per_sm\": %d, \"refill_idle\": %d, \"steps_per_round\": "
            "%d, \"tile_w\": %d, \"chunk\": %d, \"cache_entries\": %d, \"reg_cap\": %d, \"ms\": %.4f}\n",
            key.c_str(), c.block_threads, c.blocks_per_sm, c.refill_idle, c.steps_per_round, c.tile_w, c.chunk,
            c.cache_entries, c.reg_cap, ms);
    fclose(fp);
}

}  // namespace
}  // namespace svo

using namespace svo;

extern "C" {

int svo_batch_destroy(svo_batch *b);

int svo_batch_default_config(svo_trace_config *cfg) {
    if (!cfg) return set_error(SVO_ERR_INVALID, "null argument");
    cfg->block_threads = 256;
    cfg->blocks_per_sm = 6;
    cfg->refill_idle = 16;
    cfg->steps_per_round = 8;
    cfg->tile_w = 8;
    cfg->chunk = 64;
    cfg->cache_entries = 0;
    cfg->reg_cap = 0;
    return SVO_OK;
}

int svo_batch_create(const svo_view *views, int n_views, svo_batch **out) {
    if (!views || n_views <= 0 || !out) return set_error(SVO_ERR_INVALID, "bad arguments");
    std::unique_ptr<svo_batch> b(new svo_batch());
    for (int i = 0; i < n_views; ++i) {
        const svo_view &v = views[i];
        if (!v.octree) return set_error(SVO_ERR_INVALID, "view %d has no octree", i);
        if (wide_octree(v.octree))
            return set_error(SVO_ERR_LIMIT, "view %d: batched tracing takes octrees of up to 2^32-1 words", i);
        if (!v.rays && (v.width == 0 || v.height == 0))
            return set_error(SVO_ERR_INVALID, "view %d: camera rays need width and height", i);
        if (v.width && (uint64_t)v.width * v.height > 0xFFFFFFFFull)
            return set_error(SVO_ERR_LIMIT, "view %d: more than 2^32-1 pixels", i);
        if (!v.width && v.n_rays > 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "view %d: more than 2^32-1 rays", i);
        if (v.ray_scale != 0.0f) b->any_lod = true;
    }
    b->views.assign(views, views + n_views);
    auto setup = [&]() -> int {
        SVO_CUDA_TRY(cudaGetDevice(&b->device));
        SVO_CUDA_TRY(cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device));
        SVO_CUDA_TRY(cudaMalloc((void **)&b->jobs_d, n_views * sizeof(JobDev)));
        SVO_CUDA_TRY(cudaMalloc((void **)&b->begin_d, (n_views + 1) * sizeof(uint64_t)));
        SVO_CUDA_TRY(cudaMalloc((void **)&b->queue_d, sizeof(unsigned long long)));
        SVO_CUDA_TRY(cudaMalloc((void **)&b->status_d, sizeof(uint32_t)));
        SVO_CUDA_TRY(cudaMemset(b->status_d, 0, sizeof(uint32_t)));
        // Tables are built here, outside any capture; one view without a
        // table puts the whole batch on the word traversal.
        b->all_tab = true;
        for (const auto &v : b->views)
            if (!octree_table(v.octree, nullptr)) b->all_tab = false;
        int rc = allow_large_smem();
        if (rc) return rc;
        return prepare_jobs(b.get(), 8);
    };
    int rc = setup();
    if (rc) {
        svo_batch_destroy(b.release());
        return rc;
    }
    *out = b.release();
    return SVO_OK;
}

int svo_batch_num_slots(svo_batch *b, uint64_t *slots) {
    if (!b || !slots) return set_error(SVO_ERR_INVALID, "null argument");
    *slots = b->total;
    return SVO_OK;
}

int svo_batch_trace(svo_batch *b, const svo_trace_config *cfg, svo_stream stream) {
    if (!b) return set_error(SVO_ERR_INVALID, "null batch");
    svo_trace_config c;
    if (cfg) c = *cfg;
    else svo_batch_default_config(&c);
    if (!config_ok(c)) return set_error(SVO_ERR_INVALID, "bad trace config");
    int rc = prepare_jobs(b, c.tile_w);
    if (rc) return rc;
    return enqueue_trace(b, c, (cudaStream_t)stream);
}

int svo_batch_capture_graph(svo_batch *b, const svo_trace_config *cfg) {
    if (!b) return set_error(SVO_ERR_INVALID, "null batch");
    svo_trace_config c;
    if (cfg) c = *cfg;
    else svo_batch_default_config(&c);
    if (!config_ok(c)) return set_error(SVO_ERR_INVALID, "bad trace config");
    int rc = prepare_jobs(b, c.tile_w);
    if (rc) return rc;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    if (!b->cap_stream) SVO_CUDA_TRY(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
    SVO_CUDA_TRY(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_trace(b, c, b->cap_stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    b->graph = g;
    SVO_CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
    return SVO_OK;
}

int svo_batch_launch_graph(svo_batch *b, svo_stream stream) {
    if (!b || !b->exec) return set_error(SVO_ERR_INVALID, "no captured graph");
    SVO_CUDA_TRY(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
    return SVO_OK;
}

int svo_batch_autotune(svo_batch *b, svo_trace_config *best, float *best_ms, svo_stream stream) {
    if (!b || !best) return set_error(SVO_ERR_INVALID, "null argument");
    cudaStream_t st = (cudaStream_t)stream;
    std::string key = workload_key(b);
    const char *force = getenv("SVO_AUTOTUNE_FORCE");
    if (!(force && *force == '1') && cache_lookup(key, best)) {
        if (best_ms) *best_ms = -1.0f;
        return prepare_jobs(b, best->tile_w);
    }
    std::vector<svo_trace_config> cands;
    auto add = [&](int bt, int refill, int steps, int tw, int chunk, int cache, int cap = 0) {
        svo_trace_config c;
        c.block_threads = bt;
        c.blocks_per_sm = 2048 / bt;
        c.refill_idle = refill;
        c.steps_per_round = steps;
        c.tile_w = tw;
        c.chunk = chunk;
        c.cache_entries = b->all_tab ? cache : 0;
        c.reg_cap = cap;
        if (cache == 0 || b->all_tab) cands.push_back(c);
    };
    // table cache depths: none; 64 entries (levels 0-1 hold at most 9 nodes,
    // level 2 at most 64 more); 256 entries (levels 0-2 hold at most 73)
    for (int cache : {0, 64, 256})
        for (int bt : {128, 256, 512})
            for (int tw : {4, 8, 16})
                for (int chunk : {32, 128}) add(bt, 0, 1, tw, chunk, cache);  // whole-warp tiles, no refill
    // lane refill, default build (64 registers) or 48-register build
    for (int cap : {0, 48})
        for (int bt : {128, 256})
            for (int refill : {8, 16, 32})
                for (int steps : {16, 64})
                    for (int tw : {4, 8}) add(bt, refill, steps, tw, 64, 0, cap);
    cudaEvent_t e0, e1;
    SVO_CUDA_TRY(cudaEventCreate(&e0));
    SVO_CUDA_TRY(cudaEventCreate(&e1));
    float best_t = 1e30f;
    svo_trace_config best_c = cands[0];
    int rc = SVO_OK;
    for (const auto &c : cands) {
        rc = prepare_jobs(b, c.tile_w);
        if (rc) break;
        rc = enqueue_trace(b, c, st);  // warm-up
        if (rc) break;
        float total = 0.0f;
        const int reps = 3;
        for (int r = 0; r < reps && !rc; ++r) {
            cudaEventRecord(e0, st);
            rc = enqueue_trace(b, c, st);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            total += ms;
        }
        if (rc) break;
        float avg = total / reps;
        if (avg < best_t) {
            best_t = avg;
            best_c = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    cache_store(key, best_c, best_t);
    *best = best_c;
    if (best_ms) *best_ms = best_t;
    return prepare_jobs(b, best_c.tile_w);
}

int svo_batch_status(svo_batch *b, uint32_t *flags) {
    if (!b || !flags) return set_error(SVO_ERR_INVALID, "null argument");
    SVO_CUDA_TRY(cudaMemcpy(flags, b->status_d, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    SVO_CUDA_TRY(cudaMemset(b->status_d, 0, sizeof(uint32_t)));
    return SVO_OK;
}

int svo_batch_destroy(svo_batch *b) {
    if (!b) return SVO_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    cudaFree(b->jobs_d);
    cudaFree(b->begin_d);
    cudaFree(b->queue_d);
    cudaFree(b->status_d);
    delete b;
    return SVO_OK;
}

}  // extern "C"
