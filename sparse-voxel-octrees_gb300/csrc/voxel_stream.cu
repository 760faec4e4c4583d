// voxel_stream.cu — the .voxel build without the whole grid on the device.
//
// VoxelData(const char *path, size_t mem) (VoxelData.cpp:37-48, 177-291)
// reads its file one cache block at a time, so the reference builds grids far
// larger than memory (README.md:8).  This build streams the file in z slabs of
// a multiple of 16 slices through pinned staging; per slab, one CTA per 16^3
// brick counts and then emits the brick's occupied voxels as (global Morton
// key, word) in local Morton order.  The rules that depend on the whole grid
// use global coordinates: the dropped last z slice of an odd depth (when the
// reference's cache block is at least 4, VoxelData.cpp:163-170) and the cache
// blocks that hold any voxel (the top lookup table, VoxelData.cpp:120-158).
// Slabs are runs of the global order, not a contiguous range of it, so one
// stable radix sort of the 64-bit keys orders all voxels before the level
// build (build_from_sorted_device).  The result is the word stream of the
// in-memory build.
#include <algorithm>
#include <cstdio>
#include <memory>
#include <vector>

#include "morton.cuh"
#include "scan.cuh"
#include "sort.cuh"
#include "svo_internal.h"

namespace svo {
namespace {

constexpr int kSlabThreads = 256;
constexpr int kSlabBrick = 16;

struct SlabGeom {
    const uint32_t *slab;  // nz slices of w x h words
    int w, h, nz;
    int z0;                // global z of the slab's first slice (a multiple of 16)
    int d;                 // global depth
    int drop;              // the global z == d-1 slice is left out
    int log_block;         // reference cache-block edge
    uint8_t *topflag;      // Morton-indexed cache blocks that hold a voxel (null: single block)
    int bx_n, by_n;        // bricks per row and column
};

__device__ __forceinline__ void slab_brick(const SlabGeom &g, uint64_t b, int &x0, int &y0, int &z0) {
    x0 = (int)(b % (uint64_t)g.bx_n) * kSlabBrick;
    uint64_t r = b / (uint64_t)g.bx_n;
    y0 = (int)(r % (uint64_t)g.by_n) * kSlabBrick;
    z0 = (int)(r / (uint64_t)g.by_n) * kSlabBrick;
}

__global__ void __launch_bounds__(kSlabThreads) k_slab_count(SlabGeom g, uint64_t n_bricks, uint32_t *__restrict__ counts) {
    constexpr int E = kSlabBrick, cells = E * E * E;
    for (uint64_t b = blockIdx.x; b < n_bricks; b += gridDim.x) {
        int x0, y0, z0;
        slab_brick(g, b, x0, y0, z0);
        uint32_t cnt = 0, any = 0;
        for (int c = threadIdx.x; c < cells; c += kSlabThreads) {
            int x = x0 + (c & (E - 1)), y = y0 + ((c >> 4) & (E - 1)), z = z0 + (c >> 8);
            if (x < g.w && y < g.h && z < g.nz) {
                uint32_t v = __ldg(g.slab + (uint64_t)x + (uint64_t)g.w * ((uint64_t)y + (uint64_t)g.h * z));
                if (v) {
                    const int gz = g.z0 + z;
                    any = 1;
                    if (!(g.drop && gz == g.d - 1)) ++cnt;
                    if (g.topflag && g.log_block < 4)
                        g.topflag[morton3((uint32_t)x >> g.log_block, (uint32_t)y >> g.log_block,
                                          (uint32_t)gz >> g.log_block)] = 1;
                }
            }
        }
        uint32_t total;
        block_excl_scan<uint32_t>(cnt, &total);
        int block_any = __syncthreads_or(any);
        if (threadIdx.x == 0) {
            counts[b] = total;
            if (block_any && g.topflag && g.log_block >= 4)
                g.topflag[morton3((uint32_t)x0 >> g.log_block, (uint32_t)y0 >> g.log_block,
                                  (uint32_t)(g.z0 + z0) >> g.log_block)] = 1;
        }
    }
}

__global__ void __launch_bounds__(kSlabThreads) k_slab_emit(SlabGeom g, uint64_t n_bricks, const uint32_t *__restrict__ counts,
                                                          const uint64_t *__restrict__ offsets, uint64_t base,
                                                          uint64_t *__restrict__ keys, uint32_t *__restrict__ payload) {
    constexpr int E = kSlabBrick, cells = E * E * E, per = cells / kSlabThreads;
    __shared__ uint32_t tile[cells];
    for (uint64_t b = blockIdx.x; b < n_bricks; b += gridDim.x) {
        if (counts[b] == 0) continue;  // uniform across the CTA
        int x0, y0, z0;
        slab_brick(g, b, x0, y0, z0);
        for (int c = threadIdx.x; c < cells; c += kSlabThreads) {
            int x = x0 + (c & (E - 1)), y = y0 + ((c >> 4) & (E - 1)), z = z0 + (c >> 8);
            uint32_t v = 0;
            if (x < g.w && y < g.h && z < g.nz && !(g.drop && g.z0 + z == g.d - 1))
                v = __ldg(g.slab + (uint64_t)x + (uint64_t)g.w * ((uint64_t)y + (uint64_t)g.h * z));
            tile[c] = v;
        }
        __syncthreads();
        uint32_t cnt = 0;
        const int m0 = threadIdx.x * per;
        for (int k = 0; k < per; ++k) {
            int m = m0 + k;
            cnt += tile[compact3((uint64_t)m) + E * (compact3((uint64_t)m >> 1) + E * compact3((uint64_t)m >> 2))] != 0;
        }
        uint32_t total;
        uint32_t pre = block_excl_scan<uint32_t>(cnt, &total);
        uint64_t out = base + offsets[b] + pre;
        const uint64_t kbase = morton3((uint32_t)x0 >> 4, (uint32_t)y0 >> 4, (uint32_t)(g.z0 + z0) >> 4) << 12;
        for (int k = 0; k < per; ++k) {
            int m = m0 + k;
            uint32_t v = tile[compact3((uint64_t)m) + E * (compact3((uint64_t)m >> 1) + E * compact3((uint64_t)m >> 2))];
            if (v) {
                keys[out] = kbase | (uint64_t)m;
                payload[out] = v;
                ++out;
            }
        }
        __syncthreads();
    }
}

template <typename T>
struct Scratch {
    T *p = nullptr;
    cudaStream_t st = nullptr;
    Scratch() = default;
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;
    cudaError_t alloc(uint64_t n, cudaStream_t s) {
        st = s;
        return scratch_alloc((void **)&p, (size_t)(n ? n : 1) * sizeof(T), s);
    }
    void release() {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
    }
    ~Scratch() { release(); }
};

#define SVO_SALLOC(buf, n)                                                          \
    do {                                                                            \
        cudaError_t _e = (buf).alloc((n), st);                                      \
        if (_e != cudaSuccess) return ::svo::cuda_fail(_e, "device allocation in streamed build"); \
    } while (0)

}  // namespace

int build_voxel_file_streamed(FILE *fp, int w, int h, int d, uint64_t mem, uint64_t slab_bytes, cudaStream_t st,
                              uint32_t **d_words, uint64_t *n_words, float center[3]) {
    int side = 1;
    while (side < std::max(w, std::max(h, d))) side <<= 1;
    if (side < 16) return set_error(SVO_ERR_INVALID, "streamed build needs a virtual side of at least 16");
    int D = 0;
    while ((1 << D) < side) ++D;
    const int lb = cache_block_log2(w, h, d, mem, 4);
    if (lb < 1) return set_error(SVO_ERR_MEMORY, "memory budget %llu admits no cache block", (unsigned long long)mem);
    const uint64_t plane = (uint64_t)w * h;
    uint64_t nz_slab = std::max<uint64_t>(16, (slab_bytes / (plane * 4)) & ~uint64_t(15));
    nz_slab = std::min<uint64_t>(nz_slab, ((uint64_t)d + 15) & ~uint64_t(15));
    const bool multi_block = lb < D;
    const uint64_t n_blocks = multi_block ? (1ull << (3 * (D - lb))) : 0;
    if (n_blocks > (1ull << 27))
        return set_error(SVO_ERR_LIMIT, "memory budget gives %llu cache blocks; the GPU build supports at most 2^27",
                         (unsigned long long)n_blocks);
    for (int k = 0; k < 3; ++k) center[k] = (float)(k == 0 ? w : k == 1 ? h : d) * 0.5f / (float)side;

    Scratch<uint32_t> slab, counts;
    Scratch<uint64_t> offs, tot;
    Scratch<uint8_t> topflag;
    SVO_SALLOC(slab, plane * nz_slab);
    const int bx_n = (w + 15) / 16, by_n = (h + 15) / 16;
    const uint64_t bricks_max = (uint64_t)bx_n * by_n * (nz_slab / 16);
    SVO_SALLOC(counts, bricks_max);
    SVO_SALLOC(offs, bricks_max);
    SVO_SALLOC(tot, 1);
    Scratch<uint64_t> scan_sc;
    SVO_SALLOC(scan_sc, scan_scratch_elems(bricks_max));
    if (multi_block) {
        SVO_SALLOC(topflag, n_blocks);
        SVO_CUDA_TRY(cudaMemsetAsync(topflag.p, 0, n_blocks, st));
    }
    // pinned staging, two halves so a read overlaps the previous copy
    const size_t stage = (size_t)std::min<uint64_t>(plane * nz_slab * 4, 64ull << 20);
    uint8_t *pin = nullptr;
    SVO_CUDA_TRY(cudaMallocHost((void **)&pin, 2 * stage));
    std::unique_ptr<uint8_t, cudaError_t (*)(void *)> pin_guard(pin, cudaFreeHost);
    cudaEvent_t ev[2];
    SVO_CUDA_TRY(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
    SVO_CUDA_TRY(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard() {
            cudaEventDestroy(e[0]);
            cudaEventDestroy(e[1]);
        }
    } ev_guard{ev};

    Scratch<uint64_t> keys;
    Scratch<uint32_t> pay;
    uint64_t cap = 0, N = 0;
    int half = 0;
    bool half_used[2] = {false, false};
    SlabGeom g;
    g.w = w;
    g.h = h;
    g.d = d;
    g.drop = ((d & 1) && lb >= 2) ? 1 : 0;
    g.log_block = lb;
    g.topflag = multi_block ? topflag.p : nullptr;
    g.bx_n = bx_n;
    g.by_n = by_n;
    for (uint64_t z0 = 0; z0 < (uint64_t)d; z0 += nz_slab) {
        const uint64_t nz = std::min<uint64_t>(nz_slab, (uint64_t)d - z0);
        // file -> pinned -> slab, in stage-sized pieces
        uint8_t *dst = (uint8_t *)slab.p;
        uint64_t left = plane * nz * 4;
        while (left) {
            size_t piece = (size_t)std::min<uint64_t>(left, stage);
            if (half_used[half]) SVO_CUDA_TRY(cudaEventSynchronize(ev[half]));
            uint8_t *buf = pin + (size_t)half * stage;
            if (fread(buf, 1, piece, fp) != piece) return set_error(SVO_ERR_FORMAT, "truncated voxel data");
            SVO_CUDA_TRY(cudaMemcpyAsync(dst, buf, piece, cudaMemcpyHostToDevice, st));
            SVO_CUDA_TRY(cudaEventRecord(ev[half], st));
            half_used[half] = true;
            half ^= 1;
            dst += piece;
            left -= piece;
        }
        g.slab = slab.p;
        g.nz = (int)nz;
        g.z0 = (int)z0;
        const uint64_t nb = (uint64_t)bx_n * by_n * ((nz + 15) / 16);
        const unsigned grid = (unsigned)std::min<uint64_t>(nb, 1u << 20);
        k_slab_count<<<grid, kSlabThreads, 0, st>>>(g, nb, counts.p);
        SVO_CUDA_TRY(cudaGetLastError());
        SVO_CUDA_TRY((exclusive_scan<uint32_t, uint64_t>(counts.p, offs.p, nb, tot.p, scan_sc.p, st)));
        uint64_t n = 0;
        SVO_CUDA_TRY(cudaMemcpyAsync(&n, tot.p, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
        SVO_CUDA_TRY(cudaStreamSynchronize(st));
        if (!n) continue;
        if (N + n > cap) {  // grow the voxel arrays
            uint64_t nc = std::max(N + n, cap * 2);
            Scratch<uint64_t> k2;
            Scratch<uint32_t> p2;
            SVO_SALLOC(k2, nc);
            SVO_SALLOC(p2, nc);
            if (N) {
                SVO_CUDA_TRY(cudaMemcpyAsync(k2.p, keys.p, N * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
                SVO_CUDA_TRY(cudaMemcpyAsync(p2.p, pay.p, N * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
            }
            std::swap(keys.p, k2.p);
            std::swap(pay.p, p2.p);
            cap = nc;
        }
        k_slab_emit<<<grid, kSlabThreads, 0, st>>>(g, nb, counts.p, offs.p, N, keys.p, pay.p);
        SVO_CUDA_TRY(cudaGetLastError());
        N += n;
    }
    slab.release();
    if (N >= 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "%llu occupied voxels exceed 2^32-1", (unsigned long long)N);

    // global Morton order
    Scratch<uint64_t> k_alt;
    Scratch<uint32_t> p_alt, sort_sc;
    SVO_SALLOC(k_alt, N);
    SVO_SALLOC(p_alt, N);
    SVO_SALLOC(sort_sc, radix_scratch_elems(N));
    bool in_alt = false;
    SVO_CUDA_TRY(radix_sort_pairs<uint64_t>(keys.p, pay.p, k_alt.p, p_alt.p, N, 3 * D, sort_sc.p, st, &in_alt));
    const uint64_t *sk = in_alt ? k_alt.p : keys.p;
    const uint32_t *sp = in_alt ? p_alt.p : pay.p;
    return build_from_sorted_device(sk, sp, N, D, lb, g.topflag, st, d_words, n_words);
}

}  // namespace svo
