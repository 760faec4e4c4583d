// sort.cuh — stable LSD radix sort of (uint32 or uint64 key, uint32 value) pairs.
//
// Eight-bit digits, three launches per digit:
//   1. per 4096-item tile, a digit histogram written digit-major
//      (hist[digit * tiles + tile]);
//   2. an exclusive scan of that table (scan.cuh), which gives every
//      (digit, tile) its first output slot;
//   3. a stable scatter: each warp ranks its 512 items in input order with
//      __match_any_sync, warps of a tile are offset by a per-digit scan, and
//      each item lands at slot(digit, tile) + its rank.
// No kernel waits on another CTA, so nothing spins.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "scan.cuh"

namespace svo {

constexpr int kSortWarps = 8;
constexpr int kSortPerLane = 16;
constexpr int kSortTile = kSortWarps * 32 * kSortPerLane;  // 4096

template <typename K>
__global__ void __launch_bounds__(kSortWarps * 32) k_radix_hist(const K *__restrict__ keys, uint64_t n,
                                                               int shift, uint32_t tiles, uint32_t *__restrict__ hist) {
    __shared__ uint32_t cnt[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
        uint64_t k = base + (uint64_t)i;
        if (k < n) atomicAdd(&cnt[(uint32_t)(keys[k] >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(uint64_t)d * tiles + blockIdx.x] = cnt[d];
}

template <typename K>
__global__ void __launch_bounds__(kSortWarps * 32) k_radix_scatter(const K *__restrict__ kin,
                                                                  const uint32_t *__restrict__ vin, uint64_t n,
                                                                  int shift, uint32_t tiles,
                                                                  const uint32_t *__restrict__ slot,
                                                                  K *__restrict__ kout,
                                                                  uint32_t *__restrict__ vout) {
    __shared__ uint32_t wcnt[kSortWarps][256];
    __shared__ uint32_t gbase[256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kSortWarps * 256; i += blockDim.x) (&wcnt[0][0])[i] = 0;
    for (int d = threadIdx.x; d < 256; d += blockDim.x) gbase[d] = slot[(uint64_t)d * tiles + blockIdx.x];
    __syncthreads();

    const uint64_t base = (uint64_t)blockIdx.x * kSortTile + (uint64_t)warp * (32 * kSortPerLane);
    const uint32_t lt = (1u << lane) - 1u;
    K key[kSortPerLane];
    uint32_t rank[kSortPerLane];
#pragma unroll
    for (int j = 0; j < kSortPerLane; ++j) {
        uint64_t i = base + (uint64_t)j * 32 + lane;
        bool valid = i < n;
        key[j] = valid ? kin[i] : K(0);
        uint32_t digit = valid ? ((uint32_t)(key[j] >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t before = valid ? wcnt[warp][digit] : 0u;
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][digit] = before + __popc(peers);
        __syncwarp();
        rank[j] = before + __popc(peers & lt);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        uint32_t run = 0;
        for (int w = 0; w < kSortWarps; ++w) {
            uint32_t c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSortPerLane; ++j) {
        uint64_t i = base + (uint64_t)j * 32 + lane;
        if (i < n) {
            uint32_t digit = (uint32_t)(key[j] >> shift) & 255u;
            uint32_t pos = gbase[digit] + wcnt[warp][digit] + rank[j];
            kout[pos] = key[j];
            vout[pos] = vin[i];
        }
    }
}

// Scratch (in uint32 elements) for radix_sort_pairs over n items.
inline uint64_t radix_scratch_elems(uint64_t n) {
    uint64_t tiles = (n + kSortTile - 1) / kSortTile;
    uint64_t h = 256 * (tiles ? tiles : 1);
    return 2 * h + scan_scratch_elems(h) + 1;
}

// Sorts n pairs (key K = uint32_t or uint64_t, uint32 value) by the low
// `bits` bits of the keys, stably.  The pairs move between (k, v) and
// (k_alt, v_alt); *in_alt tells which pair of arrays holds the result.
// n < 2^32.
template <typename K>
inline cudaError_t radix_sort_pairs(K *k, uint32_t *v, K *k_alt, uint32_t *v_alt, uint64_t n,
                                    int bits, uint32_t *scratch, cudaStream_t st, bool *in_alt) {
    *in_alt = false;
    if (n <= 1 || bits <= 0) return cudaSuccess;
    const uint32_t tiles = (uint32_t)((n + kSortTile - 1) / kSortTile);
    const uint64_t h = 256ull * tiles;
    uint32_t *hist = scratch, *slot = scratch + h, *total = scratch + 2 * h, *sc = scratch + 2 * h + 1;
    K *ki = k, *ko = k_alt;
    uint32_t *vi = v, *vo = v_alt;
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_hist<K><<<tiles, kSortWarps * 32, 0, st>>>(ki, n, shift, tiles, hist);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        e = exclusive_scan<uint32_t, uint32_t>(hist, slot, h, total, sc, st);
        if (e != cudaSuccess) return e;
        k_radix_scatter<K><<<tiles, kSortWarps * 32, 0, st>>>(ki, vi, n, shift, tiles, slot, ko, vo);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        K *tk = ki;
        uint32_t *tv = vi;
        ki = ko;
        vi = vo;
        ko = tk;
        vo = tv;
        *in_alt = !*in_alt;
    }
    return cudaSuccess;
}

}  // namespace svo
