// scan.cuh — device-wide exclusive prefix sum (reduce, scan tile sums, scan).
//
// Three launches per level of tile sums and no inter-CTA waiting, so nothing
// can spin.  Tiles are 256 threads x 8 items; tile sums are scanned by the
// same routine recursively until they fit one tile.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace svo {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) >= o) v += n;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total (all threads).
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T *total) {
    __shared__ T warp_sums[kScanThreads / 32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T incl = warp_incl_scan(v);
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        T s = lane < kScanThreads / 32 ? warp_sums[lane] : T(0);
        s = warp_incl_scan(s);
        if (lane < kScanThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    T warp_prefix = wid ? warp_sums[wid - 1] : T(0);
    *total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return warp_prefix + incl - v;
}

template <typename TI, typename TO>
__global__ void __launch_bounds__(kScanThreads) k_tile_reduce(const TI *__restrict__ in, uint64_t n, TO *__restrict__ sums) {
    uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    TO acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        uint64_t i = base + (uint64_t)k * kScanThreads + threadIdx.x;
        if (i < n) acc += (TO)in[i];
    }
    TO total;
    block_excl_scan<TO>(acc, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// out[i] = offsets[tile] + exclusive prefix of in within the tile.
template <typename TI, typename TO>
__global__ void __launch_bounds__(kScanThreads) k_tile_scan(const TI *__restrict__ in, uint64_t n,
                                                         const TO *__restrict__ offsets, TO *__restrict__ out,
                                                         TO *__restrict__ grand_total) {
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    TO v[kScanItems];
    TO acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        uint64_t i = base + k;
        v[k] = i < n ? (TO)in[i] : TO(0);
        acc += v[k];
    }
    TO total;
    TO pre = block_excl_scan<TO>(acc, &total);
    TO off = offsets ? offsets[blockIdx.x] : TO(0);
    pre += off;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        uint64_t i = base + k;
        if (i < n) out[i] = pre;
        pre += v[k];
    }
    if (grand_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *grand_total = off + total;
}

// Exclusive scan of n values; writes the grand total to d_total (device).
// scratch must hold scan_scratch_elems(n) elements of TO.
inline uint64_t scan_scratch_elems(uint64_t n) {
    uint64_t s = 0;
    while (n > (uint64_t)kScanTile) {
        n = (n + kScanTile - 1) / kScanTile;
        s += 2 * n;
    }
    return s + 1;
}

template <typename TI, typename TO>
cudaError_t exclusive_scan(const TI *in, TO *out, uint64_t n, TO *d_total, TO *scratch, cudaStream_t st) {
    if (n == 0) return cudaMemsetAsync(d_total, 0, sizeof(TO), st);
    uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 1) {
        k_tile_scan<TI, TO><<<1, kScanThreads, 0, st>>>(in, n, (const TO *)nullptr, out, d_total);
        return cudaGetLastError();
    }
    TO *sums = scratch;
    TO *sums_scanned = scratch + tiles;
    k_tile_reduce<TI, TO><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, sums);
    cudaError_t e = exclusive_scan<TO, TO>(sums, sums_scanned, tiles, d_total, scratch + 2 * tiles, st);
    if (e != cudaSuccess) return e;
    k_tile_scan<TI, TO><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, sums_scanned, out, d_total);
    return cudaGetLastError();
}

}  // namespace svo
