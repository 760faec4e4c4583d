// build.cu — GPU octree construction from a dense voxel grid.
//
// Replaces VoxelOctree(VoxelData*) (VoxelOctree.cpp:125-205) with its
// ChunkedAllocator far-pointer splice (ChunkedAllocator.hpp:76-114).  The
// reference builds depth first and patches far pointers afterwards; this
// pipeline computes the same word stream in three data-parallel phases:
//
//  1. Extraction.  The grid is read brick by brick (16^3 voxels per CTA,
//     bricks visited in Morton order) and occupied voxels are emitted as
//     (Morton key, payload) pairs in global Morton order.  Child slots in the
//     reference are in descending octant index i, and octant i = 7 - m where
//     m = xbit | ybit<<1 | zbit<<2 (VoxelOctree.cpp:144-146), so ascending
//     Morton order is exactly the reference's depth-first child order.
//  2. Bottom-up levels.  Children are grouped by key>>3 (head flags + scan);
//     each parent gets its valid mask (bit m for child m, i.e. 128>>i) and,
//     from its children's subtree word counts S, the far-pointer decision of
//     VoxelOctree.cpp:172-183: offset_i = (k-i) + sum_{j<i} S_j and the
//     parent's children carry far words when any offset_i > 0x3FFF.
//     S = k*(far ? 2 : 1) + sum_j S_j (k payload words at the bottom level).
//  3. Top-down placement.  Root at 0 with its child block at 1; a parent with
//     block start B puts child i at B + i*stride and child i's block at
//     B + k*stride + sum_{j<i} S_j, then writes the child's descriptor with
//     offset = block - position (plus k-i far words, VoxelOctree.cpp:190-191)
//     and, when far, the low 32 bits in the next word.
//
// VoxelData corner cases (VoxelData.cpp:160-175, 120-158, 211-262) that the
// reference's output depends on, for cache-block edge M chosen from `mem`:
//   - with M >= 4 and odd data depth the last z slice never reaches the
//     low-level lookup table, so its voxels are dropped;
//   - nodes of edge >= M come from the top lookup table, which is built from
//     the full data, so an M-block whose only voxels lie in that slice still
//     appears as a descriptor with no children.
#include <cstdio>
#include <mutex>

#include "morton.cuh"
#include "scan.cuh"
#include "svo_internal.h"

namespace svo {
namespace {

constexpr int kBrickThreads = 256;

struct GridGeom {
    const uint32_t *grid;
    int w, h, d;
    int log_brick;      // brick edge E = 1 << log_brick
    int drop_last_z;    // 1: voxels at z == d-1 are excluded from the output
    int log_block;      // cache-block edge M = 1 << log_block
    uint8_t *topflag;   // per M-block "has any voxel" (Morton-indexed), or null
};

// A 16^3 brick wholly inside the grid, whose rows start on 16-byte
// boundaries, is read as 1024 uint4 (4 per thread of a 256-thread CTA).
// uint4 q of the brick covers x = 4*(q & 3) .. +3, y = (q >> 2) & 15,
// z = q >> 6, i.e. cells 4q .. 4q+3 of the brick's row-major order.
__device__ __forceinline__ bool brick_vec4(const GridGeom &g, int gx0, int gy0, int gz0) {
    return g.log_brick == 4 && kBrickThreads == 256 && gx0 + 16 <= g.w && gy0 + 16 <= g.h && gz0 + 16 <= g.d &&
           (g.w & 3) == 0 && (reinterpret_cast<uintptr_t>(g.grid) & 15) == 0;
}

// Loads the brick's 4 uint4 of this thread, all issued before any is used:
// a scan of the whole grid is bound by the loads in flight, not by the
// instructions that test them.
__device__ __forceinline__ void brick_load4(const GridGeom &g, int gx0, int gy0, int gz0, uint4 (&v)[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int q = threadIdx.x + k * 256;
        const int gx = gx0 + ((q & 3) << 2), gy = gy0 + ((q >> 2) & 15), gz = gz0 + (q >> 6);
        v[k] = __ldg(reinterpret_cast<const uint4 *>(g.grid + (uint64_t)gx +
                                                     (uint64_t)g.w * ((uint64_t)gy + (uint64_t)g.h * gz)));
    }
}

// Phase 1a: per brick, count voxels that survive (V') and flag M-blocks that
// hold any voxel (V).  One CTA per brick; consecutive threads read
// consecutive x so each warp load covers whole 32-byte sectors of a row.
__global__ void __launch_bounds__(kBrickThreads, 8) k_brick_count(GridGeom g, uint64_t n_bricks, uint32_t *__restrict__ counts) {
    const int lb = g.log_brick;
    const int E = 1 << lb;
    const int cells = E * E * E;
    for (uint64_t b = blockIdx.x; b < n_bricks; b += gridDim.x) {
        uint32_t bx = compact3(b), by = compact3(b >> 1), bz = compact3(b >> 2);
        int gx0 = (int)(bx << lb), gy0 = (int)(by << lb), gz0 = (int)(bz << lb);
        uint32_t cnt = 0, any = 0;
        if (brick_vec4(g, gx0, gy0, gz0)) {
            uint4 v[4];
            brick_load4(g, gx0, gy0, gz0, v);
            if (!(g.topflag && g.log_block < lb)) {
                // no cell-level flags: count the row's nonzero words and OR
                // them for the brick's flag (a scan of the grid is otherwise
                // bound by these instructions, not by its loads)
                uint32_t bits = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int gz = gz0 + ((threadIdx.x + k * 256) >> 6);
                    bits |= v[k].x | v[k].y | v[k].z | v[k].w;
                    const uint32_t nz = (uint32_t)(v[k].x != 0u) + (uint32_t)(v[k].y != 0u) +
                                        (uint32_t)(v[k].z != 0u) + (uint32_t)(v[k].w != 0u);
                    if (!(g.drop_last_z && gz == g.d - 1)) cnt += nz;
                }
                any = bits != 0u;
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int q = threadIdx.x + k * 256;
                    const int gx = gx0 + ((q & 3) << 2), gy = gy0 + ((q >> 2) & 15), gz = gz0 + (q >> 6);
                    const uint32_t e[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        if (e[j]) {
                            any = 1;
                            if (!(g.drop_last_z && gz == g.d - 1)) ++cnt;
                            g.topflag[morton3((uint32_t)(gx + j) >> g.log_block, (uint32_t)gy >> g.log_block,
                                              (uint32_t)gz >> g.log_block)] = 1;
                        }
                    }
                }
            }
        } else if (gx0 < g.w && gy0 < g.h && gz0 < g.d) {
            for (int c = threadIdx.x; c < cells; c += kBrickThreads) {
                int gx = gx0 + (c & (E - 1)), gy = gy0 + ((c >> lb) & (E - 1)), gz = gz0 + (c >> (2 * lb));
                if (gx < g.w && gy < g.h && gz < g.d) {
                    uint32_t v = __ldg(g.grid + (uint64_t)gx + (uint64_t)g.w * ((uint64_t)gy + (uint64_t)g.h * gz));
                    if (v) {
                        any = 1;
                        if (!(g.drop_last_z && gz == g.d - 1)) ++cnt;
                        if (g.topflag && g.log_block < lb)
                            g.topflag[morton3((uint32_t)gx >> g.log_block, (uint32_t)gy >> g.log_block,
                                              (uint32_t)gz >> g.log_block)] = 1;
                    }
                }
            }
        }
        uint32_t total;
        block_excl_scan<uint32_t>(cnt, &total);
        int block_any = __syncthreads_or(any);
        if (threadIdx.x == 0) {
            counts[b] = total;
            if (block_any && g.topflag && g.log_block >= lb)
                g.topflag[b >> (3 * (g.log_block - lb))] = 1;
        }
    }
}

// Phase 1b: emit (key, payload) for V' in Morton order.  The brick goes into
// shared memory in local Morton order as it is read (a thread's uint4 holds
// cells x .. x+3 of a row, whose codes are m, m+1, m+8 and m+9 with m the
// code of x), so nothing is decoded afterwards.  Warp w then owns codes
// [w * span, (w + 1) * span): one pass counts its occupied cells with
// ballots, and after the warps' totals are known, a second pass writes their
// keys and payloads at consecutive positions.
__global__ void __launch_bounds__(kBrickThreads) k_brick_emit(GridGeom g, uint64_t n_bricks, const uint32_t *__restrict__ counts,
                                                            const uint64_t *__restrict__ offsets,
                                                            uint64_t *__restrict__ keys, uint32_t *__restrict__ payload) {
    constexpr int kWarps = kBrickThreads / 32;
    __shared__ __align__(16) uint32_t tile[16 * 16 * 16];  // the brick's words by local Morton code
    __shared__ uint32_t wtot[kWarps];
    const int lb = g.log_brick;
    const int E = 1 << lb;
    const int cells = E * E * E;
    const int span = (cells + kWarps - 1) / kWarps;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const int m_lo = wid * span, m_hi = min(cells, m_lo + span);
    for (uint64_t b = blockIdx.x; b < n_bricks; b += gridDim.x) {
        if (counts[b] == 0) continue;  // uniform across the CTA
        uint32_t bx = compact3(b), by = compact3(b >> 1), bz = compact3(b >> 2);
        int gx0 = (int)(bx << lb), gy0 = (int)(by << lb), gz0 = (int)(bz << lb);
        if (brick_vec4(g, gx0, gy0, gz0)) {
            uint4 v[4];
            brick_load4(g, gx0, gy0, gz0, v);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int q = threadIdx.x + k * 256;
                if (g.drop_last_z && gz0 + (q >> 6) == g.d - 1) v[k] = make_uint4(0u, 0u, 0u, 0u);
                const uint32_t m = (uint32_t)morton3((uint32_t)((q & 3) << 2), (uint32_t)((q >> 2) & 15),
                                                     (uint32_t)(q >> 6));
                tile[m] = v[k].x;
                tile[m + 1] = v[k].y;
                tile[m + 8] = v[k].z;
                tile[m + 9] = v[k].w;
            }
        } else {
            for (int c = threadIdx.x; c < cells; c += kBrickThreads) {
                int lx = c & (E - 1), ly = (c >> lb) & (E - 1), lz = c >> (2 * lb);
                int gx = gx0 + lx, gy = gy0 + ly, gz = gz0 + lz;
                uint32_t v = 0;
                if (gx < g.w && gy < g.h && gz < g.d && !(g.drop_last_z && gz == g.d - 1))
                    v = __ldg(g.grid + (uint64_t)gx + (uint64_t)g.w * ((uint64_t)gy + (uint64_t)g.h * gz));
                tile[morton3((uint32_t)lx, (uint32_t)ly, (uint32_t)lz)] = v;
            }
        }
        __syncthreads();
        uint32_t run = 0;
        for (int m0 = m_lo; m0 < m_hi; m0 += 32) {
            const int m = m0 + lane;
            run += (uint32_t)__popc(__ballot_sync(0xffffffffu, m < m_hi && tile[m] != 0u));
        }
        if (lane == 0) wtot[wid] = run;
        __syncthreads();
        uint64_t out = offsets[b];
        for (int w = 0; w < wid; ++w) out += wtot[w];
        const uint64_t kbase = b << (3 * lb);
        for (int m0 = m_lo; m0 < m_hi; m0 += 32) {
            const int m = m0 + lane;
            const uint32_t v = m < m_hi ? tile[m] : 0u;
            const uint32_t ball = __ballot_sync(0xffffffffu, v != 0u);
            if (v) {
                const uint64_t o = out + (uint64_t)__popc(ball & lt);
                keys[o] = kbase | (uint64_t)m;
                payload[o] = v;
            }
            out += (uint64_t)__popc(ball);
        }
        __syncthreads();  // the next brick overwrites tile and wtot
    }
}

// ---- level grouping --------------------------------------------------------
//
// Every level kernel takes its element count twice: `n` from the host and
// `dn`, a device copy or nullptr.  With dn the count stays on the device
// (the small top levels are chained without host round trips); n is then an
// upper bound that sizes the arrays and the grid.

__device__ __forceinline__ uint64_t level_count(uint64_t n, const uint32_t *dn) { return dn ? (uint64_t)*dn : n; }

// head[i] = 1 where child i starts a new parent; zero for i in [count, n), so
// a scan over all n entries totals the parents.
__global__ void k_heads(const uint64_t *__restrict__ key, uint64_t n, const uint32_t *__restrict__ dn,
                        uint32_t *__restrict__ head) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t c = level_count(n, dn);
    head[i] = i < c && (i == 0 || (key[i] >> 3) != (key[i - 1] >> 3)) ? 1u : 0u;
}

__global__ void k_parents_from_heads(const uint64_t *__restrict__ ckey, uint64_t n, const uint32_t *__restrict__ dn,
                                     const uint32_t *__restrict__ head, const uint32_t *__restrict__ pidx,
                                     uint64_t *__restrict__ pkey, uint32_t *__restrict__ pstart) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= level_count(n, dn) || !head[i]) return;
    uint32_t p = pidx[i];
    pkey[p] = ckey[i] >> 3;
    pstart[p] = (uint32_t)i;
}

// pidx holds the exclusive scan of head flags: right for a head, one too high
// for the siblings after it.  Turn it into the parent index of every child.
__global__ void k_child_pidx_from_heads(const uint32_t *__restrict__ head, uint64_t n, const uint32_t *__restrict__ dn,
                                        uint32_t *__restrict__ pidx) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= level_count(n, dn)) return;
    pidx[i] = pidx[i] + head[i] - 1u;
}

// Fused grouping of one level's children (sorted Morton keys) into parents,
// in tiles of kLvlTile children.  k_level_count counts each tile's heads
// (children whose key >> 3 differs from the previous child's); an exclusive
// scan of those counts gives each tile's first parent; k_level_emit stages
// the tile's keys in shared memory and writes every parent's key, first
// child, valid mask and child count.  The keys are read twice and only the
// parents are written, where head flags, a scan over every child and
// separate passes for the parents, the children's parent indices and the
// masks read and wrote about three times as many bytes per child.
constexpr int kLvlThreads = 256, kLvlItems = 8, kLvlTile = kLvlThreads * kLvlItems;

__global__ void __launch_bounds__(kLvlThreads) k_level_count(const uint64_t *__restrict__ ckey, uint64_t n,
                                                             const uint32_t *__restrict__ dn,
                                                             uint32_t *__restrict__ tile_heads) {
    __shared__ uint32_t wsum[kLvlThreads / 32];
    const uint64_t c = level_count(n, dn);
    const uint64_t base = (uint64_t)blockIdx.x * kLvlTile;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint64_t k[kLvlItems], k0[kLvlItems];
    // every load issued before any is used; lane 0 also reads the child
    // before its own (the previous lane's in every other lane)
#pragma unroll
    for (int j = 0; j < kLvlItems; ++j) {
        const uint64_t i = base + (uint64_t)(j * kLvlThreads + threadIdx.x);
        k[j] = i < c ? __ldg(ckey + i) : 0ull;
        k0[j] = (lane == 0 && i > 0 && i < c) ? __ldg(ckey + i - 1) : 0ull;
    }
    uint32_t cnt = 0;
#pragma unroll
    for (int j = 0; j < kLvlItems; ++j) {
        const uint64_t i = base + (uint64_t)(j * kLvlThreads + threadIdx.x);
        uint64_t prev = __shfl_up_sync(0xffffffffu, k[j], 1);
        if (lane == 0) prev = k0[j];
        const bool head = i < c && (i == 0 || (k[j] >> 3) != (prev >> 3));
        cnt += (uint32_t)__popc(__ballot_sync(0xffffffffu, head));
    }
    if (lane == 0) wsum[wid] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
#pragma unroll
        for (int w = 0; w < kLvlThreads / 32; ++w) t += wsum[w];
        tile_heads[blockIdx.x] = t;
    }
}

// Children go through the tile in rounds of kLvlThreads, so each warp holds
// 32 consecutive children per round.  A child's parent index is the number
// of heads up to it, minus one.  A parent's run (at most 8 children) is the
// lanes from its head to the next head; three shuffle steps OR the run's
// octant bits into the head's valid mask, and the head writes the parent.
// A run that continues past its warp's 32 children ends in the next 32
// children's leading run, which that round's lane 0 has already ORed and
// counted (one table entry per round); past the tile's last round it ends
// in the keys that follow the tile, staged in shared memory.
__global__ void __launch_bounds__(kLvlThreads) k_level_emit(const uint64_t *__restrict__ ckey, uint64_t n,
                                                            const uint32_t *__restrict__ dn,
                                                            const uint32_t *__restrict__ tile_first,
                                                            uint64_t *__restrict__ pkey, uint32_t *__restrict__ pstart,
                                                            uint8_t *__restrict__ pmask, uint8_t *__restrict__ pcount) {
    // sk[0]: the child before the tile; sk[1 + q]: child base + q, for q below
    // kLvlTile + 7
    __shared__ uint64_t sk[kLvlTile + 8];
    __shared__ uint32_t wpre[kLvlItems * (kLvlThreads / 32)];  // heads per (round, warp), then their exclusive prefix
    __shared__ uint16_t mh[kLvlItems][kLvlThreads];  // per child: run mask (low 8 bits) and run end lane
    __shared__ uint32_t lead[kLvlItems * (kLvlThreads / 32)];  // per round: its leading run's mask and length
    const uint64_t c = level_count(n, dn);
    const uint64_t base = (uint64_t)blockIdx.x * kLvlTile;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int kWarps = kLvlThreads / 32;
#pragma unroll
    for (int j = 0; j < kLvlItems; ++j) {
        const int q = j * kLvlThreads + threadIdx.x;
        sk[1 + q] = base + q < c ? __ldg(ckey + base + q) : 0ull;
    }
    if (threadIdx.x < 8) {
        if (threadIdx.x == 0)
            sk[0] = (base > 0 && base - 1 < c) ? __ldg(ckey + base - 1) : 0ull;
        else {
            const uint64_t i = base + kLvlTile + threadIdx.x - 1;
            sk[kLvlTile + threadIdx.x] = i < c ? __ldg(ckey + i) : 0ull;
        }
    }
    __syncthreads();
    // heads (parent keys differ: the keys differ above their low 3 bits),
    // kept as this warp's ballot per round
    unsigned hb[kLvlItems];
#pragma unroll
    for (int j = 0; j < kLvlItems; ++j) {
        const int q = j * kLvlThreads + threadIdx.x;
        const bool head = base + q < c && (base + q == 0 || ((sk[1 + q] ^ sk[q]) & ~7ull) != 0ull);
        hb[j] = __ballot_sync(0xffffffffu, head);
        if (lane == 0) wpre[j * kWarps + wid] = (uint32_t)__popc(hb[j]);
    }
    __syncthreads();
    static_assert(kLvlItems * kWarps == 64, "one warp scans two entries per lane");
    if (wid == 0) {
        const uint32_t a0 = wpre[2 * lane], a1 = wpre[2 * lane + 1];
        uint32_t incl = a0 + a1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const uint32_t ex = incl - a0 - a1;
        wpre[2 * lane] = ex;
        wpre[2 * lane + 1] = ex + a0;
    }
    __syncthreads();
    const uint32_t first = tile_first[blockIdx.x];
    const unsigned upto = 0xffffffffu >> (31 - lane);  // lanes 0..lane
    // Pass 2a: each lane's octant bits with its run-mates' after it, and its
    // run's end; each round's leading run (the lanes before its first head,
    // the tail of the previous round's last parent) as one table entry.
#pragma unroll
    for (int j = 0; j < kLvlItems; ++j) {
        const int q = j * kLvlThreads + threadIdx.x;
        const uint64_t i = base + q;
        const bool live = i < c;
        const uint64_t k = sk[1 + q];
        const unsigned b = hb[j];
        // a run ends at the next head or at the first lane past the last
        // child (the live lanes are a prefix of the warp's 32)
        const uint64_t w0 = base + (uint64_t)(q - lane);
        const unsigned livem = w0 >= c ? 0u : (c - w0 >= 32 ? 0xffffffffu : (1u << (uint32_t)(c - w0)) - 1u);
        const unsigned after = (b | ~livem) & ~upto;
        const int hi = after ? __ffs(after) - 1 : 32;
        // octant bits of this lane and the run-mates after it (at most 7),
        // by doubling: runs are contiguous, so lane + d in the run means the
        // lanes between are too
        unsigned m = live ? 1u << (k & 7) : 0u;
#pragma unroll
        for (int d = 1; d < 8; d <<= 1) {
            const unsigned o = __shfl_down_sync(0xffffffffu, m, d);
            if (lane + d < hi) m |= o;
        }
        mh[j][threadIdx.x] = (uint16_t)(m | ((unsigned)hi << 8));
        if (lane == 0) lead[j * kWarps + wid] = (b & 1u) || !live ? 0u : (m | ((unsigned)hi << 8));
    }
    __syncthreads();
    // Pass 2b: the heads write their parents; a run reaching its round's last
    // lane continues in the next round's leading run (runs are at most 8
    // long), and past the tile's last round in the keys that follow it.
#pragma unroll
    for (int j = 0; j < kLvlItems; ++j) {
        const unsigned b = hb[j];
        if (!((b >> lane) & 1u)) continue;
        const int q = j * kLvlThreads + threadIdx.x;
        const uint64_t i = base + q;
        const uint64_t k = sk[1 + q];
        const unsigned v = mh[j][threadIdx.x];
        const int hi = (int)(v >> 8);
        unsigned mm = v & 0xFFu, cnt = (unsigned)(hi - lane);
        if (hi == 32) {
            const int nxt = j * kWarps + wid + 1;  // the next round of 32 children
            if (nxt < kLvlItems * kWarps) {
                const unsigned l = lead[nxt];
                mm |= l & 0xFFu;
                cnt += l >> 8;
            } else {
                for (int t = q + (int)cnt; cnt < 8 && base + t < c && ((sk[1 + t] ^ k) & ~7ull) == 0ull; ++t, ++cnt)
                    mm |= 1u << (sk[1 + t] & 7);
            }
        }
        const uint32_t p = first + wpre[j * kWarps + wid] + (uint32_t)__popc(b & upto) - 1u;
        pkey[p] = k >> 3;
        pstart[p] = (uint32_t)i;
        pmask[p] = (uint8_t)mm;
        pcount[p] = (uint8_t)cnt;
    }
}

// Dense grouping at the cache-block level: blk_first[b] = first child of
// block b (or 0xFFFFFFFF); present = has children or top flag.
__global__ void k_block_first(const uint64_t *__restrict__ ckey, uint64_t n, const uint32_t *__restrict__ dn,
                              const uint32_t *__restrict__ head, uint32_t *__restrict__ blk_first) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= level_count(n, dn) || !head[i]) return;
    blk_first[ckey[i] >> 3] = (uint32_t)i;
}

__global__ void k_block_present(const uint32_t *__restrict__ blk_first, const uint8_t *__restrict__ topflag,
                                uint64_t nb, uint32_t *__restrict__ present) {
    uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    present[b] = (blk_first[b] != 0xFFFFFFFFu || topflag[b]) ? 1u : 0u;
}

__global__ void k_block_parents(const uint32_t *__restrict__ blk_first, const uint32_t *__restrict__ present,
                                const uint32_t *__restrict__ bidx, uint64_t nb, uint64_t n_child,
                                const uint32_t *__restrict__ dn_child, uint64_t *__restrict__ pkey,
                                uint32_t *__restrict__ pstart) {
    uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb || !present[b]) return;
    uint32_t p = bidx[b];
    pkey[p] = b;
    pstart[p] = blk_first[b] != 0xFFFFFFFFu ? blk_first[b] : (uint32_t)level_count(n_child, dn_child);
}

__global__ void k_child_pidx_from_blocks(const uint64_t *__restrict__ ckey, uint64_t n, const uint32_t *__restrict__ dn,
                                         const uint32_t *__restrict__ bidx, uint32_t *__restrict__ pidx) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= level_count(n, dn)) return;
    pidx[i] = bidx[ckey[i] >> 3];
}

// The root exists even over an empty grid: a root level with no node gets
// one, with no children (the device-count form of the host's fix-up).
__global__ void k_root_node(uint32_t *__restrict__ dn, uint64_t *__restrict__ key, uint32_t *__restrict__ start) {
    if (*dn == 0) {
        *dn = 1;
        key[0] = 0;
        start[0] = 0;
    }
}

// Per parent: valid mask and child count from its run of children.
__global__ void k_parent_masks(const uint64_t *__restrict__ pkey, const uint32_t *__restrict__ pstart, uint64_t np,
                               const uint32_t *__restrict__ dnp, const uint64_t *__restrict__ ckey, uint64_t nc,
                               const uint32_t *__restrict__ dnc, uint8_t *__restrict__ mask,
                               uint8_t *__restrict__ count) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= level_count(np, dnp)) return;
    const uint64_t c_n = level_count(nc, dnc);
    uint64_t k = pkey[p];
    uint32_t m = 0, c = 0;
    for (uint64_t i = pstart[p]; i < c_n && c < 8 && (ckey[i] >> 3) == k; ++i, ++c) m |= 1u << (ckey[i] & 7);
    mask[p] = (uint8_t)m;
    count[p] = (uint8_t)c;
}

// The same per parent from its children, one thread per child: the lanes
// holding one parent's children (a run, at most 8) find each other with a
// match and OR their octant bits into the parent's valid mask with one warp
// reduction.  The run's first lane writes mask and count; a run that started
// in the previous warp is that warp's to write, and one that continues past
// this warp is finished by reading its remaining children (at most 7).
// Parents without children (cache blocks only the top table marks, an empty
// root) are zeroed beforehand.
__global__ void k_parent_masks_warp(const uint64_t *__restrict__ ckey, uint64_t nc, const uint32_t *__restrict__ dnc,
                                    const uint32_t *__restrict__ pidx, uint8_t *__restrict__ mask,
                                    uint8_t *__restrict__ count) {
    const uint64_t n = level_count(nc, dnc);
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31u;
    const bool live = i < n;
    const uint32_t p = live ? pidx[i] : 0xFFFFFFFFu;
    const unsigned peers = __match_any_sync(0xffffffffu, p);
    const unsigned m = __reduce_or_sync(peers, live ? 1u << (ckey[i] & 7) : 0u);
    if (!live || lane != (unsigned)(__ffs(peers) - 1)) return;
    if (lane == 0 && i > 0 && pidx[i - 1] == p) return;
    unsigned mm = m, c = (unsigned)__popc(peers);
    for (uint64_t k = i + c; k < n && c < 8 && pidx[k] == p; ++k, ++c) mm |= 1u << (ckey[k] & 7);
    mask[p] = (uint8_t)mm;
    count[p] = (uint8_t)c;
}

// ---- subtree sizes and far-pointer decisions (bottom-up) -------------------

__global__ void k_subtree(uint64_t np, const uint32_t *__restrict__ dnp, const uint8_t *__restrict__ count,
                          const uint32_t *__restrict__ pstart, const uint64_t *__restrict__ childS, int bottom,
                          uint64_t *__restrict__ S, uint8_t *__restrict__ large) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= level_count(np, dnp)) return;
    uint32_t k = count[p];
    if (bottom) {
        S[p] = k;
        large[p] = 0;
        return;
    }
    uint64_t run = 0;
    bool far = false;
    uint32_t s0 = pstart[p];
    for (uint32_t i = 0; i < k; ++i) {
        if ((uint64_t)(k - i) + run > 0x3FFFull) far = true;
        run += childS[s0 + i];
    }
    S[p] = (uint64_t)k * (far ? 2u : 1u) + run;
    large[p] = far ? 1 : 0;
}

// ---- placement (top-down) ---------------------------------------------------

__global__ void k_root_word(const uint8_t *__restrict__ mask, const uint8_t *__restrict__ large, int root_is_bottom,
                            uint32_t *__restrict__ words) {
    uint32_t m = mask[0];
    words[0] = (m << 8) | (root_is_bottom ? 0u : m) | (large[0] ? 0x10000u : 0u) | (1u << 18);
}

// Parents at one level place their (internal) children and write the
// children's descriptors; child_is_bottom selects leafMask = 0.
// Every word write is checked against W; a violation (an internal
// inconsistency) is skipped and reported through *err.
__global__ void k_place(uint64_t np, const uint32_t *__restrict__ dnp, const uint8_t *__restrict__ count,
                        const uint32_t *__restrict__ pstart, const uint8_t *__restrict__ plarge,
                        const uint64_t *__restrict__ pB, const uint64_t *__restrict__ cS,
                        const uint8_t *__restrict__ cmask, const uint8_t *__restrict__ clarge, int child_is_bottom,
                        uint64_t *__restrict__ cB, uint32_t *__restrict__ words, uint64_t W,
                        uint32_t *__restrict__ err) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= level_count(np, dnp)) return;
    uint32_t k = count[p];
    bool far = plarge[p] != 0;
    uint64_t stride = far ? 2 : 1;
    uint64_t B = pB[p];
    uint64_t run = 0;
    uint32_t s0 = pstart[p];
    for (uint32_t i = 0; i < k; ++i) {
        uint32_t c = s0 + i;
        uint64_t pos = B + (uint64_t)i * stride;
        uint64_t blk = B + (uint64_t)k * stride + run;
        run += cS[c];
        cB[c] = blk;
        uint64_t off = blk - pos;
        uint32_t m = cmask[c];
        uint32_t w = (m << 8) | (child_is_bottom ? 0u : m) | (clarge[c] ? 0x10000u : 0u);
        if (pos + (far ? 1 : 0) >= W) {
            atomicOr(err, 1u);
            continue;
        }
        if (far) {
            w |= 0x20000u | (uint32_t)((off >> 32) << 18);
            words[pos + 1] = (uint32_t)off;
        } else {
            w |= (uint32_t)(off << 18);
        }
        words[pos] = w;
    }
}

__global__ void k_place_leaves(uint64_t n, const uint32_t *__restrict__ pidx, uint64_t np,
                               const uint32_t *__restrict__ dnp, const uint32_t *__restrict__ pstart,
                               const uint64_t *__restrict__ pB, const uint32_t *__restrict__ payload,
                               uint32_t *__restrict__ words, uint64_t W, uint32_t *__restrict__ err) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t p = pidx[i];
    if (p >= level_count(np, dnp) || i < pstart[p] || i - pstart[p] >= 8) {
        atomicOr(err, 2u);
        return;
    }
    uint64_t dst = pB[p] + (i - pstart[p]);
    if (dst >= W) {
        atomicOr(err, 4u);
        return;
    }
    words[dst] = payload[i];
}

// The same placement with a lane per child: a warp takes 32 consecutive
// parents, whose children follow one another (at most 256), marks which lane
// owns each child in a per-warp table, and places the children 32 at a time.
// A child's block offset is the sum of the subtree sizes of its earlier
// siblings: a segmented scan over the round's lanes (runs are at most 8
// long, so three shuffle steps), plus what a run that began in the previous
// round carried over.  The descriptors and far words are those of k_place.
__global__ void __launch_bounds__(256) k_place_warp(uint64_t np, const uint32_t *__restrict__ dnp,
                                                    const uint8_t *__restrict__ count,
                                                    const uint32_t *__restrict__ pstart,
                                                    const uint8_t *__restrict__ plarge,
                                                    const uint64_t *__restrict__ pB, const uint64_t *__restrict__ cS,
                                                    const uint8_t *__restrict__ cmask,
                                                    const uint8_t *__restrict__ clarge, int child_is_bottom,
                                                    uint64_t nc, const uint32_t *__restrict__ dnc,
                                                    uint64_t *__restrict__ cB, uint32_t *__restrict__ words,
                                                    uint64_t W, uint32_t *__restrict__ err) {
    __shared__ uint8_t owner[8][256];  // per warp: the lane whose parent holds child s0 + i
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned upto = 0xffffffffu >> (31 - lane);
    const uint64_t n = level_count(np, dnp);
    const uint64_t p0 = ((uint64_t)blockIdx.x * blockDim.x) + (uint64_t)wid * 32;
    if (p0 >= n) return;  // uniform per warp
    const uint64_t p = p0 + lane;
    const bool live = p < n;
    const uint32_t k = live ? count[p] : 0u;
    const uint32_t stride = (live && plarge[p]) ? 2u : 1u;
    const uint64_t s = live ? pstart[p] : 0ull, B = live ? pB[p] : 0ull;
    // parents without children (cache blocks only the top table marks) have
    // none to place; the others' children follow one another
    const unsigned runs = __ballot_sync(0xffffffffu, k != 0);
    if (!runs) return;
    const uint64_t s0 = __shfl_sync(0xffffffffu, s, __ffs(runs) - 1);
    uint32_t before = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, before, o);
        if (lane >= o) before += t;
    }
    before -= k;
    const bool bad = k != 0 && (s != s0 + before || s + k > level_count(nc, dnc));
    if (__any_sync(0xffffffffu, bad)) {
        if (bad) atomicOr(err, 2u);
        return;
    }
    for (uint32_t j = 0; j < k; ++j) owner[wid][before + j] = (uint8_t)lane;
    const uint32_t total = __reduce_max_sync(0xffffffffu, k ? before + k : 0u);
    __syncwarp();
    uint64_t carry = 0;  // subtree sizes of the earlier siblings of the round's first child, from earlier rounds
    for (uint32_t i0 = 0; i0 < total; i0 += 32) {
        const uint32_t i = i0 + lane;
        const bool in = i < total;
        const int l = in ? owner[wid][i] : 0;
        const uint64_t c = s0 + i;
        const uint64_t S = in ? cS[c] : 0ull;
        // the lanes of one parent in this round form a segment
        const bool start = !in || lane == 0 || owner[wid][i - 1] != (uint8_t)l;
        const unsigned starts = __ballot_sync(0xffffffffu, start);
        const int lo = 31 - __clz((int)(starts & upto));
        uint64_t incl = S;
#pragma unroll
        for (int d = 1; d < 8; d <<= 1) {
            const uint64_t t = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane - d >= lo) incl += t;
        }
        const uint64_t Bl = __shfl_sync(0xffffffffu, B, l);
        const uint64_t sl = __shfl_sync(0xffffffffu, s, l);
        const uint32_t kl = __shfl_sync(0xffffffffu, k, l);
        const uint32_t stl = __shfl_sync(0xffffffffu, stride, l);
        // the first segment continues a run from the previous round when its
        // first child is not its parent's first
        const uint64_t add = (lo == 0 && i0 > 0 && s0 + i0 != sl) ? carry : 0ull;
        const uint64_t run = add + incl - S;
        // what the last lane's run carries into the next round
        const uint64_t last_total = __shfl_sync(0xffffffffu, add + incl, 31);
        carry = last_total;
        if (in) {
            const uint64_t jj = c - sl;
            const uint64_t pos = Bl + jj * stl;
            const uint64_t blk = Bl + (uint64_t)kl * stl + run;
            cB[c] = blk;
            const uint64_t off = blk - pos;
            const uint32_t m = cmask[c];
            uint32_t w = (m << 8) | (child_is_bottom ? 0u : m) | (clarge[c] ? 0x10000u : 0u);
            if (pos + (stl == 2u ? 1u : 0u) >= W) {
                atomicOr(err, 1u);
            } else {
                if (stl == 2u) {
                    w |= 0x20000u | (uint32_t)((off >> 32) << 18);
                    words[pos + 1] = (uint32_t)off;
                } else {
                    w |= (uint32_t)(off << 18);
                }
                words[pos] = w;
            }
        }
    }
}

// The leaves: every bottom-level parent's run of leaf words goes into its
// child block, in key order (the slots k_place_leaves fills one leaf at a
// time).  A warp takes 32 consecutive parents, whose runs are consecutive
// (each starts where the previous one ends), so their at most 256 leaves are
// one range: each lane marks its run's slots in a per-warp owner table, then
// the warp copies the range with consecutive lanes on consecutive leaves.
// A run reaching past the word count or the leaves is reported through *err.
__global__ void __launch_bounds__(256) k_place_leaf_runs(uint64_t np, const uint32_t *__restrict__ dnp,
                                                         const uint8_t *__restrict__ count,
                                                         const uint32_t *__restrict__ pstart,
                                                         const uint64_t *__restrict__ pB,
                                                         const uint32_t *__restrict__ payload, uint64_t n_leaves,
                                                         uint32_t *__restrict__ words, uint64_t W,
                                                         uint32_t *__restrict__ err) {
    __shared__ uint8_t owner[8][256];  // per warp: the lane whose parent holds leaf slot s0 + i
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint64_t n = level_count(np, dnp);
    const uint64_t p0 = ((uint64_t)blockIdx.x * blockDim.x) + (uint64_t)wid * 32;
    if (p0 >= n) return;  // uniform per warp
    const uint64_t p = p0 + lane;
    const bool live = p < n;
    const uint32_t k = live ? count[p] : 0u;
    const uint64_t s = live ? pstart[p] : 0ull, B = live ? pB[p] : 0ull;
    // parents without children (cache blocks only the top table marks) have
    // no run; the others' runs follow one another from the first one's start
    const unsigned runs = __ballot_sync(0xffffffffu, k != 0);
    if (!runs) return;
    const uint64_t s0 = __shfl_sync(0xffffffffu, s, __ffs(runs) - 1);
    // the runs must tile the range in lane order: each starts where the
    // earlier lanes' runs end
    uint32_t before = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, before, o);
        if (lane >= o) before += t;
    }
    before -= k;
    const bool bad = k != 0 && (B + k > W || s + k > n_leaves || s != s0 + before);
    if (__any_sync(0xffffffffu, bad)) {
        if (bad) atomicOr(err, 4u);
        return;
    }
    const uint32_t rel = k ? (uint32_t)(s - s0) : 0u;
    for (uint32_t j = 0; j < k; ++j) owner[wid][rel + j] = (uint8_t)lane;
    const uint32_t total = __reduce_max_sync(0xffffffffu, k ? rel + k : 0u);
    __syncwarp();
    // every lane takes the same number of rounds: the shuffles read lanes
    // that may own no leaf of the round
    for (uint32_t i0 = 0; i0 < total; i0 += 32) {
        const uint32_t i = i0 + lane;
        const int l = i < total ? owner[wid][i] : 0;
        const uint64_t Bl = __shfl_sync(0xffffffffu, B, l);
        const uint64_t sl = __shfl_sync(0xffffffffu, s, l);
        if (i < total) words[Bl + (s0 + i - sl)] = payload[s0 + i];
    }
}

__global__ void k_set_u64(uint64_t *p, uint64_t v) { *p = v; }

inline unsigned blocks_for(uint64_t n, int t = 256) {
    uint64_t b = (n + t - 1) / t;
    return (unsigned)(b ? b : 1);  // kernels check their own bounds; never launch an empty grid
}

#define SVO_LAUNCH_CHECK(name)                                        \
    do {                                                              \
        cudaError_t _e = cudaGetLastError();                          \
        if (_e != cudaSuccess) return ::svo::cuda_fail(_e, "launch of " name); \
    } while (0)

// Bump allocator over a few pool chunks for the level build's many
// short-lived arrays.  One stream-ordered allocation and free per array cost
// about 240 driver calls per build, most of them right after a host
// synchronisation, when the GPU waits on the host.  The chunks return to the
// pool (stream-ordered) when the arena is destroyed, after every launch that
// uses them has been enqueued.
class BuildArena {
public:
    explicit BuildArena(cudaStream_t s) : st_(s) {}
    BuildArena(const BuildArena &) = delete;
    BuildArena &operator=(const BuildArena &) = delete;
    ~BuildArena() {
        for (void *c : chunks_) cudaFreeAsync(c, st_);
    }
    cudaError_t alloc(void **p, size_t bytes) {
        bytes = (bytes + 255) & ~size_t(255);
        if (bytes > left_) {
            const size_t cb = std::max(bytes, kChunk);
            void *c = nullptr;
            cudaError_t e = scratch_alloc(&c, cb, st_);
            if (e != cudaSuccess) return e;
            chunks_.push_back(c);
            cur_ = static_cast<char *>(c);
            left_ = cb;
        }
        *p = cur_;
        cur_ += bytes;
        left_ -= bytes;
        return cudaSuccess;
    }

private:
    static constexpr size_t kChunk = size_t(64) << 20;
    cudaStream_t st_;
    std::vector<void *> chunks_;
    char *cur_ = nullptr;
    size_t left_ = 0;
};

// Stream-ordered temporary buffer, from the pool or from a BuildArena.
template <typename T>
struct DevBuf {
    T *p = nullptr;
    cudaStream_t st = nullptr;
    bool owned = false;  // false: memory of a BuildArena (freed with the arena)
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    cudaError_t alloc(uint64_t n, cudaStream_t s) {
        st = s;
        owned = true;
        return scratch_alloc((void **)&p, (size_t)(n ? n : 1) * sizeof(T), s);
    }
    cudaError_t alloc(uint64_t n, BuildArena &a) {
        owned = false;
        return a.alloc((void **)&p, (size_t)(n ? n : 1) * sizeof(T));
    }
    void release() {
        if (p && owned) cudaFreeAsync(p, st);
        p = nullptr;
    }
    ~DevBuf() { release(); }
};

struct LevelArrays {
    uint64_t n = 0;                // node count, or its upper bound when dn != nullptr
    const uint32_t *dn = nullptr;  // the node count on the device (levels chained without round trips)
    DevBuf<uint64_t> key;
    DevBuf<uint32_t> start;
    DevBuf<uint8_t> mask, count, large;
    DevBuf<uint64_t> S, B;
};

#define SVO_TRY_ALLOC(expr)                                                   \
    do {                                                                      \
        cudaError_t _e = (expr);                                              \
        if (_e != cudaSuccess) return ::svo::cuda_fail(_e, "device allocation in build"); \
    } while (0)

template <typename TO>
int scan_to(const uint32_t *in, TO *out, uint64_t n, TO *total_host, cudaStream_t st, BuildArena *arena = nullptr) {
    DevBuf<TO> scratch, tot;
    if (arena) {
        SVO_TRY_ALLOC(scratch.alloc(scan_scratch_elems(n), *arena));
        SVO_TRY_ALLOC(tot.alloc(1, *arena));
    } else {
        SVO_TRY_ALLOC(scratch.alloc(scan_scratch_elems(n), st));
        SVO_TRY_ALLOC(tot.alloc(1, st));
    }
    SVO_CUDA_TRY((exclusive_scan<uint32_t, TO>(in, out, n, tot.p, scratch.p, st)));
    SVO_CUDA_TRY(cudaMemcpyAsync(total_host, tot.p, sizeof(TO), cudaMemcpyDeviceToHost, st));
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    return SVO_OK;
}

// Exclusive scan with the total left on the device (no round trip).
template <typename TO>
int scan_on_device(const uint32_t *in, TO *out, uint64_t n, TO *d_total, cudaStream_t st, BuildArena &arena) {
    DevBuf<TO> scratch;
    SVO_TRY_ALLOC(scratch.alloc(scan_scratch_elems(n), arena));
    SVO_CUDA_TRY((exclusive_scan<uint32_t, TO>(in, out, n, d_total, scratch.p, st)));
    return SVO_OK;
}

// Levels whose children number at most this many are chained on the device.
constexpr uint64_t kDeviceLevels = 1ull << 20;

}  // namespace

int build_from_sorted_device(const uint64_t *d_keys, const uint32_t *d_payload, uint64_t N, int log_side,
                             int log_block, const uint8_t *d_topflag, cudaStream_t st, uint32_t **d_words_out,
                             uint64_t *n_words_out) {
    const int D = log_side;
    const bool multi_block = log_block < D;
    const uint64_t n_blocks = multi_block ? (1ull << (3 * (D - log_block))) : 0;
    if (multi_block && !d_topflag) return set_error(SVO_ERR_INVALID, "build: missing cache-block flags");
    if (N >= 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "%llu occupied voxels exceed 2^32-1", (unsigned long long)N);
    int rc = SVO_OK;
    BuildArena arena(st);  // declared first: released after every array below

    // Phase 2: levels e = 1..D (node edge 2^e); level 0 is the leaves.
    // While a level's children number more than kDeviceLevels, the parent
    // count is read back (exact array sizes).  From the first level with
    // fewer children on, the counts stay on the device (dcount[e]) and the
    // arrays are sized by upper bounds: no host round trip per level.
    std::vector<LevelArrays> lv(D + 1);
    DevBuf<uint32_t> dcount;
    SVO_TRY_ALLOC(dcount.alloc(D + 1, arena));
    const uint64_t *ckey = d_keys;
    uint64_t nc = N;              // children: exact count, or an upper bound when cdn != nullptr
    const uint32_t *cdn = nullptr;  // device count of the children
    bool on_device = false;
    for (int e = 1; e <= D; ++e) {
        LevelArrays &L = lv[e];
        if (!on_device && nc <= kDeviceLevels) on_device = true;
        uint32_t *dn = on_device ? dcount.p + e : nullptr;
        // at most one node per cell of edge 2^e, and never more parents than children
        const uint64_t cells = 3 * (D - e) >= 63 ? ~0ull : 1ull << (3 * (D - e));
        if (multi_block && e == log_block) {
            // Dense grouping over cache blocks, adding blocks that only the top
            // lookup table marks (descriptors without children).
            DevBuf<uint32_t> head, pidx, first, present, bidx;
            SVO_TRY_ALLOC(head.alloc(nc, arena));
            SVO_TRY_ALLOC(pidx.alloc(nc, arena));
            SVO_TRY_ALLOC(first.alloc(n_blocks, arena));
            SVO_TRY_ALLOC(present.alloc(n_blocks, arena));
            SVO_TRY_ALLOC(bidx.alloc(n_blocks, arena));
            if (nc) {
                k_heads<<<blocks_for(nc), 256, 0, st>>>(ckey, nc, cdn, head.p);
                SVO_LAUNCH_CHECK("k_heads");
            }
            SVO_CUDA_TRY(cudaMemsetAsync(first.p, 0xFF, n_blocks * sizeof(uint32_t), st));
            if (nc) k_block_first<<<blocks_for(nc), 256, 0, st>>>(ckey, nc, cdn, head.p, first.p);
            k_block_present<<<blocks_for(n_blocks), 256, 0, st>>>(first.p, d_topflag, n_blocks, present.p);
            SVO_LAUNCH_CHECK("k_block_present");
            if (on_device) {
                rc = scan_on_device<uint32_t>(present.p, bidx.p, n_blocks, dn, st, arena);
                L.n = n_blocks;
            } else {
                uint32_t np = 0;
                rc = scan_to<uint32_t>(present.p, bidx.p, n_blocks, &np, st, &arena);
                L.n = np;
            }
            if (rc) return rc;
            if (e == D && L.n == 0) L.n = 1;  // the root (fixed up below)
            SVO_TRY_ALLOC(L.key.alloc(L.n, arena));
            SVO_TRY_ALLOC(L.start.alloc(L.n, arena));
            SVO_TRY_ALLOC(L.mask.alloc(L.n, arena));
            SVO_TRY_ALLOC(L.count.alloc(L.n, arena));
            // blocks only the top table marks keep mask and count 0
            SVO_CUDA_TRY(cudaMemsetAsync(L.mask.p, 0, L.n, st));
            SVO_CUDA_TRY(cudaMemsetAsync(L.count.p, 0, L.n, st));
            k_block_parents<<<blocks_for(n_blocks), 256, 0, st>>>(first.p, present.p, bidx.p, n_blocks, nc, cdn,
                                                                  L.key.p, L.start.p);
            if (nc) {
                k_child_pidx_from_blocks<<<blocks_for(nc), 256, 0, st>>>(ckey, nc, cdn, bidx.p, pidx.p);
                k_parent_masks_warp<<<blocks_for(nc), 256, 0, st>>>(ckey, nc, cdn, pidx.p, L.mask.p, L.count.p);
                SVO_LAUNCH_CHECK("k_parent_masks_warp");
            }
        } else {
            // Fused grouping: tile head counts, their scan, then the parents.
            const uint64_t tiles = (nc + kLvlTile - 1) / kLvlTile;
            DevBuf<uint32_t> th, tf;
            SVO_TRY_ALLOC(th.alloc(tiles, arena));
            SVO_TRY_ALLOC(tf.alloc(tiles, arena));
            if (nc) {
                k_level_count<<<(unsigned)tiles, kLvlThreads, 0, st>>>(ckey, nc, cdn, th.p);
                SVO_LAUNCH_CHECK("k_level_count");
            }
            if (on_device) {
                if (tiles)
                    rc = scan_on_device<uint32_t>(th.p, tf.p, tiles, dn, st, arena);
                else
                    SVO_CUDA_TRY(cudaMemsetAsync(dn, 0, sizeof(uint32_t), st));
                L.n = std::min(nc, cells);
            } else {
                uint32_t np = 0;
                if (tiles) rc = scan_to<uint32_t>(th.p, tf.p, tiles, &np, st, &arena);
                L.n = np;
            }
            if (rc) return rc;
            if (e == D && L.n == 0) L.n = 1;  // the root (fixed up below)
            SVO_TRY_ALLOC(L.key.alloc(L.n, arena));
            SVO_TRY_ALLOC(L.start.alloc(L.n, arena));
            SVO_TRY_ALLOC(L.mask.alloc(L.n, arena));
            SVO_TRY_ALLOC(L.count.alloc(L.n, arena));
            if (e == D) {  // a root added over an empty grid has no children
                SVO_CUDA_TRY(cudaMemsetAsync(L.key.p, 0, sizeof(uint64_t), st));
                SVO_CUDA_TRY(cudaMemsetAsync(L.start.p, 0, sizeof(uint32_t), st));
                SVO_CUDA_TRY(cudaMemsetAsync(L.mask.p, 0, 1, st));
                SVO_CUDA_TRY(cudaMemsetAsync(L.count.p, 0, 1, st));
            }
            if (nc) {
                k_level_emit<<<(unsigned)tiles, kLvlThreads, 0, st>>>(ckey, nc, cdn, tf.p, L.key.p, L.start.p,
                                                                    L.mask.p, L.count.p);
                SVO_LAUNCH_CHECK("k_level_emit");
            }
        }
        // The root always exists, even over an empty grid.
        if (e == D && on_device) {
            k_root_node<<<1, 1, 0, st>>>(dn, L.key.p, L.start.p);
            SVO_LAUNCH_CHECK("k_root_node");
        }
        L.dn = dn;
        ckey = L.key.p;
        nc = L.n;
        cdn = L.dn;
    }

    // Subtree sizes, bottom-up.
    for (int e = 1; e <= D; ++e) {
        LevelArrays &L = lv[e];
        SVO_TRY_ALLOC(L.S.alloc(L.n, arena));
        SVO_TRY_ALLOC(L.large.alloc(L.n, arena));
        k_subtree<<<blocks_for(L.n), 256, 0, st>>>(L.n, L.dn, L.count.p, L.start.p, e > 1 ? lv[e - 1].S.p : nullptr,
                                                  e == 1, L.S.p, L.large.p);
        SVO_LAUNCH_CHECK("k_subtree");
    }
    uint64_t S_root = 0;
    SVO_CUDA_TRY(cudaMemcpyAsync(&S_root, lv[D].S.p, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    const uint64_t W = 1 + S_root;

    uint32_t *words = nullptr;
    SVO_CUDA_TRY(cudaMallocAsync((void **)&words, (size_t)W * sizeof(uint32_t), st));
    DevBuf<uint32_t> err;
    SVO_TRY_ALLOC(err.alloc(1, arena));
    SVO_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(uint32_t), st));

    // Placement, top-down.
    SVO_TRY_ALLOC(lv[D].B.alloc(1, arena));
    k_set_u64<<<1, 1, 0, st>>>(lv[D].B.p, 1);
    k_root_word<<<1, 1, 0, st>>>(lv[D].mask.p, lv[D].large.p, D == 1, words);
    for (int e = D; e >= 2; --e) {
        LevelArrays &P = lv[e];
        LevelArrays &C = lv[e - 1];
        SVO_TRY_ALLOC(C.B.alloc(C.n, arena));
        k_place_warp<<<blocks_for(P.n), 256, 0, st>>>(P.n, P.dn, P.count.p, P.start.p, P.large.p, P.B.p, C.S.p,
                                                     C.mask.p, C.large.p, e - 1 == 1, C.n, C.dn, C.B.p, words, W,
                                                     err.p);
        SVO_LAUNCH_CHECK("k_place_warp");
    }
    if (N) {
        k_place_leaf_runs<<<blocks_for(lv[1].n), 256, 0, st>>>(lv[1].n, lv[1].dn, lv[1].count.p, lv[1].start.p,
                                                               lv[1].B.p, d_payload, N, words, W, err.p);
        SVO_LAUNCH_CHECK("k_place_leaf_runs");
    }
    uint32_t err_h = 0;
    cudaError_t e = cudaMemcpyAsync(&err_h, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(words);
        return cuda_fail(e, "octree build");
    }
    if (err_h) {
        cudaFree(words);
        return set_error(SVO_ERR_DEVICE, "octree build placement check failed (flags %u)", err_h);
    }
    *d_words_out = words;
    *n_words_out = W;
    return SVO_OK;
}

int build_dense_device(const uint32_t *d_grid, int w, int h, int d, int log_side, int log_block, cudaStream_t st,
                       uint32_t **d_words_out, uint64_t *n_words_out) {
    const int D = log_side;
    const int log_brick = D < 4 ? D : 4;
    const uint64_t n_bricks = 1ull << (3 * (D - log_brick));
    const bool multi_block = log_block < D;

    GridGeom g;
    g.grid = d_grid;
    g.w = w;
    g.h = h;
    g.d = d;
    g.log_brick = log_brick;
    g.drop_last_z = ((d & 1) && log_block >= 2) ? 1 : 0;
    g.log_block = log_block;
    g.topflag = nullptr;

    const uint64_t n_blocks = multi_block ? (1ull << (3 * (D - log_block))) : 0;
    if (n_blocks > (1ull << 27))
        return set_error(SVO_ERR_LIMIT, "memory budget gives %llu cache blocks; the GPU build supports at most 2^27",
                         (unsigned long long)n_blocks);
    DevBuf<uint8_t> topflag;
    if (multi_block) {
        SVO_TRY_ALLOC(topflag.alloc(n_blocks, st));
        SVO_CUDA_TRY(cudaMemsetAsync(topflag.p, 0, n_blocks, st));
        g.topflag = topflag.p;
    }

    // Phase 1: extraction in Morton order.
    DevBuf<uint32_t> bcount;
    DevBuf<uint64_t> boff;
    SVO_TRY_ALLOC(bcount.alloc(n_bricks, st));
    SVO_TRY_ALLOC(boff.alloc(n_bricks, st));
    unsigned grid1 = (unsigned)(n_bricks < (1ull << 20) ? n_bricks : (1ull << 20));
    k_brick_count<<<grid1, kBrickThreads, 0, st>>>(g, n_bricks, bcount.p);
    SVO_LAUNCH_CHECK("k_brick_count");
    uint64_t N = 0;
    int rc = scan_to<uint64_t>(bcount.p, boff.p, n_bricks, &N, st);
    if (rc) return rc;
    if (N >= 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "%llu occupied voxels exceed 2^32-1", (unsigned long long)N);

    DevBuf<uint64_t> lkey;
    DevBuf<uint32_t> lpay;
    SVO_TRY_ALLOC(lkey.alloc(N, st));
    SVO_TRY_ALLOC(lpay.alloc(N, st));
    if (N) {
        k_brick_emit<<<grid1, kBrickThreads, 0, st>>>(g, n_bricks, bcount.p, boff.p, lkey.p, lpay.p);
        SVO_LAUNCH_CHECK("k_brick_emit");
    }
    bcount.release();
    boff.release();

    // Phases 2 and 3.
    return build_from_sorted_device(lkey.p, lpay.p, N, D, log_block, topflag.p, st, d_words_out, n_words_out);
}

}  // namespace svo

// ---- allocation-free build ---------------------------------------------------
//
// svo_octree_build_dense_noalloc: the build above for callers that must not
// allocate device memory at call time.  Its scratch is the file-scope arena
// below (32 MiB, reserved on every device that loads the library until the
// process exits); inputs and the output word buffer come from the caller.
namespace svo {
namespace {

constexpr size_t kNoAllocScratchBytes = 32ull << 20;
constexpr uint64_t kNoAllocMaxVoxels = 1ull << 18;
constexpr int kNoAllocMaxSide = 256;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_build_scratch[kNoAllocScratchBytes];

std::mutex g_scratch_mtx;
void *g_scratch_addr[kNoAllocMaxDevices] = {};

// Device address of the arena for the current device.  The first call on a
// device resolves it (cudaGetSymbolAddress) with that device current.
int scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    SVO_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error(SVO_ERR_LIMIT, "device ordinal %d unsupported", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mtx);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_build_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(build scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = (unsigned char *)g_scratch_addr[dev];
    return SVO_OK;
}

// Bump allocator over the arena; every call starts from offset 0.
struct Arena {
    unsigned char *base;
    size_t used = 0;
    template <typename T>
    T *take(uint64_t n) {
        size_t bytes = ((size_t)(n ? n : 1) * sizeof(T) + 255) & ~size_t(255);
        if (used + bytes > kNoAllocScratchBytes) return nullptr;
        T *p = (T *)(base + used);
        used += bytes;
        return p;
    }
};

#define SVO_ARENA_TAKE(ptr, T, n)                                                                  \
    T *ptr = arena.take<T>(n);                                                                     \
    if (!ptr) return set_error(SVO_ERR_LIMIT, "build scratch (%zu bytes) exhausted", kNoAllocScratchBytes)

template <typename TO>
int arena_scan(Arena &arena, const uint32_t *in, TO *out, uint64_t n, TO *total_host, cudaStream_t st) {
    size_t mark = arena.used;
    SVO_ARENA_TAKE(scratch, TO, scan_scratch_elems(n));
    SVO_ARENA_TAKE(tot, TO, 1);
    SVO_CUDA_TRY((exclusive_scan<uint32_t, TO>(in, out, n, tot, scratch, st)));
    SVO_CUDA_TRY(cudaMemcpyAsync(total_host, tot, sizeof(TO), cudaMemcpyDeviceToHost, st));
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    arena.used = mark;
    return SVO_OK;
}

struct ArenaLevel {
    uint64_t n = 0;
    uint64_t *key = nullptr, *S = nullptr, *B = nullptr;
    uint32_t *start = nullptr;
    uint8_t *mask = nullptr, *count = nullptr, *large = nullptr;
};

int build_dense_noalloc(const uint32_t *d_grid, int w, int h, int d, int log_side, int log_block, cudaStream_t st,
                        uint32_t *d_words, uint64_t capacity, uint64_t *n_words_out) {
    Arena arena;
    int rc = scratch_for_current_device(&arena.base);
    if (rc) return rc;
    const int D = log_side;
    const int log_brick = D < 4 ? D : 4;
    const uint64_t n_bricks = 1ull << (3 * (D - log_brick));
    const bool multi_block = log_block < D;
    const uint64_t n_blocks = multi_block ? (1ull << (3 * (D - log_block))) : 0;

    GridGeom g;
    g.grid = d_grid;
    g.w = w;
    g.h = h;
    g.d = d;
    g.log_brick = log_brick;
    g.drop_last_z = ((d & 1) && log_block >= 2) ? 1 : 0;
    g.log_block = log_block;
    g.topflag = nullptr;
    if (multi_block) {
        SVO_ARENA_TAKE(tf, uint8_t, n_blocks);
        SVO_CUDA_TRY(cudaMemsetAsync(tf, 0, n_blocks, st));  // the arena keeps the previous call's bytes
        g.topflag = tf;
    }
    SVO_ARENA_TAKE(bcount, uint32_t, n_bricks);
    SVO_ARENA_TAKE(boff, uint64_t, n_bricks);
    unsigned grid1 = (unsigned)(n_bricks < (1ull << 20) ? n_bricks : (1ull << 20));
    k_brick_count<<<grid1, kBrickThreads, 0, st>>>(g, n_bricks, bcount);
    SVO_LAUNCH_CHECK("k_brick_count");
    uint64_t N = 0;
    rc = arena_scan<uint64_t>(arena, bcount, boff, n_bricks, &N, st);
    if (rc) return rc;
    if (N > kNoAllocMaxVoxels)
        return set_error(SVO_ERR_LIMIT, "%llu occupied voxels exceed the allocation-free build's limit of %llu",
                         (unsigned long long)N, (unsigned long long)kNoAllocMaxVoxels);
    SVO_ARENA_TAKE(lkey, uint64_t, N);
    SVO_ARENA_TAKE(lpay, uint32_t, N);
    if (N) {
        k_brick_emit<<<grid1, kBrickThreads, 0, st>>>(g, n_bricks, bcount, boff, lkey, lpay);
        SVO_LAUNCH_CHECK("k_brick_emit");
    }

    ArenaLevel lv[17];
    uint32_t *leaf_pidx = nullptr;
    const uint64_t *ckey = lkey;
    uint64_t nc = N;
    for (int e = 1; e <= D; ++e) {
        ArenaLevel &L = lv[e];
        SVO_ARENA_TAKE(head, uint32_t, nc);
        SVO_ARENA_TAKE(pidx, uint32_t, nc);
        if (nc) {
            k_heads<<<blocks_for(nc), 256, 0, st>>>(ckey, nc, nullptr, head);
            SVO_LAUNCH_CHECK("k_heads");
        }
        uint32_t np = 0;
        if (multi_block && e == log_block) {
            SVO_ARENA_TAKE(first, uint32_t, n_blocks);
            SVO_ARENA_TAKE(present, uint32_t, n_blocks);
            SVO_ARENA_TAKE(bidx, uint32_t, n_blocks);
            SVO_CUDA_TRY(cudaMemsetAsync(first, 0xFF, n_blocks * sizeof(uint32_t), st));
            if (nc) k_block_first<<<blocks_for(nc), 256, 0, st>>>(ckey, nc, nullptr, head, first);
            k_block_present<<<blocks_for(n_blocks), 256, 0, st>>>(first, g.topflag, n_blocks, present);
            SVO_LAUNCH_CHECK("k_block_present");
            rc = arena_scan<uint32_t>(arena, present, bidx, n_blocks, &np, st);
            if (rc) return rc;
            L.n = np;
            SVO_ARENA_TAKE(key, uint64_t, np);
            SVO_ARENA_TAKE(start, uint32_t, np);
            L.key = key;
            L.start = start;
            k_block_parents<<<blocks_for(n_blocks), 256, 0, st>>>(first, present, bidx, n_blocks, nc, nullptr, L.key,
                                                                  L.start);
            if (nc) k_child_pidx_from_blocks<<<blocks_for(nc), 256, 0, st>>>(ckey, nc, nullptr, bidx, pidx);
            SVO_LAUNCH_CHECK("k_child_pidx_from_blocks");
        } else {
            rc = arena_scan<uint32_t>(arena, head, pidx, nc, &np, st);
            if (rc) return rc;
            L.n = np;
            SVO_ARENA_TAKE(key, uint64_t, np);
            SVO_ARENA_TAKE(start, uint32_t, np);
            L.key = key;
            L.start = start;
            if (nc) {
                k_parents_from_heads<<<blocks_for(nc), 256, 0, st>>>(ckey, nc, nullptr, head, pidx, L.key, L.start);
                k_child_pidx_from_heads<<<blocks_for(nc), 256, 0, st>>>(head, nc, nullptr, pidx);
                SVO_LAUNCH_CHECK("k_child_pidx_from_heads");
            }
        }
        if (e == D && L.n == 0) {
            L.n = 1;
            SVO_ARENA_TAKE(key, uint64_t, 1);
            SVO_ARENA_TAKE(start, uint32_t, 1);
            L.key = key;
            L.start = start;
            SVO_CUDA_TRY(cudaMemsetAsync(L.key, 0, sizeof(uint64_t), st));
            SVO_CUDA_TRY(cudaMemsetAsync(L.start, 0, sizeof(uint32_t), st));
        }
        SVO_ARENA_TAKE(mask, uint8_t, L.n);
        SVO_ARENA_TAKE(count, uint8_t, L.n);
        L.mask = mask;
        L.count = count;
        k_parent_masks<<<blocks_for(L.n), 256, 0, st>>>(L.key, L.start, L.n, nullptr, ckey, nc, nullptr, L.mask,
                                                        L.count);
        SVO_LAUNCH_CHECK("k_parent_masks");
        if (e == 1) leaf_pidx = pidx;
        ckey = L.key;
        nc = L.n;
    }
    for (int e = 1; e <= D; ++e) {
        ArenaLevel &L = lv[e];
        SVO_ARENA_TAKE(S, uint64_t, L.n);
        SVO_ARENA_TAKE(large, uint8_t, L.n);
        L.S = S;
        L.large = large;
        k_subtree<<<blocks_for(L.n), 256, 0, st>>>(L.n, nullptr, L.count, L.start, e > 1 ? lv[e - 1].S : nullptr, e == 1,
                                                  L.S, L.large);
        SVO_LAUNCH_CHECK("k_subtree");
    }
    uint64_t S_root = 0;
    SVO_CUDA_TRY(cudaMemcpyAsync(&S_root, lv[D].S, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    const uint64_t W = 1 + S_root;
    *n_words_out = W;
    if (W > capacity)
        return set_error(SVO_ERR_LIMIT, "octree needs %llu words; the output buffer holds %llu",
                         (unsigned long long)W, (unsigned long long)capacity);
    SVO_ARENA_TAKE(err, uint32_t, 1);
    SVO_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    SVO_ARENA_TAKE(rootB, uint64_t, 1);
    lv[D].B = rootB;
    k_set_u64<<<1, 1, 0, st>>>(lv[D].B, 1);
    k_root_word<<<1, 1, 0, st>>>(lv[D].mask, lv[D].large, D == 1, d_words);
    for (int e = D; e >= 2; --e) {
        ArenaLevel &P = lv[e];
        ArenaLevel &C = lv[e - 1];
        SVO_ARENA_TAKE(cB, uint64_t, C.n);
        C.B = cB;
        k_place<<<blocks_for(P.n), 256, 0, st>>>(P.n, nullptr, P.count, P.start, P.large, P.B, C.S, C.mask, C.large,
                                                e - 1 == 1, C.B, d_words, W, err);
        SVO_LAUNCH_CHECK("k_place");
    }
    if (N) {
        k_place_leaves<<<blocks_for(N), 256, 0, st>>>(N, leaf_pidx, lv[1].n, nullptr, lv[1].start, lv[1].B, lpay, d_words, W,
                                                      err);
        SVO_LAUNCH_CHECK("k_place_leaves");
    }
    uint32_t err_h = 0;
    SVO_CUDA_TRY(cudaMemcpyAsync(&err_h, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    if (err_h) return set_error(SVO_ERR_DEVICE, "octree build placement check failed (flags %u)", err_h);
    return SVO_OK;
}

}  // namespace
}  // namespace svo

extern "C" int svo_octree_build_dense_noalloc(const uint32_t *d_grid, int w, int h, int d, uint64_t mem,
                                              uint32_t *d_words, uint64_t capacity, uint64_t *n_words,
                                              float center[3], svo_stream stream) {
    using namespace svo;
    if (!d_grid || !d_words || !n_words || !center || w <= 0 || h <= 0 || d <= 0)
        return set_error(SVO_ERR_INVALID, "bad arguments");
    // checked before the doubling below, which would overflow past 2^30
    if (w > kNoAllocMaxSide || h > kNoAllocMaxSide || d > kNoAllocMaxSide)
        return set_error(SVO_ERR_LIMIT, "grid %d x %d x %d exceeds the allocation-free build's limit of side %d", w,
                         h, d, kNoAllocMaxSide);
    int side = 1;
    while (side < w || side < h || side < d) side *= 2;
    if (side < 2) return set_error(SVO_ERR_INVALID, "virtual side %d below 2 (the reference recurses forever)", side);
    int lb = cache_block_log2(w, h, d, mem, 4);
    if (lb < 1) return set_error(SVO_ERR_MEMORY, "memory budget %llu admits no cache block", (unsigned long long)mem);
    int log_side = 0;
    while ((1 << log_side) < side) ++log_side;
    int rc = build_dense_noalloc(d_grid, w, h, d, log_side, lb, (cudaStream_t)stream, d_words, capacity, n_words);
    if (rc) {
        // an error can leave earlier launches queued; they still write to the
        // shared arena, so wait for them before returning (the error already
        // recorded stays the one reported)
        cudaStreamSynchronize((cudaStream_t)stream);
        return rc;
    }
    center[0] = (float)w * 0.5f / (float)side;
    center[1] = (float)h * 0.5f / (float)side;
    center[2] = (float)d * 0.5f / (float)side;
    return SVO_OK;
}
