// octree_table.cuh — the per-node check behind the descriptor table that the
// table traversal (ray_step_tab in svo_device.cuh) walks.
//
// The table is built breadth first from the root (octree_table.cu): level 0
// is the root, the internal children of the level-L nodes, in node order and
// within a node in block order, are level L+1, and entry k holds
//   {descriptor word, ordinal of its first internal child, word index of its
//    child block, 0}.
// A table is built only when every node reachable from the root passes
// table_node; otherwise the octree keeps the checked traversal, which ends a
// ray at the first out-of-range index with kFault exactly where it did.
#pragma once

#include <cstdint>

namespace svo {

__host__ __device__ inline uint32_t popc32(uint32_t v) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__popc(v);
#else
    return (uint32_t)__builtin_popcount(v);
#endif
}

// Deepest level that may hold internal children: a PUSH from a level-L node
// happens at scale 22 - L, and the traversal allows it only at scale >= 1.
constexpr int kTableMaxParentLevel = 21;

// Node at word d (< n_words) on tree level `level`.  On success returns true
// with its child block start `cb` and slot stride (1, or 2 when its children
// carry far words, the 0x10000 flag) and its internal-child count; every
// index the traversal can compute from this node — the far word d + 1, leaf
// slots cb + (valid children below), internal-child slots
// cb + stride * (internal children below) — then lies below n_words.
// Fails on: a non-leaf bit outside the valid mask, a zero child offset, a
// far offset with bits above 32, a child block past the end, internal
// children below kTableMaxParentLevel.  A node with no valid child has no
// block (cb = 0).
__host__ __device__ inline bool table_node(const uint32_t *words, uint32_t n_words, uint32_t d, int level,
                                           uint32_t &cb, uint32_t &stride, uint32_t &n_int) {
    const uint32_t desc = words[d];
    const uint32_t valid = (desc >> 8) & 0xFFu, nonleaf = desc & 0xFFu;
    cb = 0;
    stride = (desc & 0x10000u) ? 2u : 1u;
    n_int = 0;
    if (nonleaf & ~valid) return false;
    if (valid == 0) return true;
    uint64_t off = desc >> 18;
    if (desc & 0x20000u) {
        if (off != 0 || (uint64_t)d + 1 >= n_words) return false;
        off = words[d + 1];
    }
    if (off == 0) return false;
    const uint64_t base = (uint64_t)d + off;
    if (base + (uint64_t)popc32(valid) * stride > n_words) return false;
    n_int = popc32(nonleaf);
    if (n_int && level > kTableMaxParentLevel) return false;
    cb = (uint32_t)base;
    return true;
}

}  // namespace svo
