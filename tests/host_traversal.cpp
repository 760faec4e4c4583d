// host_traversal.cpp — the library's device traversal (csrc/svo_device.cuh:
// ray_init / ray_step for both word-index widths, ray_step_tab over the
// descriptor table) and the table's per-node check (csrc/octree_table.cuh)
// compiled for the host, so the CPU tests can hold the product's step logic
// against the oracle without a GPU.  The table is built here by the same
// breadth-first order as octree_table.cu.  The CUDA intrinsics it uses are
// given their plain C++ meanings; the FP operations are the same IEEE float
// operations (built with -ffp-contract=off, as the device code is built with
// -fmad=false).
#include <cmath>
#include <cstdint>
#include <cstring>

#include <vector>

#define __device__
#define __host__
#define __forceinline__ inline

struct uint4 {
    uint32_t x, y, z, w;
};
static inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return uint4{x, y, z, w}; }
struct uint2 {
    uint32_t x, y;
};
static inline uint2 make_uint2(uint32_t x, uint32_t y) { return uint2{x, y}; }
static inline uint32_t __ldg(const uint32_t *p) { return *p; }
static inline uint4 __ldg(const uint4 *p) { return *p; }
static inline int __popc(uint32_t v) { return __builtin_popcount(v); }
static inline int __clz(int v) { return v ? __builtin_clz((uint32_t)v) : 32; }
static inline uint32_t __float_as_uint(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
static inline float __uint_as_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
static inline float __int_as_float(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}
using std::isnan;

#include "octree_table.cuh"
#include "svo_device.cuh"

namespace {

template <typename Idx>
void run(const uint32_t *oct, uint64_t n_words, const float *rays, uint64_t n, float ray_scale, uint64_t max_steps,
         uint8_t *status, float *t, uint64_t *leaf, uint32_t *word, uint64_t *steps) {
    using namespace svo;
    for (uint64_t i = 0; i < n; ++i) {
        const float *r = rays + 6 * i;
        RayStack stk;
        RayStateT<Idx> s;
        RayResultT<Idx> res;
        res.status = kMiss;
        res.t = __int_as_float(0x7f800000);
        res.leaf = (Idx)~(Idx)0;
        res.word = 0;
        ray_init(s, oct, r[0], r[1], r[2], r[3], r[4], r[5]);
        uint64_t k = 0;
        bool done = false;
        while (k < max_steps && !done) {
            ++k;
            done = ray_scale != 0.0f ? ray_step<false, true, Idx>(s, stk, oct, (Idx)n_words, ray_scale, res)
                                     : ray_step<false, false, Idx>(s, stk, oct, (Idx)n_words, ray_scale, res);
        }
        status[i] = done ? (uint8_t)res.status : (uint8_t)255;  // 255: still running after max_steps
        t[i] = res.t;
        leaf[i] = (uint64_t)res.leaf;
        word[i] = res.word;
        steps[i] = k;
    }
}

}  // namespace

// status: 0 miss, 1 leaf hit, 2 level-of-detail exit, 3 fault, 255 not finished.
extern "C" void host_traverse(const uint32_t *oct, uint64_t n_words, const float *rays, uint64_t n, float ray_scale,
                              int wide, uint64_t max_steps, uint8_t *status, float *t, uint64_t *leaf, uint32_t *word,
                              uint64_t *steps) {
    if (wide)
        run<uint64_t>(oct, n_words, rays, n, ray_scale, max_steps, status, t, leaf, word, steps);
    else
        run<uint32_t>(oct, n_words, rays, n, ray_scale, max_steps, status, t, leaf, word, steps);
}

// Breadth-first table of the octree (see octree_table.cuh).  Returns the
// number of entries, or 0 when some reachable node fails table_node or the
// table would exceed `cap` entries.
extern "C" uint64_t host_build_table(const uint32_t *words, uint32_t n_words, uint32_t *tab, uint64_t cap) {
    std::vector<uint32_t> level{0}, next;
    uint64_t base = 0;
    for (int L = 0; !level.empty(); ++L) {
        const uint64_t next_base = base + level.size();
        next.clear();
        for (size_t i = 0; i < level.size(); ++i) {
            uint32_t cb, stride, n_int;
            if (!svo::table_node(words, n_words, level[i], L, cb, stride, n_int)) return 0;
            if (base + i >= cap) return 0;
            uint32_t *e = tab + 4 * (base + i);
            e[0] = words[level[i]];
            e[1] = (uint32_t)(next_base + next.size());
            e[2] = cb;
            e[3] = 0;
            for (uint32_t j = 0; j < n_int; ++j) next.push_back(cb + j * stride);
        }
        base = next_base;
        level.swap(next);
    }
    return base;
}

extern "C" void host_traverse_tab(const uint32_t *words, const uint32_t *tab, const float *rays, uint64_t n,
                                  float ray_scale, uint64_t max_steps, uint8_t *status, float *t, uint64_t *leaf,
                                  uint32_t *word, uint64_t *steps) {
    using namespace svo;
    const uint4 *tb = reinterpret_cast<const uint4 *>(tab);
    for (uint64_t i = 0; i < n; ++i) {
        const float *r = rays + 6 * i;
        TabStack stk;
        RayState s;
        RayResult res;
        res.status = kMiss;
        res.t = __int_as_float(0x7f800000);
        res.leaf = 0xFFFFFFFFu;
        res.word = 0;
        ray_init(s, tb, r[0], r[1], r[2], r[3], r[4], r[5]);
        uint64_t k = 0;
        bool done = false;
        while (k < max_steps && !done) {
            ++k;
            done = ray_scale != 0.0f ? ray_step_tab<true>(s, stk, words, tb, ray_scale, res)
                                     : ray_step_tab<false>(s, stk, words, tb, ray_scale, res);
        }
        status[i] = done ? (uint8_t)res.status : (uint8_t)255;
        t[i] = res.t;
        leaf[i] = res.leaf;
        word[i] = res.word;
        steps[i] = k;
    }
}
