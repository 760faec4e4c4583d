// host_traversal.cpp — the library's device traversal (csrc/svo_device.cuh:
// ray_init / ray_step, both word-index widths) compiled for the host, so the
// CPU tests can hold the product's step logic against the oracle without a
// GPU.  The CUDA intrinsics it uses are given their plain C++ meanings; the
// FP operations are the same IEEE float operations (built with
// -ffp-contract=off, as the device code is built with -fmad=false).
#include <cmath>
#include <cstdint>
#include <cstring>

#define __device__
#define __forceinline__ inline

struct uint4 {
    uint32_t x, y, z, w;
};
static inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return uint4{x, y, z, w}; }
static inline uint32_t __ldg(const uint32_t *p) { return *p; }
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
