// svo_device.cuh — device math for the octree hot path.
//
// Compiled with -fmad=false and IEEE division/sqrt (no fast math) so every
// float operation rounds exactly as the reference's x86-64 build does
// (g++ -O2 without -march performs no contraction).  Comparisons use the
// std::min/std::max forms of the reference, which differ from fminf/fmaxf on
// signed zeros and NaNs.
#pragma once

#include <cstdint>
#include <type_traits>

namespace svo {

constexpr int kMaxScale = 23;  // VoxelOctree.hpp:38

__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }

// Util.hpp:47-58 — Quake III inverse square root, one Newton step.
__device__ __forceinline__ float inv_sqrt(float x) {
    float x2 = x * 0.5f;
    uint32_t i = __float_as_uint(x);
    i = 0x5f3759dfu - (i >> 1);
    float y = __uint_as_float(i);
    y = y * (1.5f - x2 * y * y);
    return y;
}

// Util.hpp:86-100.  Face value 3 lies outside the codec (the reference
// would index past its tables); it is read as face 2.
__device__ __forceinline__ void decompress_material(uint32_t word, float &nx, float &ny, float &nz, float &shade) {
    uint32_t sign = word >> 31;
    uint32_t face = (word >> 29) & 3u;
    float u = (float)((word >> 18) & 0x7FFu) * 4.8852e-4f * 2.0f - 1.0f;
    float v = (float)((word >> 7) & 0x7FFu) * 4.8852e-4f * 2.0f - 1.0f;
    float s = sign ? -1.0f : 1.0f;
    // n[face] = s, n[(face+1)%3] = u, n[(face+2)%3] = v
    if (face == 0) { nx = s; ny = u; nz = v; }
    else if (face == 1) { ny = s; nz = u; nx = v; }
    else { nz = s; nx = u; ny = v; }
    float r = inv_sqrt(nx * nx + ny * ny + nz * nz);
    nx *= r;
    ny *= r;
    nz *= r;
    shade = (float)(word & 0x7Fu) * 1.0f / 127.0f;
}

// float -> int32 truncation as x86-64's cvttss2si performs it (the platform
// the reference is built for): NaN and values outside the int32 range give
// INT32_MIN.  A plain cast on the GPU saturates and maps NaN to 0 instead,
// which changes compressMaterial's word for a NaN normal or shade (a
// degenerate triangle's interpolation weights).
__device__ __forceinline__ int32_t f2i_x86(float f) {
    return (f < 2147483648.0f && f >= -2147483648.0f) ? (int32_t)f : (int32_t)0x80000000u;
}

// Util.hpp:64-84.
__device__ __forceinline__ uint32_t compress_material(float nx, float ny, float nz, float shade) {
    const float scale = (float)((1 << 11) - 1);
    float n[3] = {nx, ny, nz};
    uint32_t face = 0;
    float dominant = fabsf(nx);
    if (fabsf(ny) > dominant) { dominant = fabsf(ny); face = 1; }
    if (fabsf(nz) > dominant) { dominant = fabsf(nz); face = 2; }
    uint32_t sign = n[face] < 0.0f;
    uint32_t f1 = face == 2 ? 0 : face + 1, f2 = face == 0 ? 2 : face - 1;
    float n1 = n[f1] / dominant;
    float n2 = n[f2] / dominant;
    int32_t ui = f2i_x86((n1 * 0.5f + 0.5f) * scale);
    int32_t vi = f2i_x86((n2 * 0.5f + 0.5f) * scale);
    int32_t ci = f2i_x86(shade * 127.0f);
    uint32_t u = (uint32_t)(ui < 0x7FF ? ui : 0x7FF);
    uint32_t v = (uint32_t)(vi < 0x7FF ? vi : 0x7FF);
    uint32_t c = (uint32_t)(ci < 0x7F ? ci : 0x7F);
    return (sign << 31) | (face << 29) | (u << 18) | (v << 7) | c;
}

// Main.cpp:81-90 (grey; the reference returns it in all three channels),
// with Vec3::reflect (math/Vec3.hpp:63-71) and Vec3::dot.
__device__ __forceinline__ float shade_grey(uint32_t word, float dx, float dy, float dz, float lx, float ly, float lz) {
    float nx, ny, nz, c;
    decompress_material(word, nx, ny, nz, c);
    float proj = (nx * dx + ny * dy + nz * dz) * 2.0f;
    float rx = dx - nx * proj;
    float ry = dy - ny * proj;
    float rz = dz - nz * proj;
    float d = smax(lx * rx + ly * ry + lz * rz, 0.0f);
    float specular = d * d;
    return c * 0.9f * fabsf(lx * nx + ly * ny + lz * nz) + specular * 0.2f;
}

// The viewer's 8-bit colour of a traced pixel (renderTile, Main.cpp:126-131,
// the non-Apple byte order): c = uint32(std::min(shade, 1.0f) * 255.0), the
// product in double, in the three colour bytes, alpha 0xFF.
__device__ __forceinline__ uint32_t pack_rgba8(float grey) {
    const uint32_t c = (uint32_t)((double)smin(grey, 1.0f) * 255.0);
    return c | (c << 8) | (c << 16) | 0xFF000000u;
}

enum : int { kMiss = 0, kLeafHit = 1, kLodHit = 2, kFault = 3 };

// Per-ray traversal state of VoxelOctree::raymarch (VoxelOctree.cpp:207-346),
// split into ray_init (setup, :213-250) and ray_step (one pass of the loop
// body, :252-339) so a persistent kernel can suspend a ray between steps and
// refill idle lanes.
//
// Differences in mechanism (not in results) from the reference:
//   - the reference's stack holds {uint64 offset, float maxT} per scale; here
//     one 16-byte record {parent, maxT, descriptor} per scale, so a PUSH is one
//     store, a POP one load, and a POP needs no descriptor reload (the octree
//     is immutable, so the reloaded word would be identical);
//   - the reference fetches a node's descriptor at the top of the next pass
//     (`if (current == 0)`, :253-254); here it is fetched at the PUSH that
//     enters the node (and at init for the root), the same word;
//   - word indices are checked against n_words; more than kPushCap PUSHes,
//     or a PUSH below scale 0 (both only possible on a corrupt octree), end
//     the ray with kFault.  Every pass that does not PUSH either advances to
//     a sibling or pops towards the root (for a ray without NaN corner
//     distances; ray_init ends those), so the PUSH cap bounds the whole loop;
//   - the per-pass corner minimum uses fminf: for finite rays no operand is
//     NaN or -0 (corner t = pos*dT - bT with pos*dT nonzero), where fminf and
//     the reference's std::min agree bit for bit (a NaN ray never terminates
//     in the reference);
//   - the POP's highest differing bit is 31 - clz(differing) instead of the
//     exponent of (float)differing: equal below 2^24, and at or above it both
//     give a scale >= 23, which leaves the octree.
// Idx: the word-index type, uint32_t for octrees of up to 2^32-1 words (the
// common case, 32-bit index arithmetic), uint64_t for larger ones.
template <typename Idx>
struct RayResultT {
    int status;
    float t;
    Idx leaf;
    uint32_t word;
};
using RayResult = RayResultT<uint32_t>;

struct RayStack {
    uint4 e[kMaxScale];  // {parent low word, maxT bits, descriptor, parent high word} per scale
};

// The table traversal's stack: {table ordinal of the node, maxT bits} per
// scale.  A POP reloads the node's entry (descriptor, children, block) from
// the table, as the reference reloads the descriptor (:253-254, `current =
// 0` at :338), so a PUSH stores 8 bytes instead of 16.
struct TabStack {
    uint2 e[kMaxScale];
};

template <bool kTab>
using RayStackFor = std::conditional_t<kTab, TabStack, RayStack>;

template <typename Idx>
struct RayStateT {
    float dTx, dTy, dTz, bTx, bTy, bTz;
    float minT, maxT, posX, posY, posZ, scaleExp2;
    Idx parent;  // the table traversal keeps the first internal child's table ordinal here
    uint32_t current, pushes, nload;
    uint32_t lbase;  // table traversal: word index of the current node's child block
    uint32_t self;   // table traversal: the current node's table ordinal
    int idx, scale, octantMask;
};
using RayState = RayStateT<uint32_t>;

constexpr uint32_t kPushCap = 1u << 20;

// Initialises the ray's geometry for (o, d) (VoxelOctree.cpp:213-250);
// ray_init adds the root node.
template <typename Idx>
__device__ __forceinline__ void ray_setup(RayStateT<Idx> &s, float ox, float oy, float oz, float dx, float dy,
                                          float dz) {
    if (fabsf(dx) < 1e-4f) dx = 1e-4f;
    if (fabsf(dy) < 1e-4f) dy = 1e-4f;
    if (fabsf(dz) < 1e-4f) dz = 1e-4f;
    s.dTx = 1.0f / -fabsf(dx);
    s.dTy = 1.0f / -fabsf(dy);
    s.dTz = 1.0f / -fabsf(dz);
    s.bTx = s.dTx * ox;
    s.bTy = s.dTy * oy;
    s.bTz = s.dTz * oz;
    s.octantMask = 7;
    if (dx > 0.0f) { s.octantMask ^= 1; s.bTx = 3.0f * s.dTx - s.bTx; }
    if (dy > 0.0f) { s.octantMask ^= 2; s.bTy = 3.0f * s.dTy - s.bTy; }
    if (dz > 0.0f) { s.octantMask ^= 4; s.bTz = 3.0f * s.dTz - s.bTz; }
    s.minT = smax(2.0f * s.dTx - s.bTx, smax(2.0f * s.dTy - s.bTy, 2.0f * s.dTz - s.bTz));
    s.maxT = smin(s.dTx - s.bTx, smin(s.dTy - s.bTy, s.dTz - s.bTz));
    s.minT = smax(s.minT, 0.0f);
    s.idx = 0;
    s.posX = 1.0f;
    s.posY = 1.0f;
    s.posZ = 1.0f;
    s.scale = kMaxScale - 1;
    s.scaleExp2 = 0.5f;
    if (1.5f * s.dTx - s.bTx > s.minT) { s.idx ^= 1; s.posX = 1.5f; }
    if (1.5f * s.dTy - s.bTy > s.minT) { s.idx ^= 2; s.posY = 1.5f; }
    if (1.5f * s.dTz - s.bTz > s.minT) { s.idx ^= 4; s.posZ = 1.5f; }
    s.pushes = 0;
    s.nload = 1;
    // A ray with a NaN corner distance on some axis (a NaN origin or
    // direction component, or an infinite origin along an infinite
    // direction; dT itself is never infinite) has no result in the
    // reference: with NaN on all three axes VoxelOctree::raymarch never
    // leaves its loop (no corner is <= the NaN minimum, so it neither
    // advances nor pops), otherwise its path hangs on std::min's operand
    // order around the NaN.  Such a ray ends as a miss: its state becomes
    // one whose first pass steps out of the root (every corner distance is
    // -1 at pos 1, so stepMask = 7, and the POP finds scale 23).
    if (isnan(s.dTx + s.bTx) || isnan(s.dTy + s.bTy) || isnan(s.dTz + s.bTz)) {
        s.dTx = s.dTy = s.dTz = -1.0f;
        s.bTx = s.bTy = s.bTz = 0.0f;
        s.posX = s.posY = s.posZ = 1.0f;
        s.idx = 0;
        s.minT = 1.0f;
        s.maxT = 0.0f;
    }
}

// Initialises the state for ray (o, d) and fetches the root descriptor
// (n_words >= 1 for every octree handle).
template <typename Idx>
__device__ __forceinline__ void ray_init(RayStateT<Idx> &s, const uint32_t *__restrict__ oct, float ox, float oy,
                                         float oz, float dx, float dy, float dz) {
    ray_setup(s, ox, oy, oz, dx, dy, dz);
    s.parent = 0;
    s.current = __ldg(oct);
}

// The same for the table traversal: the root's table entry (ordinal 0).
__device__ __forceinline__ void ray_init(RayState &s, const uint4 *__restrict__ tab, float ox, float oy, float oz,
                                         float dx, float dy, float dz) {
    ray_setup(s, ox, oy, oz, dx, dy, dz);
    uint4 r = __ldg(tab);
    s.current = r.x;
    s.parent = r.y;
    s.lbase = r.z;
    s.self = 0;
}

// One pass of the loop body.  Returns false while the ray continues; true
// when it has finished, with `res` filled (status kMiss/kLeafHit/kLodHit/kFault).
// kCountLoads: also count the words the reference reads (descriptor at :254
// at the start and after every PUSH and POP, far word :279, leaf word :282)
// in s.nload.  kLod: evaluate the level-of-detail exit (:265-268); with
// rayScale == 0 that test is always false, so kLod=false skips it.
template <bool kCountLoads, bool kLod, typename Idx>
__device__ __forceinline__ bool ray_step(RayStateT<Idx> &s, RayStack &stk, const uint32_t *__restrict__ oct,
                                         Idx n_words, float rayScale, RayResultT<Idx> &res) {
    // The loop condition of :252 (scale < MaxScale) holds on entry: scale
    // starts at 22, a PUSH lowers it and a POP past the root returns below.
    float cornerTX = s.posX * s.dTx - s.bTx;
    float cornerTY = s.posY * s.dTy - s.bTy;
    float cornerTZ = s.posZ * s.dTz - s.bTz;
    float maxTC = fminf(cornerTX, fminf(cornerTY, cornerTZ));

    int childShift = s.idx ^ s.octantMask;
    uint32_t childMasks = s.current << childShift;

    if ((childMasks & 0x8000u) && s.minT <= s.maxT) {
        if (kLod && maxTC * rayScale >= s.scaleExp2) {
            res.status = kLodHit;
            res.t = maxTC;
            return true;
        }
        float maxTV = fminf(s.maxT, maxTC);
        float half = s.scaleExp2 * 0.5f;
        float centerTX = half * s.dTx + cornerTX;
        float centerTY = half * s.dTy + cornerTY;
        float centerTZ = half * s.dTz + cornerTZ;

        if (s.minT <= maxTV) {
            Idx base, np;
            if constexpr (sizeof(Idx) == 4) {
                // Word indices are below 2^32 (n_words <= 2^32-1), so a far
                // offset's high part (the descriptor's top 14 bits) must be 0
                // and all index sums fit 32 bits unless they wrap, which the
                // bounds checks below catch.
                uint32_t childOffset = s.current >> 18;
                if (s.current & 0x20000u) {
                    if (childOffset != 0u || s.parent + 1u >= n_words) { res.status = kFault; return true; }
                    childOffset = __ldg(oct + s.parent + 1);
                    if (kCountLoads) ++s.nload;
                }
                base = s.parent + childOffset;
                if (base < s.parent) { res.status = kFault; return true; }  // wrapped
            } else {
                // :276-280 with 64-bit indices: offset = (high 14 bits << 32) | far word
                uint64_t childOffset = s.current >> 18;
                if (s.current & 0x20000u) {
                    if (s.parent + 1u >= n_words) { res.status = kFault; return true; }
                    childOffset = (childOffset << 32) | (uint64_t)__ldg(oct + s.parent + 1);
                    if (kCountLoads) ++s.nload;
                }
                base = s.parent + childOffset;
            }
            if (!(childMasks & 0x80u)) {
                Idx li = base + (Idx)__popc(((childMasks >> (8 + childShift)) << childShift) & 127u);
                if (li >= n_words || li < base) { res.status = kFault; return true; }
                res.word = __ldg(oct + li);
                res.leaf = li;
                res.status = kLeafHit;
                res.t = s.minT;
                if (kCountLoads) ++s.nload;
                return true;
            }
            uint32_t siblingCount = __popc(childMasks & 127u);
            np = base + siblingCount;
            if (s.current & 0x10000u) np += siblingCount;
            if (np >= n_words || np < base || s.scale <= 0 || ++s.pushes > kPushCap) { res.status = kFault; return true; }
            if constexpr (sizeof(Idx) == 4)
                stk.e[s.scale] = make_uint4(s.parent, __float_as_uint(s.maxT), s.current, 0u);
            else
                stk.e[s.scale] = make_uint4((uint32_t)s.parent, __float_as_uint(s.maxT), s.current,
                                            (uint32_t)((uint64_t)s.parent >> 32));
            s.parent = np;
            s.current = __ldg(oct + np);
            if (kCountLoads) ++s.nload;

            s.idx = 0;
            s.scale--;
            s.scaleExp2 = half;
            if (centerTX > s.minT) { s.idx ^= 1; s.posX += s.scaleExp2; }
            if (centerTY > s.minT) { s.idx ^= 2; s.posY += s.scaleExp2; }
            if (centerTZ > s.minT) { s.idx ^= 4; s.posZ += s.scaleExp2; }
            s.maxT = maxTV;
            return false;
        }
    }

    int stepMask = 0;
    if (cornerTX <= maxTC) { stepMask ^= 1; s.posX -= s.scaleExp2; }
    if (cornerTY <= maxTC) { stepMask ^= 2; s.posY -= s.scaleExp2; }
    if (cornerTZ <= maxTC) { stepMask ^= 4; s.posZ -= s.scaleExp2; }

    s.minT = maxTC;
    s.idx ^= stepMask;

    if ((s.idx & stepMask) != 0) {
        uint32_t differing = 0;
        if (stepMask & 1) differing |= __float_as_uint(s.posX) ^ __float_as_uint(s.posX + s.scaleExp2);
        if (stepMask & 2) differing |= __float_as_uint(s.posY) ^ __float_as_uint(s.posY + s.scaleExp2);
        if (stepMask & 4) differing |= __float_as_uint(s.posZ) ^ __float_as_uint(s.posZ + s.scaleExp2);
        s.scale = 31 - __clz((int)differing);
        if (s.scale >= kMaxScale || s.scale < 0) {  // left the root: a miss (:341)
            res.status = kMiss;
            return true;
        }
        s.scaleExp2 = __uint_as_float((uint32_t)(s.scale - kMaxScale + 127) << 23);
        uint4 e = stk.e[s.scale];
        if constexpr (sizeof(Idx) == 4)
            s.parent = e.x;
        else
            s.parent = (Idx)e.x | ((Idx)e.w << 32);
        s.maxT = __uint_as_float(e.y);
        s.current = e.z;
        if (kCountLoads) ++s.nload;
        uint32_t shX = __float_as_uint(s.posX) >> s.scale;
        uint32_t shY = __float_as_uint(s.posY) >> s.scale;
        uint32_t shZ = __float_as_uint(s.posZ) >> s.scale;
        s.posX = __uint_as_float(shX << s.scale);
        s.posY = __uint_as_float(shY << s.scale);
        s.posZ = __uint_as_float(shZ << s.scale);
        s.idx = (int)((shX & 1u) | ((shY & 1u) << 1) | ((shZ & 1u) << 2));
    }
    return false;
}

// The loop body over a descriptor table (an octree handle builds one after
// checking the whole tree): entry k = {descriptor word, table ordinal of its
// first internal child, word index of its child block, 0}, the internal
// children of a node holding consecutive ordinals in block order.  A PUSH is
// then one 16-byte load, child = ordinal + (internal siblings before it), and
// needs neither the offset and far-word decoding of :276-280 nor bounds
// checks (the table exists only when every reachable offset, far word, child
// slot and leaf slot is in range and no node is deeper than 22 levels).  The
// stack keeps 8 bytes per scale (the node's ordinal and maxT) and a POP
// reloads the node's entry: local-memory stores are written through to L2,
// and halving them was worth 9% on the 2048^3 terrain step (32 1080p views
// plus shadow rays).  The geometry, the
// visiting order and every result are those of ray_step.
// kStaged: the first stage_n table entries (the top levels, stored first)
// are also in shared memory at stab, and PUSHes and POPs into them read them
// there (the same values as the global table).
template <bool kLod, bool kStaged = false>
__device__ __forceinline__ bool ray_step_tab(RayState &s, TabStack &stk, const uint32_t *__restrict__ words,
                                             const uint4 *__restrict__ tab, float rayScale, RayResult &res,
                                             const uint4 *stab = nullptr, uint32_t stage_n = 0) {
    float cornerTX = s.posX * s.dTx - s.bTx;
    float cornerTY = s.posY * s.dTy - s.bTy;
    float cornerTZ = s.posZ * s.dTz - s.bTz;
    float maxTC = fminf(cornerTX, fminf(cornerTY, cornerTZ));

    int childShift = s.idx ^ s.octantMask;
    uint32_t childMasks = s.current << childShift;

    if ((childMasks & 0x8000u) && s.minT <= s.maxT) {
        if (kLod && maxTC * rayScale >= s.scaleExp2) {
            res.status = kLodHit;
            res.t = maxTC;
            return true;
        }
        float maxTV = fminf(s.maxT, maxTC);
        float half = s.scaleExp2 * 0.5f;
        float centerTX = half * s.dTx + cornerTX;
        float centerTY = half * s.dTy + cornerTY;
        float centerTZ = half * s.dTz + cornerTZ;

        if (s.minT <= maxTV) {
            if (!(childMasks & 0x80u)) {
                uint32_t li = s.lbase + __popc(((childMasks >> (8 + childShift)) << childShift) & 127u);
                res.word = __ldg(words + li);
                res.leaf = li;
                res.status = kLeafHit;
                res.t = s.minT;
                return true;
            }
            stk.e[s.scale] = make_uint2(s.self, __float_as_uint(s.maxT));
            const uint32_t k = s.parent + __popc(childMasks & 127u);
            uint4 c;
            if (kStaged && k < stage_n)
                c = stab[k];
            else
                c = __ldg(tab + k);
            s.self = k;
            s.current = c.x;
            s.parent = c.y;
            s.lbase = c.z;

            s.idx = 0;
            s.scale--;
            s.scaleExp2 = half;
            if (centerTX > s.minT) { s.idx ^= 1; s.posX += s.scaleExp2; }
            if (centerTY > s.minT) { s.idx ^= 2; s.posY += s.scaleExp2; }
            if (centerTZ > s.minT) { s.idx ^= 4; s.posZ += s.scaleExp2; }
            s.maxT = maxTV;
            return false;
        }
    }

    int stepMask = 0;
    if (cornerTX <= maxTC) { stepMask ^= 1; s.posX -= s.scaleExp2; }
    if (cornerTY <= maxTC) { stepMask ^= 2; s.posY -= s.scaleExp2; }
    if (cornerTZ <= maxTC) { stepMask ^= 4; s.posZ -= s.scaleExp2; }

    s.minT = maxTC;
    s.idx ^= stepMask;

    if ((s.idx & stepMask) != 0) {
        uint32_t differing = 0;
        if (stepMask & 1) differing |= __float_as_uint(s.posX) ^ __float_as_uint(s.posX + s.scaleExp2);
        if (stepMask & 2) differing |= __float_as_uint(s.posY) ^ __float_as_uint(s.posY + s.scaleExp2);
        if (stepMask & 4) differing |= __float_as_uint(s.posZ) ^ __float_as_uint(s.posZ + s.scaleExp2);
        s.scale = 31 - __clz((int)differing);
        if (s.scale >= kMaxScale || s.scale < 0) {
            res.status = kMiss;
            return true;
        }
        s.scaleExp2 = __uint_as_float((uint32_t)(s.scale - kMaxScale + 127) << 23);
        const uint2 e = stk.e[s.scale];
        s.self = e.x;
        s.maxT = __uint_as_float(e.y);
        uint4 c;
        if (kStaged && s.self < stage_n)
            c = stab[s.self];
        else
            c = __ldg(tab + s.self);
        s.current = c.x;
        s.parent = c.y;
        s.lbase = c.z;
        uint32_t shX = __float_as_uint(s.posX) >> s.scale;
        uint32_t shY = __float_as_uint(s.posY) >> s.scale;
        uint32_t shZ = __float_as_uint(s.posZ) >> s.scale;
        s.posX = __uint_as_float(shX << s.scale);
        s.posY = __uint_as_float(shY << s.scale);
        s.posZ = __uint_as_float(shZ << s.scale);
        s.idx = (int)((shX & 1u) | ((shY & 1u) << 1) | ((shZ & 1u) << 2));
    }
    return false;
}

// Where an octree has a table (tab != nullptr on the host side, selected at
// compile time here), the table step, else the checked word step.
template <bool kTab, bool kLod>
__device__ __forceinline__ bool ray_step_any(RayState &s, RayStackFor<kTab> &stk, const uint32_t *__restrict__ words,
                                             const uint4 *__restrict__ tab, uint32_t n_words, float rayScale,
                                             RayResult &res) {
    if constexpr (kTab)
        return ray_step_tab<kLod>(s, stk, words, tab, rayScale, res);
    else
        return ray_step<false, kLod, uint32_t>(s, stk, words, n_words, rayScale, res);
}

template <bool kTab>
__device__ __forceinline__ void ray_init_any(RayState &s, const uint32_t *__restrict__ words,
                                             const uint4 *__restrict__ tab, float ox, float oy, float oz, float dx,
                                             float dy, float dz) {
    if constexpr (kTab)
        ray_init(s, tab, ox, oy, oz, dx, dy, dz);
    else
        ray_init(s, words, ox, oy, oz, dx, dy, dz);
}

// A whole ray, checked or over a table.
template <bool kTab>
__device__ __forceinline__ RayResult trace_ray(const uint32_t *__restrict__ words, const uint4 *__restrict__ tab,
                                               uint32_t n_words, float ox, float oy, float oz, float dx, float dy,
                                               float dz, float rayScale) {
    RayStackFor<kTab> stk;
    RayState s;
    RayResult res;
    res.status = kMiss;
    res.t = __int_as_float(0x7f800000);
    res.leaf = 0xFFFFFFFFu;
    res.word = 0;
    ray_init_any<kTab>(s, words, tab, ox, oy, oz, dx, dy, dz);
    if (rayScale != 0.0f) {
        while (!ray_step_any<kTab, true>(s, stk, words, tab, n_words, rayScale, res)) {
        }
    } else {
        while (!ray_step_any<kTab, false>(s, stk, words, tab, n_words, rayScale, res)) {
        }
    }
    return res;
}

template <bool kCountLoads, typename Idx = uint32_t>
__device__ __forceinline__ RayResultT<Idx> raymarch(const uint32_t *__restrict__ oct, Idx n_words, float ox, float oy,
                                                    float oz, float dx, float dy, float dz, float rayScale,
                                                    uint32_t *loads) {
    RayStack stk;
    RayStateT<Idx> s;
    RayResultT<Idx> res;
    res.status = kMiss;
    res.t = __int_as_float(0x7f800000);
    res.leaf = (Idx)~(Idx)0;
    res.word = 0;
    ray_init(s, oct, ox, oy, oz, dx, dy, dz);
    if (rayScale != 0.0f) {
        while (!ray_step<kCountLoads, true, Idx>(s, stk, oct, n_words, rayScale, res)) {
        }
    } else {
        while (!ray_step<kCountLoads, false, Idx>(s, stk, oct, n_words, rayScale, res)) {
        }
    }
    if (kCountLoads) *loads = s.nload;
    return res;
}

}  // namespace svo
