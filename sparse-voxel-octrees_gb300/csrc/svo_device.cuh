// svo_device.cuh — device math for the octree hot path.
//
// Compiled with -fmad=false and IEEE division/sqrt (no fast math) so every
// float operation rounds exactly as the reference's x86-64 build does
// (g++ -O2 without -march performs no contraction).  Comparisons use the
// std::min/std::max forms of the reference, which differ from fminf/fmaxf on
// signed zeros and NaNs.
#pragma once

#include <cstdint>

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
    int32_t ui = (int32_t)((n1 * 0.5f + 0.5f) * scale);
    int32_t vi = (int32_t)((n2 * 0.5f + 0.5f) * scale);
    int32_t ci = (int32_t)(shade * 127.0f);
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

enum : int { kMiss = 0, kLeafHit = 1, kLodHit = 2, kFault = 3 };

// Per-ray traversal state for VoxelOctree::raymarch (VoxelOctree.cpp:207-346).
// The reference's stack holds {uint64 offset, float maxT} per scale; this one
// also keeps the descriptor word so a POP needs no reload (the octree is
// immutable, so the reloaded word would be identical).  Words are addressed
// with 32-bit indices (octrees up to 2^32-1 words).
struct RayResult {
    int status;
    float t;
    uint32_t leaf;
    uint32_t word;
};

// kCountLoads: count the words the reference reads (descriptor at :254 on
// every PUSH/POP/start, far word :279, leaf word :282) instead of caching.
// Every index is checked against n_words; a violation or more than
// kStepCap iterations ends the ray with kFault.
constexpr uint32_t kStepCap = 1u << 20;

template <bool kCountLoads>
__device__ __forceinline__ RayResult raymarch(const uint32_t *__restrict__ oct, uint32_t n_words, float ox, float oy,
                                              float oz, float dx, float dy, float dz, float rayScale,
                                              uint32_t *loads) {
    uint32_t stkParent[kMaxScale + 1];
    float stkMaxT[kMaxScale + 1];
    uint32_t stkDesc[kMaxScale + 1];
    uint32_t nload = 0;
    RayResult res;
    res.status = kMiss;
    res.t = __int_as_float(0x7f800000);
    res.leaf = 0xFFFFFFFFu;
    res.word = 0;

    if (fabsf(dx) < 1e-4f) dx = 1e-4f;
    if (fabsf(dy) < 1e-4f) dy = 1e-4f;
    if (fabsf(dz) < 1e-4f) dz = 1e-4f;

    float dTx = 1.0f / -fabsf(dx);
    float dTy = 1.0f / -fabsf(dy);
    float dTz = 1.0f / -fabsf(dz);
    float bTx = dTx * ox;
    float bTy = dTy * oy;
    float bTz = dTz * oz;

    int octantMask = 7;
    if (dx > 0.0f) { octantMask ^= 1; bTx = 3.0f * dTx - bTx; }
    if (dy > 0.0f) { octantMask ^= 2; bTy = 3.0f * dTy - bTy; }
    if (dz > 0.0f) { octantMask ^= 4; bTz = 3.0f * dTz - bTz; }

    float minT = smax(2.0f * dTx - bTx, smax(2.0f * dTy - bTy, 2.0f * dTz - bTz));
    float maxT = smin(dTx - bTx, smin(dTy - bTy, dTz - bTz));
    minT = smax(minT, 0.0f);

    uint32_t current = 0;
    uint32_t parent = 0;
    int idx = 0;
    float posX = 1.0f, posY = 1.0f, posZ = 1.0f;
    int scale = kMaxScale - 1;
    float scaleExp2 = 0.5f;

    if (1.5f * dTx - bTx > minT) { idx ^= 1; posX = 1.5f; }
    if (1.5f * dTy - bTy > minT) { idx ^= 2; posY = 1.5f; }
    if (1.5f * dTz - bTz > minT) { idx ^= 4; posZ = 1.5f; }

    bool need_load = true;
    uint32_t steps = 0;
    while (scale < kMaxScale) {
        if (++steps > kStepCap) { res.status = kFault; return res; }
        if (need_load) {
            if (parent >= n_words) { res.status = kFault; return res; }
            current = __ldg(oct + parent);
            if (kCountLoads) ++nload;
            need_load = false;
        }
        float cornerTX = posX * dTx - bTx;
        float cornerTY = posY * dTy - bTy;
        float cornerTZ = posZ * dTz - bTz;
        float maxTC = smin(cornerTX, smin(cornerTY, cornerTZ));

        int childShift = idx ^ octantMask;
        uint32_t childMasks = current << childShift;

        if ((childMasks & 0x8000u) && minT <= maxT) {
            if (maxTC * rayScale >= scaleExp2) {
                res.status = kLodHit;
                res.t = maxTC;
                if (kCountLoads) *loads = nload;
                return res;
            }
            float maxTV = smin(maxT, maxTC);
            float half = scaleExp2 * 0.5f;
            float centerTX = half * dTx + cornerTX;
            float centerTY = half * dTy + cornerTY;
            float centerTZ = half * dTz + cornerTZ;

            if (minT <= maxTV) {
                uint64_t childOffset = current >> 18;
                if (current & 0x20000u) {
                    if (parent + 1u >= n_words) { res.status = kFault; return res; }
                    childOffset = (childOffset << 32) | (uint64_t)__ldg(oct + parent + 1);
                    if (kCountLoads) ++nload;
                }
                if (!(childMasks & 0x80u)) {
                    uint64_t li = childOffset + parent +
                                  (uint64_t)__popc(((childMasks >> (8 + childShift)) << childShift) & 127u);
                    if (li >= n_words) { res.status = kFault; return res; }
                    res.word = __ldg(oct + li);
                    res.leaf = (uint32_t)li;
                    res.status = kLeafHit;
                    res.t = minT;
                    if (kCountLoads) *loads = nload + 1;
                    return res;
                }
                stkParent[scale] = parent;
                stkMaxT[scale] = maxT;
                stkDesc[scale] = current;

                uint32_t siblingCount = __popc(childMasks & 127u);
                uint64_t np = (uint64_t)parent + childOffset + siblingCount;
                if (current & 0x10000u) np += siblingCount;
                if (np >= n_words) { res.status = kFault; return res; }
                parent = (uint32_t)np;

                idx = 0;
                scale--;
                scaleExp2 = half;
                if (centerTX > minT) { idx ^= 1; posX += scaleExp2; }
                if (centerTY > minT) { idx ^= 2; posY += scaleExp2; }
                if (centerTZ > minT) { idx ^= 4; posZ += scaleExp2; }
                maxT = maxTV;
                need_load = true;
                continue;
            }
        }

        int stepMask = 0;
        if (cornerTX <= maxTC) { stepMask ^= 1; posX -= scaleExp2; }
        if (cornerTY <= maxTC) { stepMask ^= 2; posY -= scaleExp2; }
        if (cornerTZ <= maxTC) { stepMask ^= 4; posZ -= scaleExp2; }

        minT = maxTC;
        idx ^= stepMask;

        if ((idx & stepMask) != 0) {
            uint32_t differing = 0;
            if (stepMask & 1) differing |= __float_as_uint(posX) ^ __float_as_uint(posX + scaleExp2);
            if (stepMask & 2) differing |= __float_as_uint(posY) ^ __float_as_uint(posY + scaleExp2);
            if (stepMask & 4) differing |= __float_as_uint(posZ) ^ __float_as_uint(posZ + scaleExp2);
            scale = (int)(__float_as_uint((float)(int32_t)differing) >> 23) - 127;
            scaleExp2 = __uint_as_float((uint32_t)(scale - kMaxScale + 127) << 23);
            if (scale >= kMaxScale || scale < 0) break;  // exits the tree (miss)

            parent = stkParent[scale];
            maxT = stkMaxT[scale];
            uint32_t shX = __float_as_uint(posX) >> scale;
            uint32_t shY = __float_as_uint(posY) >> scale;
            uint32_t shZ = __float_as_uint(posZ) >> scale;
            posX = __uint_as_float(shX << scale);
            posY = __uint_as_float(shY << scale);
            posZ = __uint_as_float(shZ << scale);
            idx = (int)((shX & 1u) | ((shY & 1u) << 1) | ((shZ & 1u) << 2));
            if (kCountLoads) {
                need_load = true;
            } else {
                current = stkDesc[scale];
            }
        }
    }
    if (kCountLoads) *loads = nload;
    return res;  // miss
}

}  // namespace svo
