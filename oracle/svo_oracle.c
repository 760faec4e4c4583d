/*
 * svo_oracle.c — CPU restatement of the reference's octree hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see svo_oracle.h).  Compiled with -O2
 * -ffp-contract=off and no -march so that every float operation rounds the
 * way the reference's own build does.  Parity of this file with the
 * reference is pinned by tests/test_oracle_vs_reference.py (against the
 * reference compiled in place) and tests/test_golden.py (committed fixtures).
 */
#define _GNU_SOURCE
#include "svo_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- helpers */

static inline float bits_to_float(uint32_t i) { float f; memcpy(&f, &i, 4); return f; }
static inline uint32_t float_to_bits(float f) { uint32_t i; memcpy(&i, &f, 4); return i; }
/* std::max / std::min semantics (including their NaN and signed-zero cases). */
static inline float smax(float a, float b) { return (a < b) ? b : a; }
static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline int imin(int a, int b) { return (b < a) ? b : a; }

static const int MOD3[5] = {0, 1, 2, 0, 1};

void svo_oracle_free(void *p) { free(p); }

/* ---------------------------------------------------------- material codec */

/* Util.hpp:47-58 */
float svo_oracle_inv_sqrt(float x) {
    float x2 = x * 0.5f;
    float y = x;
    uint32_t i = float_to_bits(y);
    i = 0x5f3759dfu - (i >> 1);
    y = bits_to_float(i);
    y = y * (1.5f - x2 * y * y);
    return y;
}

/* float -> int32 truncation with x86-64 cvttss2si semantics (the reference's
 * platform): NaN and out-of-range values give INT32_MIN.  A plain C cast is
 * undefined there, and Arm's conversion saturates and maps NaN to 0. */
static inline int32_t f2i_x86(float f) {
    return (f < 2147483648.0f && f >= -2147483648.0f) ? (int32_t)f : INT32_MIN;
}

/* Util.hpp:64-84 */
uint32_t svo_oracle_compress_material(const float n[3], float shade) {
    const int32_t uScale = (1 << 11) - 1;
    const int32_t vScale = (1 << 11) - 1;
    uint32_t face = 0;
    float dominant = fabsf(n[0]);
    if (fabsf(n[1]) > dominant) { dominant = fabsf(n[1]); face = 1; }
    if (fabsf(n[2]) > dominant) { dominant = fabsf(n[2]); face = 2; }
    uint32_t sign = n[face] < 0.0f;
    float n1 = n[MOD3[face + 1]] / dominant;
    float n2 = n[MOD3[face + 2]] / dominant;
    uint32_t u = (uint32_t)imin(f2i_x86((n1 * 0.5f + 0.5f) * (float)uScale), 0x7FF);
    uint32_t v = (uint32_t)imin(f2i_x86((n2 * 0.5f + 0.5f) * (float)vScale), 0x7FF);
    uint32_t c = (uint32_t)imin(f2i_x86(shade * 127.0f), 0x7F);
    return (sign << 31) | (face << 29) | (u << 18) | (v << 7) | c;
}

/* Util.hpp:86-100 (face 3 is outside the codec; it is mapped to face 2 here
 * and in the device code, where the reference would index out of bounds). */
void svo_oracle_decompress_material(uint32_t word, float n[3], float *shade) {
    uint32_t sign = (word & 0x80000000u) >> 31;
    uint32_t face = (word & 0x60000000u) >> 29;
    uint32_t u = (word & 0x1FFC0000u) >> 18;
    uint32_t v = (word & 0x0003FF80u) >> 7;
    uint32_t c = (word & 0x0000007Fu);
    if (face > 2) face = 2;
    n[face] = sign ? -1.0f : 1.0f;
    n[MOD3[face + 1]] = (float)u * 4.8852e-4f * 2.0f - 1.0f;
    n[MOD3[face + 2]] = (float)v * 4.8852e-4f * 2.0f - 1.0f;
    /* fastNormalization, Util.hpp:60-62: v *= invSqrt(v.dot(v)) */
    float s = svo_oracle_inv_sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] *= s;
    n[1] *= s;
    n[2] *= s;
    *shade = (float)c * 1.0f / 127.0f;
}

/* Main.cpp:81-90 with Vec3::reflect (math/Vec3.hpp:63-71) and Vec3::dot. */
float svo_oracle_shade(uint32_t word, const float dir[3], const float light[3]) {
    float n[3], c;
    svo_oracle_decompress_material(word, n, &c);
    float proj = (n[0] * dir[0] + n[1] * dir[1] + n[2] * dir[2]) * 2.0f;
    float r0 = dir[0] - n[0] * proj;
    float r1 = dir[1] - n[1] * proj;
    float r2 = dir[2] - n[2] * proj;
    float d = smax(light[0] * r0 + light[1] * r1 + light[2] * r2, 0.0f);
    float specular = d * d;
    return c * 0.9f * fabsf(light[0] * n[0] + light[1] * n[1] + light[2] * n[2]) + specular * 0.2f;
}

/* ---------------------------------------------------------------- raymarch */

enum { MAX_SCALE = 23 };

/* VoxelOctree.cpp:207-346, step for step.  The reference keeps a 24-entry
 * stack indexed by `scale` and reads it even when the POP computes a scale
 * past the top (then exits the loop); those reads are skipped here since
 * their values are never used. */
int svo_oracle_raymarch(const uint32_t *oct, uint64_t nwords, const float o[3], const float d[3],
                        float rayScale, uint32_t *word, float *t, uint64_t *leaf, uint64_t *loads) {
    struct { uint64_t offset; float maxT; } stack[MAX_SCALE + 1];
    uint64_t nload = 0;
    (void)nwords;

    float ox = o[0], oy = o[1], oz = o[2];
    float dx = d[0], dy = d[1], dz = d[2];
    if (fabsf(dx) < 1e-4f) dx = 1e-4f;
    if (fabsf(dy) < 1e-4f) dy = 1e-4f;
    if (fabsf(dz) < 1e-4f) dz = 1e-4f;

    float dTx = 1.0f / -fabsf(dx);
    float dTy = 1.0f / -fabsf(dy);
    float dTz = 1.0f / -fabsf(dz);
    float bTx = dTx * ox;
    float bTy = dTy * oy;
    float bTz = dTz * oz;

    uint32_t octantMask = 7;
    if (dx > 0.0f) { octantMask ^= 1; bTx = 3.0f * dTx - bTx; }
    if (dy > 0.0f) { octantMask ^= 2; bTy = 3.0f * dTy - bTy; }
    if (dz > 0.0f) { octantMask ^= 4; bTz = 3.0f * dTz - bTz; }

    float minT = smax(2.0f * dTx - bTx, smax(2.0f * dTy - bTy, 2.0f * dTz - bTz));
    float maxT = smin(dTx - bTx, smin(dTy - bTy, dTz - bTz));
    minT = smax(minT, 0.0f);

    uint32_t current = 0;
    uint64_t parent = 0;
    int idx = 0;
    float posX = 1.0f, posY = 1.0f, posZ = 1.0f;
    int scale = MAX_SCALE - 1;
    float scaleExp2 = 0.5f;

    if (1.5f * dTx - bTx > minT) { idx ^= 1; posX = 1.5f; }
    if (1.5f * dTy - bTy > minT) { idx ^= 2; posY = 1.5f; }
    if (1.5f * dTz - bTz > minT) { idx ^= 4; posZ = 1.5f; }

    /* Not in the reference: a ray with a NaN corner distance on some axis
     * (NaN in o or d, or an infinite o along an infinite d) either never
     * leaves the loop below (NaN on all three axes: nothing advances or
     * pops) or follows std::min's operand order around the NaN.  It ends
     * here as a miss after the root load, as the kernels end it. */
    if (isnan(dTx + bTx) || isnan(dTy + bTy) || isnan(dTz + bTz)) {
        if (loads) *loads += 1;
        return 0;
    }

    int result = 0;
    while (scale < MAX_SCALE) {
        if (current == 0) {
            current = oct[parent];
            nload++;
        }
        float cornerTX = posX * dTx - bTx;
        float cornerTY = posY * dTy - bTy;
        float cornerTZ = posZ * dTz - bTz;
        float maxTC = smin(cornerTX, smin(cornerTY, cornerTZ));

        int childShift = idx ^ (int)octantMask;
        uint32_t childMasks = current << childShift;

        if ((childMasks & 0x8000u) && minT <= maxT) {
            if (maxTC * rayScale >= scaleExp2) {
                *t = maxTC;
                if (loads) *loads += nload;
                return 2;
            }
            float maxTV = smin(maxT, maxTC);
            float half = scaleExp2 * 0.5f;
            float centerTX = half * dTx + cornerTX;
            float centerTY = half * dTy + cornerTY;
            float centerTZ = half * dTz + cornerTZ;

            if (minT <= maxTV) {
                uint64_t childOffset = current >> 18;
                if (current & 0x20000u) {
                    childOffset = (childOffset << 32) | (uint64_t)oct[parent + 1];
                    nload++;
                }
                if (!(childMasks & 0x80u)) {
                    uint64_t li = childOffset + parent +
                        (uint64_t)__builtin_popcount(((childMasks >> (8 + childShift)) << childShift) & 127u);
                    *word = oct[li];
                    nload++;
                    if (leaf) *leaf = li;
                    result = 1;
                    break;
                }
                stack[scale].offset = parent;
                stack[scale].maxT = maxT;

                uint32_t siblingCount = (uint32_t)__builtin_popcount(childMasks & 127u);
                parent += childOffset + siblingCount;
                if (current & 0x10000u) parent += siblingCount;

                idx = 0;
                scale--;
                scaleExp2 = half;
                if (centerTX > minT) { idx ^= 1; posX += scaleExp2; }
                if (centerTY > minT) { idx ^= 2; posY += scaleExp2; }
                if (centerTZ > minT) { idx ^= 4; posZ += scaleExp2; }
                maxT = maxTV;
                current = 0;
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
            if (stepMask & 1) differing |= float_to_bits(posX) ^ float_to_bits(posX + scaleExp2);
            if (stepMask & 2) differing |= float_to_bits(posY) ^ float_to_bits(posY + scaleExp2);
            if (stepMask & 4) differing |= float_to_bits(posZ) ^ float_to_bits(posZ + scaleExp2);
            scale = (int)(float_to_bits((float)(int32_t)differing) >> 23) - 127;
            scaleExp2 = bits_to_float((uint32_t)(scale - MAX_SCALE + 127) << 23);

            if (scale >= 0 && scale <= MAX_SCALE) {
                parent = stack[scale].offset;
                maxT = stack[scale].maxT;
            }
            if (scale >= 0 && scale < 32) {
                uint32_t shX = float_to_bits(posX) >> scale;
                uint32_t shY = float_to_bits(posY) >> scale;
                uint32_t shZ = float_to_bits(posZ) >> scale;
                posX = bits_to_float(shX << scale);
                posY = bits_to_float(shY << scale);
                posZ = bits_to_float(shZ << scale);
                idx = (int)((shX & 1) | ((shY & 1) << 1) | ((shZ & 1) << 2));
            }
            current = 0;
        }
    }

    if (loads) *loads += nload;
    if (result == 0 && scale >= MAX_SCALE) return 0;
    *t = minT;
    return 1;
}

typedef struct {
    const uint32_t *oct;
    uint64_t nwords;
    const float *rays;
    uint64_t nrays;
    float rayScale;
    const float *light;
    uint8_t *hit;
    float *t;
    uint32_t *leaf, *word, *loads;
    float *grey;
    int nthreads, id;
} batch_job;

static void *batch_worker(void *arg) {
    batch_job *j = (batch_job *)arg;
    const uint64_t chunk = 1024;
    for (uint64_t base = (uint64_t)j->id * chunk; base < j->nrays; base += (uint64_t)j->nthreads * chunk) {
        uint64_t end = base + chunk < j->nrays ? base + chunk : j->nrays;
        for (uint64_t i = base; i < end; ++i) {
            const float *r = j->rays + 6 * i;
            uint32_t w = 0;
            float tt = INFINITY;
            uint64_t li = 0xFFFFFFFFu, nl = 0;
            int h = svo_oracle_raymarch(j->oct, j->nwords, r, r + 3, j->rayScale, &w, &tt, &li, &nl);
            if (h != 1) { w = 0; li = 0xFFFFFFFFu; }
            if (h == 0) tt = INFINITY;
            if (j->hit) j->hit[i] = (uint8_t)h;
            if (j->t) j->t[i] = tt;
            if (j->leaf) j->leaf[i] = (uint32_t)li;
            if (j->word) j->word[i] = w;
            if (j->loads) j->loads[i] = (uint32_t)nl;
            if (j->grey) j->grey[i] = (h == 1) ? svo_oracle_shade(w, r + 3, j->light) : 0.0f;
        }
    }
    return NULL;
}

void svo_oracle_raymarch_batch(const uint32_t *oct, uint64_t nwords, const float *rays, uint64_t nrays,
                               float rayScale, const float light[3], uint8_t *hit, float *t,
                               uint32_t *leaf, uint32_t *word, float *grey, uint32_t *loads, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 512) threads = 512;
    batch_job jobs[512];
    pthread_t tids[512];
    for (int k = 0; k < threads; ++k) {
        batch_job j = {oct, nwords, rays, nrays, rayScale, light, hit, t, leaf, word, loads, grey, threads, k};
        jobs[k] = j;
    }
    if (threads == 1) {
        batch_worker(&jobs[0]);
        return;
    }
    for (int k = 0; k < threads; ++k) pthread_create(&tids[k], NULL, batch_worker, &jobs[k]);
    for (int k = 0; k < threads; ++k) pthread_join(tids[k], NULL);
}

/* ------------------------------------------------------------------- build */

/* Util.hpp:102-106 */
static int round_to_pow2(int x) {
    int y;
    for (y = 1; y < x; y *= 2) {}
    return y;
}

/* Util.hpp:108-117 (bit-hack integer log2, exact for powers of two) */
static int find_highest_bit(uint32_t v) {
    static const uint32_t b[] = {0xAAAAAAAAu, 0xCCCCCCCCu, 0xF0F0F0F0u, 0xFF00FF00u, 0xFFFF0000u};
    uint32_t r = (v & b[0]) != 0;
    for (int i = 4; i > 0; i--) r |= ((v & b[i]) != 0) << i;
    return (int)r;
}

/* VoxelData.cpp:65-74 */
static uint64_t cells_in_pyramid(int levels) {
    uint64_t result = 0, size = 1;
    for (int i = 0; i < levels; ++i) { result += size; size *= 8; }
    return result;
}

/* ply_oracle.c: the PlyLoader side of VoxelData's loader mode */
void svo_oracle_mesh_process_block(void *mesh, uint32_t *data, int x, int y, int z, int w, int h, int d);
int svo_oracle_mesh_block_empty(void *mesh, int x, int y, int z);
void svo_oracle_mesh_dims(void *mesh, int side, int dims[3]);
int svo_oracle_mesh_setup(void *mesh, int side, int block, const int dims[3], int threads);

/* State of VoxelData (VoxelData.hpp:38-99): a .voxel payload in memory
 * (`grid`) or a PlyLoader (`loader`). */
typedef struct {
    void *loader;
    const uint32_t *grid;
    int dataW, dataH, dataD;
    int virtW, virtH, virtD;
    int highestVirtualBit, lowLutLevels, topLutLevels;
    uint64_t maxCacheable;
    uint8_t *topLut, *lowLut;
    uint8_t *topTable[32], *lowTable[32];
    uint32_t *buffered;
    int bufX, bufY, bufZ, bufW, bufH, bufD;
} voxel_source;

static inline uint64_t lut_idx(int l, int x, int y, int z) {
    return (uint64_t)x + ((uint64_t)y << l) + ((uint64_t)z << (2 * l));
}

/* VoxelData::init partition search, VoxelData.cpp:211-244. */
static int choose_lower_level(int highestVirtualBit, uint64_t cellCost, uint64_t mem) {
    int largest = -1;
    for (int i = highestVirtualBit; i >= 0; --i) {
        int lowBit = highestVirtualBit - i;
        uint64_t cost = cells_in_pyramid(i + 1) + cells_in_pyramid(lowBit) +
                        ((uint64_t)1 << (uint64_t)(lowBit * 3)) * cellCost;
        if (cost < mem) largest = highestVirtualBit - i;
    }
    return largest;
}

uint64_t svo_oracle_cache_block(int w, int h, int d, uint64_t mem, uint64_t cell_cost) {
    int vw = round_to_pow2(w), vh = round_to_pow2(h), vd = round_to_pow2(d);
    int m = vw > vh ? vw : vh;
    m = m > vd ? m : vd;
    int lower = choose_lower_level(find_highest_bit((uint32_t)m), cell_cost, mem);
    return lower < 0 ? 0 : ((uint64_t)1 << lower);
}

/* VoxelData::upsampleLutLevel, VoxelData.cpp:87-118 (single-threaded; the
 * reference's z-slab split over threads does not change the result). */
static void upsample(uint8_t **table, int l) {
    int size = 2 << l;
    for (int z = 0; z < size; z += 2)
        for (int y = 0; y < size; y += 2)
            for (int x = 0; x < size; x += 2) {
                uint8_t *c = table[l + 1];
                int value = c[lut_idx(l + 1, x, y, z)] | c[lut_idx(l + 1, x + 1, y, z)] |
                            c[lut_idx(l + 1, x, y + 1, z)] | c[lut_idx(l + 1, x + 1, y + 1, z)] |
                            c[lut_idx(l + 1, x, y, z + 1)] | c[lut_idx(l + 1, x + 1, y, z + 1)] |
                            c[lut_idx(l + 1, x, y + 1, z + 1)] | c[lut_idx(l + 1, x + 1, y + 1, z + 1)];
                table[l][lut_idx(l, x >> 1, y >> 1, z >> 1)] = (uint8_t)(value != 0);
            }
}

/* VoxelData::cacheData, VoxelData.cpp:177-209: the loader writes into the
 * buffer as it stands (it is never cleared between blocks); the file branch
 * overwrites the block's w*h*d words. */
static void cache_data(voxel_source *s, int x, int y, int z, int w, int h, int d) {
    if (s->loader) {
        svo_oracle_mesh_process_block(s->loader, s->buffered, x, y, z, w, h, d);
        return;
    }
    for (uint64_t vz = 0; vz < (uint64_t)d; vz++)
        for (uint64_t vy = 0; vy < (uint64_t)h; vy++) {
            const uint32_t *src = s->grid + (uint64_t)x + (uint64_t)s->dataW * ((uint64_t)y + vy +
                                  (uint64_t)s->dataH * ((uint64_t)z + vz));
            memcpy(s->buffered + (vy + vz * (uint64_t)h) * (uint64_t)w, src, (size_t)w * 4);
        }
}

/* VoxelData::buildLowLut, VoxelData.cpp:160-175.  The z range covers
 * 2*floor(bufD/2) slices, so an odd-depth buffer never marks its last slice. */
static void build_low_lut(voxel_source *s) {
    int end = (s->bufD / 2) * 2;
    for (int z = 0; z < end; ++z)
        for (int y = 0; y < s->bufH; ++y)
            for (int x = 0; x < s->bufW; ++x)
                if (s->buffered[(uint64_t)x + (uint64_t)s->bufW * ((uint64_t)y + (uint64_t)s->bufH * z)])
                    s->lowTable[s->lowLutLevels - 1][lut_idx(s->lowLutLevels - 1, x / 2, y / 2, z / 2)] = 1;
    for (int i = s->lowLutLevels - 2; i >= 0; i--) upsample(s->lowTable, i);
}

/* VoxelData::buildTopLut / buildTopLutBlock, VoxelData.cpp:120-158. */
static void build_top_lut(voxel_source *s) {
    if (s->topLutLevels == 0) return;
    int size = (int)s->maxCacheable;
    for (int z = 0; z < s->virtD; z += size)
        for (int y = 0; y < s->virtH; y += size)
            for (int x = 0; x < s->virtW; x += size) {
                int bw = imin(size, s->dataW - x), bh = imin(size, s->dataH - y), bd = imin(size, s->dataD - z);
                if (bw <= 0 || bh <= 0 || bd <= 0) continue;
                int empty = 1;
                if (s->loader) {
                    empty = svo_oracle_mesh_block_empty(s->loader, x, y, z);
                } else {
                    cache_data(s, x, y, z, bw, bh, bd);
                    for (uint64_t i = 0; i < (uint64_t)bw * bh * bd; ++i)
                        if (s->buffered[i]) { empty = 0; break; }
                }
                if (!empty) {
                    int l = s->topLutLevels - 1;
                    s->topTable[l][lut_idx(l, x >> s->lowLutLevels, y >> s->lowLutLevels, z >> s->lowLutLevels)] = 1;
                }
            }
    for (int i = s->topLutLevels - 2; i >= 0; i--) upsample(s->topTable, i);
}

/* VoxelData::prepareDataAccess, VoxelData.cpp:264-291. */
static void prepare_access(voxel_source *s, int x, int y, int z, int size) {
    int width = imin(size, s->dataW - x);
    int height = imin(size, s->dataH - y);
    int depth = imin(size, s->dataD - z);
    if (width <= 0 || height <= 0 || depth <= 0) return;
    if (x >= s->bufX && y >= s->bufY && z >= s->bufZ && x + width <= s->bufX + s->bufW &&
        y + height <= s->bufY + s->bufH && z + depth <= s->bufZ + s->bufD)
        return;
    if ((uint64_t)size <= s->maxCacheable) {
        s->bufX = x; s->bufY = y; s->bufZ = z;
        s->bufW = width; s->bufH = height; s->bufD = depth;
        cache_data(s, x, y, z, width, height, depth);
        build_low_lut(s);
    }
}

static inline uint64_t buf_idx(const voxel_source *s, int x, int y, int z) {
    return (uint64_t)(x - s->bufX) + (uint64_t)s->bufW * ((uint64_t)(y - s->bufY) + (uint64_t)s->bufH * (uint64_t)(z - s->bufZ));
}

/* VoxelData::getVoxel / getVoxelDestructive, VoxelData.hpp:106-121. */
static uint32_t get_voxel(voxel_source *s, int x, int y, int z, int destructive) {
    if (x >= s->dataW || y >= s->dataH || z >= s->dataD) return 0;
    uint64_t i = buf_idx(s, x, y, z);
    uint32_t v = s->buffered[i];
    if (destructive && v) s->buffered[i] = 0;
    return v;
}

/* VoxelData::cubeContainsVoxelsDestructive, VoxelData.hpp:123-138. */
static int cube_contains(voxel_source *s, int x, int y, int z, int size) {
    if (x >= s->dataW || y >= s->dataH || z >= s->dataD) return 0;
    int bit = find_highest_bit((uint32_t)size);
    if (size == 1) return get_voxel(s, x, y, z, 0) != 0;
    if (bit < s->lowLutLevels) {
        int l = s->lowLutLevels - bit;
        uint8_t *v = &s->lowTable[l][lut_idx(l, (x - s->bufX) >> bit, (y - s->bufY) >> bit, (z - s->bufZ) >> bit)];
        uint8_t value = *v;
        if (value) *v = 0;
        return value != 0;
    }
    int l = s->highestVirtualBit - bit;
    return s->topTable[l][lut_idx(l, x >> bit, y >> bit, z >> bit)] != 0;
}

/* ChunkedAllocator (ChunkedAllocator.hpp:32-115): a growable word stream plus
 * deferred insertions (index in pre-insertion coordinates, value). */
typedef struct { uint64_t idx; uint32_t val; } insertion;
typedef struct {
    uint32_t *data;
    uint64_t size, cap;
    insertion *ins;
    uint64_t nins, capins;
    int oom;
} word_stream;

static void ws_push(word_stream *w, uint32_t v) {
    if (w->size == w->cap) {
        uint64_t nc = w->cap ? w->cap * 2 : 4096;
        uint32_t *nd = (uint32_t *)realloc(w->data, nc * 4);
        if (!nd) { w->oom = 1; return; }
        w->data = nd; w->cap = nc;
    }
    w->data[w->size++] = v;
}

static void ws_insert(word_stream *w, uint64_t idx, uint32_t v) {
    if (w->nins == w->capins) {
        uint64_t nc = w->capins ? w->capins * 2 : 256;
        insertion *ni = (insertion *)realloc(w->ins, nc * sizeof(insertion));
        if (!ni) { w->oom = 1; return; }
        w->ins = ni; w->capins = nc;
    }
    w->ins[w->nins].idx = idx;
    w->ins[w->nins].val = v;
    w->nins++;
}

static int ins_cmp(const void *a, const void *b) {
    uint64_t x = ((const insertion *)a)->idx, y = ((const insertion *)b)->idx;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* ChunkedAllocator::finalize, ChunkedAllocator.hpp:76-114: each insertion
 * lands before the pre-insertion word it names. */
static uint32_t *ws_finalize(word_stream *w, uint64_t *out_len) {
    qsort(w->ins, (size_t)w->nins, sizeof(insertion), ins_cmp);
    uint64_t len = w->size + w->nins;
    uint32_t *out = (uint32_t *)malloc((size_t)(len ? len : 1) * 4);
    if (!out) return NULL;
    uint64_t o = 0, in = 0, k = 0;
    while (in < w->size) {
        uint64_t upto = (k < w->nins) ? w->ins[k].idx : w->size;
        if (upto > w->size) upto = w->size;
        if (upto > in) {
            memcpy(out + o, w->data + in, (size_t)(upto - in) * 4);
            o += upto - in;
            in = upto;
        }
        if (k < w->nins && w->ins[k].idx == in) out[o++] = w->ins[k++].val;
    }
    *out_len = o;
    return out;
}

/* VoxelOctree::buildOctree, VoxelOctree.cpp:139-205. */
static uint64_t build_node(voxel_source *s, word_stream *ws, int x, int y, int z, int size, uint64_t desc) {
    prepare_access(s, x, y, z, size);
    int half = size >> 1;
    int px[8] = {x + half, x, x + half, x, x + half, x, x + half, x};
    int py[8] = {y + half, y + half, y, y, y + half, y + half, y, y};
    int pz[8] = {z + half, z + half, z + half, z + half, z, z, z, z};

    uint64_t childOffset = ws->size - desc;
    int count = 0, children[8];
    uint32_t childMask = 0;
    for (int i = 0; i < 8; i++)
        if (cube_contains(s, px[i], py[i], pz[i], half)) {
            childMask |= 128u >> i;
            children[count++] = i;
        }

    int large = 0;
    uint32_t leafMask;
    if (half == 1) {
        leafMask = 0;
        for (int i = 0; i < count; i++) {
            int c = children[count - i - 1];
            ws_push(ws, get_voxel(s, px[c], py[c], pz[c], 1));
        }
    } else {
        leafMask = childMask;
        for (int i = 0; i < count; i++) ws_push(ws, 0);
        uint64_t grand[8];
        uint64_t delta = 0, nins = ws->nins;
        for (int i = 0; i < count; i++) {
            int c = children[count - i - 1];
            grand[i] = delta + build_node(s, ws, px[c], py[c], pz[c], half, desc + childOffset + (uint64_t)i);
            delta += ws->nins - nins;
            nins = ws->nins;
            if (grand[i] > 0x3FFF) large = 1;
        }
        for (int i = 0; i < count; i++) {
            uint64_t ci = desc + childOffset + (uint64_t)i;
            uint64_t off = grand[i];
            if (large) {
                off += (uint64_t)(count - i);
                ws_insert(ws, ci + 1, (uint32_t)off);
                ws->data[ci] |= 0x20000u;
                off >>= 32;
            }
            ws->data[ci] |= (uint32_t)(off << 18);
        }
    }
    ws->data[desc] = (childMask << 8) | leafMask;
    if (large) ws->data[desc] |= 0x10000u;
    return childOffset;
}

/* VoxelData::init + buildTopLut, then VoxelOctree(VoxelData*). */
static int build_from_source(voxel_source *s, int w, int h, int d, uint64_t mem, uint64_t cell_cost, int side_arg,
                             int threads, uint32_t **words, uint64_t *nwords, float center[3]) {
    s->dataW = w; s->dataH = h; s->dataD = d;
    s->virtW = round_to_pow2(w);
    s->virtH = round_to_pow2(h);
    s->virtD = round_to_pow2(d);
    int side = s->virtW > s->virtH ? s->virtW : s->virtH;
    side = side > s->virtD ? side : s->virtD;
    if (side < 2) return -2;
    s->highestVirtualBit = find_highest_bit((uint32_t)side);
    int lower = choose_lower_level(s->highestVirtualBit, cell_cost, mem);
    if (lower < 0) return -1;
    /* lowLutLevels == 0 makes the reference index lowTable[-1]; reject it. */
    if (lower < 1) return -1;
    s->lowLutLevels = lower;
    s->topLutLevels = s->highestVirtualBit - lower + 1;
    s->maxCacheable = (uint64_t)1 << lower;
    if (s->loader) {  /* VoxelData.cpp:53-54 */
        int dims[3] = {w, h, d};
        int rc = svo_oracle_mesh_setup(s->loader, side_arg, (int)s->maxCacheable, dims, threads);
        if (rc) return rc;
    }
    s->topLut = (uint8_t *)calloc((size_t)cells_in_pyramid(s->topLutLevels), 1);
    s->lowLut = (uint8_t *)calloc((size_t)cells_in_pyramid(s->lowLutLevels), 1);
    s->buffered = (uint32_t *)calloc((size_t)1 << (3 * lower), 4);
    if (!s->topLut || !s->lowLut || !s->buffered) {
        free(s->topLut); free(s->lowLut); free(s->buffered);
        return -3;
    }
    /* VoxelData.cpp:76-85 */
    uint64_t off = 0, sz = 1;
    for (int i = 0; i < s->topLutLevels; ++i) { s->topTable[i] = s->topLut + off; off += sz; sz *= 8; }
    off = 0; sz = 1;
    for (int i = 0; i < s->lowLutLevels; ++i) { s->lowTable[i] = s->lowLut + off; off += sz; sz *= 8; }

    build_top_lut(s);

    word_stream ws;
    memset(&ws, 0, sizeof(ws));
    ws_push(&ws, 0);
    build_node(s, &ws, 0, 0, 0, side, 0);
    ws.data[0] |= 1u << 18;
    int rc = 0;
    if (ws.oom) {
        rc = -3;
    } else {
        uint64_t n = 0;
        uint32_t *out = ws_finalize(&ws, &n);
        if (!out) rc = -3;
        *words = out;
        *nwords = n;
        /* VoxelData::getCenter, VoxelData.cpp:297-303 */
        center[0] = (float)w * 0.5f / (float)side;
        center[1] = (float)h * 0.5f / (float)side;
        center[2] = (float)d * 0.5f / (float)side;
    }
    free(ws.data); free(ws.ins);
    free(s->topLut); free(s->lowLut); free(s->buffered);
    return rc;
}

int svo_oracle_build_dense(const uint32_t *grid, int w, int h, int d, uint64_t mem,
                           uint32_t **words, uint64_t *nwords, float center[3]) {
    voxel_source s;
    memset(&s, 0, sizeof(s));
    s.grid = grid;
    return build_from_source(&s, w, h, d, mem, 4, 0, 0, words, nwords, center);
}

/* VoxelData(PlyLoader*, side, mem) (VoxelData.cpp:50-56) + VoxelOctree:
 * cell cost 4 + 1 (blockMemRequirement, PlyLoader.cpp:376-379), dims from
 * suggestedDimensions, sub-block partition for `threads` threads. */
int svo_oracle_build_mesh(void *mesh, int side, int threads, uint64_t mem, uint32_t **words, uint64_t *nwords,
                          float center[3]) {
    voxel_source s;
    memset(&s, 0, sizeof(s));
    s.loader = mesh;
    int dims[3];
    svo_oracle_mesh_dims(mesh, side, dims);
    return build_from_source(&s, dims[0], dims[1], dims[2], mem, 5, side, threads, words, nwords, center);
}

/* --------------------------------------------------------------- .oct I/O */

/* LZ4 block decode into out[pos0, pos0+outLen) where earlier bytes of `out`
 * are valid history (LZ4_decompress_fast_continue on one contiguous
 * destination, VoxelOctree.cpp:70-80).  Format: token (literal length high
 * nibble, match length low nibble, 15 = extended by bytes until one < 255),
 * literals, 16-bit little-endian offset, match of length + 4. */
static int lz4_block_decode(const uint8_t *src, uint64_t srcLen, uint8_t *out, uint64_t pos0, uint64_t outLen) {
    uint64_t ip = 0, op = pos0, end = pos0 + outLen;
    while (op < end) {
        if (ip >= srcLen) return -1;
        uint8_t token = src[ip++];
        uint64_t lit = token >> 4;
        if (lit == 15) {
            uint8_t b;
            do {
                if (ip >= srcLen) return -1;
                b = src[ip++];
                lit += b;
            } while (b == 255);
        }
        if (ip + lit > srcLen || op + lit > end) return -1;
        memcpy(out + op, src + ip, (size_t)lit);
        ip += lit;
        op += lit;
        if (op == end) break;
        if (ip + 2 > srcLen) return -1;
        uint64_t offset = (uint64_t)src[ip] | ((uint64_t)src[ip + 1] << 8);
        ip += 2;
        if (offset == 0 || offset > op) return -1;
        uint64_t ml = token & 15;
        if (ml == 15) {
            uint8_t b;
            do {
                if (ip >= srcLen) return -1;
                b = src[ip++];
                ml += b;
            } while (b == 255);
        }
        ml += 4;
        if (op + ml > end) return -1;
        for (uint64_t k = 0; k < ml; ++k, ++op) out[op] = out[op - offset];
    }
    return 0;
}

int svo_oracle_oct_decode(const uint8_t *bytes, uint64_t len, uint32_t **words, uint64_t *nwords, float center[3]) {
    const uint64_t block = 64ull * 1024 * 1024;
    if (len < 20) return -1;
    memcpy(center, bytes, 12);
    uint64_t n;
    memcpy(&n, bytes + 12, 8);
    if (n > (1ull << 40)) return -2;
    uint8_t *out = (uint8_t *)malloc((size_t)(n ? n * 4 : 4));
    if (!out) return -3;
    uint64_t ip = 20;
    for (uint64_t off = 0; off < n * 4; off += block) {
        uint64_t comp;
        if (ip + 8 > len) { free(out); return -1; }
        memcpy(&comp, bytes + ip, 8);
        ip += 8;
        if (comp > len - ip) { free(out); return -1; }
        uint64_t outLen = n * 4 - off < block ? n * 4 - off : block;
        if (lz4_block_decode(bytes + ip, comp, out, off, outLen) != 0) { free(out); return -4; }
        ip += comp;
    }
    *words = (uint32_t *)out;
    *nwords = n;
    return 0;
}
