/*
 * scene_build.c — CPU-only setup for the benchmark's reference leg.
 *
 * TEST/BENCH INFRASTRUCTURE ONLY.  bench.py --impl reference must run
 * without the GPU library, so this file provides, on host threads:
 *
 *  1. the synthetic scene of sparse-voxel-octrees_gb300/scenes.py (terrain
 *     shell + solid spheres, central-difference normals, hashed shade,
 *     compressMaterial packing), computed with the same float32 operation
 *     order, as an occupancy bitmap and then Morton-ordered voxels;
 *  2. an octree build from Morton-ordered voxels that produces the word
 *     stream of VoxelOctree(VoxelData*) (VoxelOctree.cpp:125-205) for grids
 *     whose dimensions are equal powers of two (no VoxelData corner cases).
 *     It computes subtree word counts bottom-up and places blocks top-down;
 *     tests check it against svo_oracle_build_dense.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "svo_oracle.h"

typedef struct {
    int side, w32;
    uint32_t *bm;
} bitmap;

static inline uint64_t bm_index(const bitmap *b, int xw, int y, int z) {
    return (uint64_t)xw + (uint64_t)b->w32 * ((uint64_t)y + (uint64_t)b->side * (uint64_t)z);
}

static inline int bm_get(const bitmap *b, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= b->side || y >= b->side || z >= b->side) return 0;
    return (b->bm[bm_index(b, x >> 5, y, z)] >> (x & 31)) & 1;
}

/* ---------------------------------------------------------- thread helper */

typedef void (*range_fn)(void *ctx, uint64_t lo, uint64_t hi);
typedef struct {
    range_fn fn;
    void *ctx;
    uint64_t lo, hi;
} range_job;

static void *range_worker(void *a) {
    range_job *j = (range_job *)a;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}

static void parallel_for(uint64_t n, int threads, range_fn fn, void *ctx) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    if ((uint64_t)threads > n) threads = n ? (int)n : 1;
    range_job jobs[256];
    pthread_t tid[256];
    for (int t = 0; t < threads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].lo = n * (uint64_t)t / (uint64_t)threads;
        jobs[t].hi = n * (uint64_t)(t + 1) / (uint64_t)threads;
    }
    for (int t = 1; t < threads; ++t) pthread_create(&tid[t], NULL, range_worker, &jobs[t]);
    range_worker(&jobs[0]);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
}

/* ---------------------------------------------------------- occupancy */

typedef struct {
    bitmap *b;
    const float *heights;
    float thickness;
    const int *box;
    const float *params;
    int n;
} occ_ctx;

/* Each task owns a range of z slices, so bitmap words are written by one thread. */
static void occ_slices(void *c, uint64_t z0, uint64_t z1) {
    occ_ctx *o = (occ_ctx *)c;
    bitmap *b = o->b;
    int side = b->side;
    for (uint64_t zz = z0; zz < z1; ++zz) {
        int z = (int)zz;
        if (o->heights) {
            for (int x = 0; x < side; ++x) {
                float h = o->heights[(uint64_t)z * side + x];
                float lo = h - o->thickness;
                int y0 = (int)floorf(lo) - 1, y1 = (int)ceilf(h) + 1;
                if (y0 < 0) y0 = 0;
                if (y1 > side - 1) y1 = side - 1;
                for (int y = y0; y <= y1; ++y) {
                    float yc = (float)y + 0.5f;
                    if (yc <= h && yc > lo) b->bm[bm_index(b, x >> 5, y, z)] |= 1u << (x & 31);
                }
            }
        }
        for (int s = 0; s < o->n; ++s) {
            const int *bx = o->box + 6 * s;
            if (z < bx[4] || z >= bx[5]) continue;
            float cx = o->params[4 * s], cy = o->params[4 * s + 1], cz = o->params[4 * s + 2], r = o->params[4 * s + 3];
            float rr = r * r;
            float dz = ((float)z + 0.5f) - cz;
            float dzz = dz * dz;
            for (int y = bx[2]; y < bx[3]; ++y) {
                float dy = ((float)y + 0.5f) - cy;
                float dyy = dy * dy;
                for (int x = bx[0]; x < bx[1]; ++x) {
                    float dx = ((float)x + 0.5f) - cx;
                    if ((dx * dx + dyy) + dzz <= rr) b->bm[bm_index(b, x >> 5, y, z)] |= 1u << (x & 31);
                }
            }
        }
    }
}

/* ---------------------------------------------------------- payload */

static inline uint32_t hash32(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t h = (x * 0x8DA6B343u) ^ (y * 0xD8163841u) ^ (z * 0xCB1AB31Fu);
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

static inline uint32_t voxel_word(const bitmap *b, int x, int y, int z) {
    float n[3];
    n[0] = (float)(bm_get(b, x - 1, y, z) - bm_get(b, x + 1, y, z));
    n[1] = (float)(bm_get(b, x, y - 1, z) - bm_get(b, x, y + 1, z));
    n[2] = (float)(bm_get(b, x, y, z - 1) - bm_get(b, x, y, z + 1));
    if (n[0] == 0.0f && n[1] == 0.0f && n[2] == 0.0f) n[1] = 1.0f;
    uint32_t h = hash32((uint32_t)x, (uint32_t)y, (uint32_t)z);
    float r = (float)(h & 255u), g = (float)((h >> 8) & 255u), bl = (float)((h >> 16) & 255u);
    float shade = (r * 0.2126f + g * 0.7152f + bl * 0.0722f) * (1.0f / 256.0f);
    uint32_t w = svo_oracle_compress_material(n, shade);
    return w ? w : 1u;
}

static inline uint32_t compact3(uint64_t x) {
    x &= 0x1249249249249249ull;
    x = (x ^ (x >> 2)) & 0x10c30c30c30c30c3ull;
    x = (x ^ (x >> 4)) & 0x100f00f00f00f00full;
    x = (x ^ (x >> 8)) & 0x1f0000ff0000ffull;
    x = (x ^ (x >> 16)) & 0x1f00000000ffffull;
    x = (x ^ (x >> 32)) & 0x1fffffull;
    return (uint32_t)x;
}

typedef struct {
    const bitmap *b;
    int lb; /* log2 brick edge */
    uint64_t *counts;
    const uint64_t *offsets;
    uint64_t *keys;
    uint32_t *payload;
} voxel_ctx;

static void count_bricks(void *c, uint64_t lo, uint64_t hi) {
    voxel_ctx *v = (voxel_ctx *)c;
    int E = 1 << v->lb;
    for (uint64_t br = lo; br < hi; ++br) {
        int x0 = (int)compact3(br) << v->lb, y0 = (int)compact3(br >> 1) << v->lb, z0 = (int)compact3(br >> 2) << v->lb;
        uint64_t n = 0;
        for (int z = z0; z < z0 + E; ++z)
            for (int y = y0; y < y0 + E; ++y)
                for (int x = x0; x < x0 + E; ++x) n += (uint64_t)bm_get(v->b, x, y, z);
        v->counts[br] = n;
    }
}

static void emit_bricks(void *c, uint64_t lo, uint64_t hi) {
    voxel_ctx *v = (voxel_ctx *)c;
    uint64_t cells = 1ull << (3 * v->lb);
    for (uint64_t br = lo; br < hi; ++br) {
        if (!v->counts[br]) continue;
        int x0 = (int)compact3(br) << v->lb, y0 = (int)compact3(br >> 1) << v->lb, z0 = (int)compact3(br >> 2) << v->lb;
        uint64_t o = v->offsets[br];
        for (uint64_t m = 0; m < cells; ++m) {
            int x = x0 + (int)compact3(m), y = y0 + (int)compact3(m >> 1), z = z0 + (int)compact3(m >> 2);
            if (!bm_get(v->b, x, y, z)) continue;
            v->keys[o] = (br << (3 * v->lb)) | m;
            v->payload[o] = voxel_word(v->b, x, y, z);
            ++o;
        }
    }
}

int svo_oracle_scene_voxels(int side, const float *heights, float thickness, const int *box, const float *params,
                            int n_spheres, int threads, uint64_t **keys, uint32_t **payload, uint64_t *n_voxels) {
    if (side < 2 || (side & (side - 1))) return -1;
    bitmap b;
    b.side = side;
    b.w32 = side >= 32 ? side / 32 : 1;
    b.bm = (uint32_t *)calloc((size_t)b.w32 * side * side, 4);
    if (!b.bm) return -3;
    occ_ctx oc = {&b, heights, thickness, box, params, n_spheres};
    parallel_for((uint64_t)side, threads, occ_slices, &oc);

    int D = 0;
    while ((1 << D) < side) ++D;
    int lb = D < 4 ? D : 4;
    uint64_t nb = 1ull << (3 * (D - lb));
    uint64_t *counts = (uint64_t *)malloc(nb * 8), *offs = (uint64_t *)malloc(nb * 8);
    if (!counts || !offs) { free(b.bm); free(counts); free(offs); return -3; }
    voxel_ctx vc = {&b, lb, counts, offs, NULL, NULL};
    parallel_for(nb, threads, count_bricks, &vc);
    uint64_t total = 0;
    for (uint64_t i = 0; i < nb; ++i) { offs[i] = total; total += counts[i]; }
    vc.keys = (uint64_t *)malloc((total ? total : 1) * 8);
    vc.payload = (uint32_t *)malloc((total ? total : 1) * 4);
    if (!vc.keys || !vc.payload) { free(b.bm); free(counts); free(offs); free(vc.keys); free(vc.payload); return -3; }
    parallel_for(nb, threads, emit_bricks, &vc);
    free(b.bm); free(counts); free(offs);
    *keys = vc.keys;
    *payload = vc.payload;
    *n_voxels = total;
    return 0;
}

/* ---------------------------------------------------------- sorted build */

typedef struct {
    uint64_t n;
    uint64_t *key;
    uint64_t *start; /* first child index in the level below */
    uint8_t *mask, *count, *large;
    uint64_t *S, *B;
} level;

/* Octree words of VoxelOctree(VoxelData*) for `n` voxels with ascending
 * Morton keys (x in bit 0, y in bit 1, z in bit 2 of each level) in a cube of
 * edge 2^log_side.  Child slot order (descending octant i, i = 7 - m) is
 * ascending Morton order, so sibling runs are contiguous.  Subtree word
 * counts S and far decisions (VoxelOctree.cpp:172-183) go bottom-up; block
 * positions go top-down. */
int svo_oracle_build_sorted(const uint64_t *keys, const uint32_t *payload, uint64_t n, int log_side,
                            uint32_t **words_out, uint64_t *n_words) {
    int D = log_side;
    if (D < 1 || D > 21) return -1;
    level *lv = (level *)calloc((size_t)D + 1, sizeof(level));
    if (!lv) return -3;
    const uint64_t *ckey = keys;
    uint64_t nc = n;
    int rc = 0;
    for (int e = 1; e <= D; ++e) {
        level *L = &lv[e];
        uint64_t np = 0;
        for (uint64_t i = 0; i < nc; ++i)
            if (i == 0 || (ckey[i] >> 3) != (ckey[i - 1] >> 3)) ++np;
        if (e == D && np == 0) np = 1;
        L->n = np;
        L->key = (uint64_t *)calloc(np, 8);
        L->start = (uint64_t *)calloc(np, 8);
        L->mask = (uint8_t *)calloc(np, 1);
        L->count = (uint8_t *)calloc(np, 1);
        L->large = (uint8_t *)calloc(np, 1);
        L->S = (uint64_t *)calloc(np, 8);
        L->B = (uint64_t *)calloc(np, 8);
        if (!L->key || !L->start || !L->mask || !L->count || !L->large || !L->S || !L->B) { rc = -3; goto done; }
        uint64_t p = (uint64_t)-1;
        for (uint64_t i = 0; i < nc; ++i) {
            if (i == 0 || (ckey[i] >> 3) != (ckey[i - 1] >> 3)) {
                ++p;
                L->key[p] = ckey[i] >> 3;
                L->start[p] = i;
            }
            L->mask[p] |= (uint8_t)(1u << (ckey[i] & 7));
            L->count[p]++;
        }
        ckey = L->key;
        nc = np;
    }
    for (int e = 1; e <= D; ++e) {
        level *L = &lv[e];
        for (uint64_t p = 0; p < L->n; ++p) {
            uint32_t k = L->count[p];
            if (e == 1) { L->S[p] = k; continue; }
            uint64_t run = 0;
            int far = 0;
            for (uint32_t i = 0; i < k; ++i) {
                if ((uint64_t)(k - i) + run > 0x3FFF) far = 1;
                run += lv[e - 1].S[L->start[p] + i];
            }
            L->large[p] = (uint8_t)far;
            L->S[p] = (uint64_t)k * (far ? 2 : 1) + run;
        }
    }
    uint64_t W = 1 + lv[D].S[0];
    uint32_t *words = (uint32_t *)malloc(W * 4);
    if (!words) { rc = -3; goto done; }
    {
        uint32_t m = lv[D].mask[0];
        words[0] = (m << 8) | (D == 1 ? 0u : m) | (lv[D].large[0] ? 0x10000u : 0u) | (1u << 18);
        lv[D].B[0] = 1;
    }
    for (int e = D; e >= 2; --e) {
        level *P = &lv[e], *C = &lv[e - 1];
        int child_bottom = (e - 1 == 1);
        for (uint64_t p = 0; p < P->n; ++p) {
            uint32_t k = P->count[p];
            int far = P->large[p];
            uint64_t stride = far ? 2 : 1, run = 0, B = P->B[p];
            for (uint32_t i = 0; i < k; ++i) {
                uint64_t c = P->start[p] + i;
                uint64_t pos = B + (uint64_t)i * stride, blk = B + (uint64_t)k * stride + run;
                run += C->S[c];
                C->B[c] = blk;
                uint64_t off = blk - pos;
                uint32_t cm = C->mask[c];
                uint32_t w = (cm << 8) | (child_bottom ? 0u : cm) | (C->large[c] ? 0x10000u : 0u);
                if (far) {
                    w |= 0x20000u | (uint32_t)((off >> 32) << 18);
                    words[pos + 1] = (uint32_t)off;
                } else {
                    w |= (uint32_t)(off << 18);
                }
                words[pos] = w;
            }
        }
    }
    for (uint64_t p = 0; p < lv[1].n; ++p)
        for (uint32_t i = 0; i < lv[1].count[p]; ++i) words[lv[1].B[p] + i] = payload[lv[1].start[p] + i];
    *words_out = words;
    *n_words = W;
done:
    for (int e = 1; e <= D; ++e) {
        free(lv[e].key); free(lv[e].start); free(lv[e].mask); free(lv[e].count);
        free(lv[e].large); free(lv[e].S); free(lv[e].B);
    }
    free(lv);
    return rc;
}
