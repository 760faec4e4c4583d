/*
 * ply_oracle.c — CPU restatement of the reference's mesh-to-octree path:
 * PlyLoader (PlyLoader.cpp) feeding VoxelData(PlyLoader*, side, mem)
 * (VoxelData.cpp:50-56) and VoxelOctree(VoxelData*) (VoxelOctree.cpp:125-205).
 *
 * TEST INFRASTRUCTURE ONLY (see svo_oracle.h).  Input is the parsed mesh
 * (float positions, optional normals, colours, polygon faces); the PLY
 * parsing itself is host I/O.  Every step keeps the reference's float
 * operation order, compiled without FP contraction.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "svo_oracle.h"

typedef struct { float x, y, z; } v3;

static inline v3 sub3(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 add3(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline v3 mul3(v3 a, float s) { v3 r = {a.x * s, a.y * s, a.z * s}; return r; }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross3(v3 a, v3 b) {  /* math/Vec3.hpp:40-42 */
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static inline float len3(v3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline v3 normalize3(v3 a) {  /* Vec3::normalize, math/Vec3.hpp:57-61 */
    float inv = 1.0f / sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    v3 r = {a.x * inv, a.y * inv, a.z * inv};
    return r;
}
static inline float fmin_std(float a, float b) { return (b < a) ? b : a; }
static inline float fmax_std(float a, float b) { return (a < b) ? b : a; }
static inline int imin_(int a, int b) { return (b < a) ? b : a; }
static inline int imax_(int a, int b) { return (a < b) ? b : a; }

typedef struct {
    v3 p[3], n[3], c[3];
    v3 lower, upper;
} tri;

/* ---------------------------------------------------------------- SAT */

/* Triangle/box overlap by the separating-axis theorem (Akenine-Moller,
 * "Fast 3D triangle-box overlap testing"), as in third-party/tribox3.c:
 * the 9 edge-axis tests first, then the box axes, then the triangle plane. */
static int plane_box(const float n[3], const float v[3], const float h[3]) {
    float vmin[3], vmax[3];
    for (int q = 0; q < 3; q++) {
        if (n[q] > 0.0f) {
            vmin[q] = -h[q] - v[q];
            vmax[q] = h[q] - v[q];
        } else {
            vmin[q] = h[q] - v[q];
            vmax[q] = -h[q] - v[q];
        }
    }
    if (n[0] * vmin[0] + n[1] * vmin[1] + n[2] * vmin[2] > 0.0f) return 0;
    if (n[0] * vmax[0] + n[1] * vmax[1] + n[2] * vmax[2] >= 0.0f) return 1;
    return 0;
}

/* One edge-axis test: projections pa, pb of two vertices on the axis and the
 * box radius fa*h[i] + fb*h[j]; the first argument order decides the min/max
 * tie-break exactly as the published code does. */
static inline int axis_sep(float pa, float pb, int a_first_if_less, float rad) {
    float mn, mx;
    if (a_first_if_less) {
        if (pa < pb) { mn = pa; mx = pb; } else { mn = pb; mx = pa; }
    } else {
        if (pb < pa) { mn = pb; mx = pa; } else { mn = pa; mx = pb; }
    }
    return mn > rad || mx < -rad;
}

int svo_oracle_tri_box_overlap(const float c[3], const float h[3], const float tv[9]) {
    float v0[3] = {tv[0] - c[0], tv[1] - c[1], tv[2] - c[2]};
    float v1[3] = {tv[3] - c[0], tv[4] - c[1], tv[5] - c[2]};
    float v2[3] = {tv[6] - c[0], tv[7] - c[1], tv[8] - c[2]};
    float e0[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    float e1[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
    float e2[3] = {v0[0] - v2[0], v0[1] - v2[1], v0[2] - v2[2]};
    float fex, fey, fez, a, b;

    fex = fabsf(e0[0]); fey = fabsf(e0[1]); fez = fabsf(e0[2]);
    a = e0[2]; b = e0[1];  /* x axis, vertices 0 and 2 */
    if (axis_sep(a * v0[1] - b * v0[2], a * v2[1] - b * v2[2], 1, fez * h[1] + fey * h[2])) return 0;
    a = e0[2]; b = e0[0];  /* y axis, vertices 0 and 2 */
    if (axis_sep(-a * v0[0] + b * v0[2], -a * v2[0] + b * v2[2], 1, fez * h[0] + fex * h[2])) return 0;
    a = e0[1]; b = e0[0];  /* z axis, vertices 1 and 2 (min picked as p2 when p2 < p1) */
    if (axis_sep(a * v1[0] - b * v1[1], a * v2[0] - b * v2[1], 0, fey * h[0] + fex * h[1])) return 0;

    fex = fabsf(e1[0]); fey = fabsf(e1[1]); fez = fabsf(e1[2]);
    a = e1[2]; b = e1[1];
    if (axis_sep(a * v0[1] - b * v0[2], a * v2[1] - b * v2[2], 1, fez * h[1] + fey * h[2])) return 0;
    a = e1[2]; b = e1[0];
    if (axis_sep(-a * v0[0] + b * v0[2], -a * v2[0] + b * v2[2], 1, fez * h[0] + fex * h[2])) return 0;
    a = e1[1]; b = e1[0];  /* z axis, vertices 0 and 1 */
    if (axis_sep(a * v0[0] - b * v0[1], a * v1[0] - b * v1[1], 1, fey * h[0] + fex * h[1])) return 0;

    fex = fabsf(e2[0]); fey = fabsf(e2[1]); fez = fabsf(e2[2]);
    a = e2[2]; b = e2[1];  /* x axis, vertices 0 and 1 */
    if (axis_sep(a * v0[1] - b * v0[2], a * v1[1] - b * v1[2], 1, fez * h[1] + fey * h[2])) return 0;
    a = e2[2]; b = e2[0];  /* y axis, vertices 0 and 1 */
    if (axis_sep(-a * v0[0] + b * v0[2], -a * v1[0] + b * v1[2], 1, fez * h[0] + fex * h[2])) return 0;
    a = e2[1]; b = e2[0];
    if (axis_sep(a * v1[0] - b * v1[1], a * v2[0] - b * v2[1], 0, fey * h[0] + fex * h[1])) return 0;

    for (int k = 0; k < 3; ++k) {  /* box axes against the triangle's bounds */
        float mn = v0[k], mx = v0[k];
        if (v1[k] < mn) mn = v1[k];
        if (v1[k] > mx) mx = v1[k];
        if (v2[k] < mn) mn = v2[k];
        if (v2[k] > mx) mx = v2[k];
        if (mn > h[k] || mx < -h[k]) return 0;
    }
    float n[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
    return plane_box(n, v0, h);
}

/* ---------------------------------------------------------------- mesh */

typedef struct {
    tri *tris;
    int ntris;
    v3 lower, upper;
    /* block processing (PlyLoader.hpp:69-78) */
    int sideLength;  /* PlyLoader::_sideLength = side - 2 */
    int blockW, blockH, blockD, subW, subH, subD, partW, partH, partD, nparts;
    int gridW, gridH, gridD;
    uint32_t *offsets;  /* gridW*gridH*gridD + 1 */
    uint32_t *lists;
    uint8_t *counts;
    int bufX, bufY, bufZ, bufW, bufH, bufD;
} mesh;

/* PlyLoader::pointToGrid, PlyLoader.cpp:226-231 */
static inline void point_to_grid(const mesh *m, v3 p, int *x, int *y, int *z) {
    float s = (float)(m->sideLength - 2);
    *x = (int)(p.x * s + 1.0f);
    *y = (int)(p.y * s + 1.0f);
    *z = (int)(p.z * s + 1.0f);
}

/* PlyLoader::iterateOverlappingBlocks, PlyLoader.cpp:233-270.  mode 0 counts,
 * mode 1 fills; returns -1 if a cell index falls outside the grid. */
static int overlap_blocks(mesh *m, const tri *t, uint32_t ti, int mode) {
    int lx, ly, lz, ux, uy, uz;
    point_to_grid(m, t->lower, &lx, &ly, &lz);
    point_to_grid(m, t->upper, &ux, &uy, &uz);
    int lgx = lx / m->subW, lgy = ly / m->subH, lgz = lz / m->subD;
    int ugx = (ux + 1) / m->subW, ugy = (uy + 1) / m->subH, ugz = (uz + 1) / m->subD;
    int maxSide = imax_(ugx - lgx, imax_(ugy - lgy, ugz - lgz));
    const uint64_t ncell = (uint64_t)m->gridW * m->gridH * m->gridD;
#define BODY(idx)                                                  \
    do {                                                           \
        uint64_t _i = (idx);                                       \
        if (_i >= ncell) return -1;                                \
        if (mode == 0) m->offsets[1 + _i]++;                       \
        else m->lists[m->offsets[_i]++] = ti;                      \
    } while (0)
    if (maxSide > 0) {
        float hx = (float)m->subW / (float)(m->sideLength - 2);
        float hy = (float)m->subH / (float)(m->sideLength - 2);
        float hz = (float)m->subD / (float)(m->sideLength - 2);
        float tv[9] = {t->p[0].x, t->p[0].y, t->p[0].z, t->p[1].x, t->p[1].y, t->p[1].z, t->p[2].x, t->p[2].y, t->p[2].z};
        float half[3] = {0.5f * hx, 0.5f * hy, 0.5f * hz};
        float c[3];
        c[2] = ((float)lgz + 0.5f) * hz;
        for (int z = lgz; z <= ugz; ++z, c[2] += hz) {
            c[1] = ((float)lgy + 0.5f) * hy;
            for (int y = lgy; y <= ugy; ++y, c[1] += hy) {
                c[0] = ((float)lgx + 0.5f) * hx;
                for (int x = lgx; x <= ugx; ++x, c[0] += hx)
                    if (svo_oracle_tri_box_overlap(c, half, tv))
                        BODY((uint64_t)x + (uint64_t)m->gridW * ((uint64_t)y + (uint64_t)m->gridH * z));
            }
        }
    } else {
        BODY((uint64_t)lgx + (uint64_t)m->gridW * ((uint64_t)lgy + (uint64_t)m->gridH * lgz));
    }
#undef BODY
    return 0;
}

/* findBestBlockPartition, PlyLoader.cpp:381-405 */
static void best_partition(int *w, int *h, int *d, int threads) {
    int used = 1;
    while (used < threads) {
        int *mx = (*w > *h && *w > *d) ? w : (*h > *d ? h : d);
        int big = *w > *h ? *w : *h; big = big > *d ? big : *d;
        int small = *w < *h ? *w : *h; small = small < *d ? small : *d;
        int *md = (*w != small && *w != big) ? w : ((*h != small && *h != big) ? h : d);
        int *mn = (*w < *h && *w < *d) ? w : (*h < *d ? h : d);
        if ((*mx % 2) == 0) *mx /= 2;
        else if ((*md % 2) == 0) *md /= 2;
        else if ((*mn % 2) == 0) *mn /= 2;
        else break;
        used *= 2;
    }
}

/* PlyLoader::setupBlockProcessing + buildBlockLists, PlyLoader.cpp:407-437,
 * 272-294, for a bw x bh x bd block over a vw x vh x vd volume */
static int setup_blocks3(mesh *m, int side, int bw, int bh, int bd, int vw, int vh, int vd, int threads) {
    m->sideLength = side - 2;
    m->blockW = m->subW = bw;
    m->blockH = m->subH = bh;
    m->blockD = m->subD = bd;
    best_partition(&m->subW, &m->subH, &m->subD, threads);
    m->partW = m->blockW / m->subW;
    m->partH = m->blockH / m->subH;
    m->partD = m->blockD / m->subD;
    m->nparts = m->partW * m->partH * m->partD;
    m->gridW = m->partW * (vw + m->blockW - 1) / m->blockW;
    m->gridH = m->partH * (vh + m->blockH - 1) / m->blockH;
    m->gridD = m->partD * (vd + m->blockD - 1) / m->blockD;
    uint64_t ncell = (uint64_t)m->gridW * m->gridH * m->gridD;
    m->offsets = (uint32_t *)calloc(ncell + 1, 4);
    if (!m->offsets) return -3;
    for (int i = 0; i < m->ntris; ++i)
        if (overlap_blocks(m, &m->tris[i], (uint32_t)i, 0)) return -5;
    for (uint64_t i = 1; i <= ncell; ++i) m->offsets[i] += m->offsets[i - 1];
    m->lists = (uint32_t *)malloc((size_t)(m->offsets[ncell] ? m->offsets[ncell] : 1) * 4);
    if (!m->lists) return -3;
    for (int i = 0; i < m->ntris; ++i)
        if (overlap_blocks(m, &m->tris[i], (uint32_t)i, 1)) return -5;
    for (uint64_t i = ncell; i >= 1; --i) m->offsets[i] = m->offsets[i - 1];
    m->offsets[0] = 0;
    return 0;
}

/* VoxelData's cache blocks are cubes */
static int setup_blocks(mesh *m, int side, int block, int vw, int vh, int vd, int threads) {
    return setup_blocks3(m, side, block, block, block, vw, vh, vd, threads);
}

/* PlyLoader::isBlockEmpty, PlyLoader.cpp:476-493 */
static int block_empty(const mesh *m, int x, int y, int z) {
    for (int pz = 0; pz < m->partD; ++pz)
        for (int py = 0; py < m->partH; ++py)
            for (int px = 0; px < m->partW; ++px) {
                uint64_t b = (uint64_t)(x / m->subW + px) +
                             (uint64_t)m->gridW * ((uint64_t)(y / m->subH + py) + (uint64_t)m->gridH * (z / m->subD + pz));
                if (m->offsets[b] != m->offsets[b + 1]) return 0;
            }
    return 1;
}

/* Triangle::barycentric, PlyLoader.cpp:55-64 */
static int barycentric(const tri *t, v3 p, float *l1, float *l2) {
    v3 f1 = sub3(t->p[0], p), f2 = sub3(t->p[1], p), f3 = sub3(t->p[2], p);
    float area = len3(cross3(sub3(t->p[0], t->p[1]), sub3(t->p[0], t->p[2])));
    *l1 = len3(cross3(f2, f3)) / area;
    *l2 = len3(cross3(f3, f1)) / area;
    return *l1 >= 0.0f && *l2 >= 0.0f && *l1 + *l2 <= 1.0f;
}

/* PlyLoader::writeTriangleCell, PlyLoader.cpp:296-336 */
static void write_cell(mesh *m, uint32_t *data, int x, int y, int z, float cx, float cy, float cz, const tri *t) {
    uint64_t idx = (uint64_t)(x - m->bufX) +
                   (uint64_t)m->bufW * ((uint64_t)(y - m->bufY) + (uint64_t)m->bufH * (uint64_t)(z - m->bufZ));
    float l1, l2, l3;
    v3 p = {cx, cy, cz};
    if (!barycentric(t, p, &l1, &l2)) {
        l1 = fmin_std(fmax_std(l1, 0.0f), 1.0f);
        l2 = fmin_std(fmax_std(l2, 0.0f), 1.0f);
        float tau = l1 + l2;
        if (tau > 1.0f) {
            l1 /= tau;
            l2 /= tau;
        }
    }
    l3 = 1.0f - l1 - l2;
    v3 normal = normalize3(add3(add3(mul3(t->n[0], l1), mul3(t->n[1], l2)), mul3(t->n[2], l3)));
    v3 color = add3(add3(mul3(t->c[0], l1), mul3(t->c[1], l2)), mul3(t->c[2], l3));
    v3 lum = {0.2126f, 0.7152f, 0.0722f};
    float shade = dot3(color, lum) * (1.0f / 256.0f);
    if (data[idx] == 0) {
        m->counts[idx] = 1;
        float nn[3] = {normal.x, normal.y, normal.z};
        data[idx] = svo_oracle_compress_material(nn, shade);
    } else {
        float currentRatio = (float)m->counts[idx] / ((float)m->counts[idx] + 1.0f);
        float newRatio = 1.0f - currentRatio;
        float cn[3], cs;
        svo_oracle_decompress_material(data[idx], cn, &cs);
        v3 cur = {cn[0], cn[1], cn[2]};
        v3 nn = add3(mul3(cur, currentRatio), mul3(normal, newRatio));
        float ns = cs * currentRatio + shade * newRatio;
        if (dot3(nn, nn) < 1e-3f) nn = cur;
        float na[3] = {nn.x, nn.y, nn.z};
        data[idx] = svo_oracle_compress_material(na, ns);
        int c = (int)m->counts[idx] + 1;
        m->counts[idx] = (uint8_t)(c < 255 ? c : 255);
    }
}

/* PlyLoader::triangleToVolume, PlyLoader.cpp:338-374 */
static void tri_to_volume(mesh *m, uint32_t *data, const tri *t, int offX, int offY, int offZ) {
    int lx, ly, lz, ux, uy, uz;
    point_to_grid(m, t->lower, &lx, &ly, &lz);
    point_to_grid(m, t->upper, &ux, &uy, &uz);
    lx = imax_(lx, m->bufX + offX);
    ly = imax_(ly, m->bufY + offY);
    lz = imax_(lz, m->bufZ + offZ);
    ux = imin_(ux, m->bufX + imin_(offX + m->subW, m->bufW) - 1);
    uy = imin_(uy, m->bufY + imin_(offY + m->subH, m->bufH) - 1);
    uz = imin_(uz, m->bufZ + imin_(offZ + m->subD, m->bufD) - 1);
    if (lx > ux || ly > uy || lz > uz) return;
    float hx = 1.0f / (float)(m->sideLength - 2);
    float tv[9] = {t->p[0].x, t->p[0].y, t->p[0].z, t->p[1].x, t->p[1].y, t->p[1].z, t->p[2].x, t->p[2].y, t->p[2].z};
    float half[3] = {0.5f * hx, 0.5f * hx, 0.5f * hx};
    float c[3];
    c[2] = ((float)lz - 0.5f) * hx;
    for (int z = lz; z <= uz; z++, c[2] += hx) {
        c[1] = ((float)ly - 0.5f) * hx;
        for (int y = ly; y <= uy; y++, c[1] += hx) {
            c[0] = ((float)lx - 0.5f) * hx;
            for (int x = lx; x <= ux; x++, c[0] += hx)
                if (svo_oracle_tri_box_overlap(c, half, tv)) write_cell(m, data, x, y, z, c[0], c[1], c[2], t);
        }
    }
}

/* PlyLoader::processBlock, PlyLoader.cpp:439-458 (partitions run one after
 * another here; each writes only its own sub-block, so the order is free). */
void svo_oracle_mesh_process_block(void *mp, uint32_t *data, int x, int y, int z, int w, int h, int d) {
    mesh *m = (mesh *)mp;
    m->bufX = x; m->bufY = y; m->bufZ = z;
    m->bufW = w; m->bufH = h; m->bufD = d;
    for (int i = 0; i < m->nparts; ++i) {
        int px = i % m->partW, py = (i / m->partW) % m->partH, pz = i / (m->partW * m->partH);
        uint64_t b = (uint64_t)(x / m->subW + px) +
                     (uint64_t)m->gridW * ((uint64_t)(y / m->subH + py) + (uint64_t)m->gridH * (z / m->subD + pz));
        for (uint32_t k = m->offsets[b]; k < m->offsets[b + 1]; ++k)
            tri_to_volume(m, data, &m->tris[m->lists[k]], px * m->subW, py * m->subH, pz * m->subD);
    }
}

int svo_oracle_mesh_block_empty(void *mp, int x, int y, int z) { return block_empty((mesh *)mp, x, y, z); }

/* PlyLoader(path) after parsing: vertex bounds (:160-163), rescale
 * (:167-181), fan triangulation and flat normals when the file has none
 * (:183-224), Triangle bounds (:40-53).  faces: for each face its vertex
 * count followed by its indices. */
void *svo_oracle_mesh_create(const float *pos, const float *nrm, const float *col, int n_verts, const int *faces,
                             int n_faces) {
    mesh *m = (mesh *)calloc(1, sizeof(mesh));
    if (!m) return NULL;
    v3 lower = {1e30f, 1e30f, 1e30f}, upper = {-1e30f, -1e30f, -1e30f};
    v3 *p = (v3 *)malloc((size_t)(n_verts ? n_verts : 1) * sizeof(v3));
    for (int i = 0; i < n_verts; ++i) {
        p[i].x = pos[3 * i]; p[i].y = pos[3 * i + 1]; p[i].z = pos[3 * i + 2];
        lower.x = fmin_std(lower.x, p[i].x); lower.y = fmin_std(lower.y, p[i].y); lower.z = fmin_std(lower.z, p[i].z);
        upper.x = fmax_std(upper.x, p[i].x); upper.y = fmax_std(upper.y, p[i].y); upper.z = fmax_std(upper.z, p[i].z);
    }
    v3 diff = sub3(upper, lower);
    int largest = 2;
    if (diff.x > diff.y && diff.x > diff.z) largest = 0;
    else if (diff.y > diff.z) largest = 1;
    float factor = 1.0f / (largest == 0 ? diff.x : (largest == 1 ? diff.y : diff.z));
    for (int i = 0; i < n_verts; ++i) p[i] = mul3(sub3(p[i], lower), factor);
    m->upper = mul3(upper, factor);
    m->lower = mul3(lower, factor);
    int cap = 0;
    for (int f = 0, o = 0; f < n_faces; ++f) {
        int c = faces[o];
        if (c > 2) cap += c - 2;
        o += 1 + c;
    }
    m->tris = (tri *)malloc((size_t)(cap ? cap : 1) * sizeof(tri));
    for (int f = 0, o = 0; f < n_faces; ++f) {
        int c = faces[o];
        const int *idx = faces + o + 1;
        o += 1 + c;
        if (c < 3) continue;  /* no triangles (the reference reads elems[1] even so) */
        int a = idx[0], b = idx[1];
        for (int k = 2; k < c; ++k) {
            int e = idx[k];
            tri *t = &m->tris[m->ntris++];
            int vi[3] = {a, b, e};
            for (int j = 0; j < 3; ++j) {
                t->p[j] = p[vi[j]];
                if (nrm) { t->n[j].x = nrm[3 * vi[j]]; t->n[j].y = nrm[3 * vi[j] + 1]; t->n[j].z = nrm[3 * vi[j] + 2]; }
                if (col) { t->c[j].x = col[3 * vi[j]]; t->c[j].y = col[3 * vi[j] + 1]; t->c[j].z = col[3 * vi[j] + 2]; }
                else { t->c[j].x = t->c[j].y = t->c[j].z = 255.0f; }
            }
            t->lower.x = fmin_std(t->p[0].x, fmin_std(t->p[1].x, t->p[2].x));
            t->lower.y = fmin_std(t->p[0].y, fmin_std(t->p[1].y, t->p[2].y));
            t->lower.z = fmin_std(t->p[0].z, fmin_std(t->p[1].z, t->p[2].z));
            t->upper.x = fmax_std(t->p[0].x, fmax_std(t->p[1].x, t->p[2].x));
            t->upper.y = fmax_std(t->p[0].y, fmax_std(t->p[1].y, t->p[2].y));
            t->upper.z = fmax_std(t->p[0].z, fmax_std(t->p[1].z, t->p[2].z));
            if (!nrm) {
                v3 n = normalize3(cross3(sub3(p[b], p[a]), sub3(p[e], p[a])));
                t->n[0] = t->n[1] = t->n[2] = n;
            }
            b = e;
        }
    }
    free(p);
    return m;
}

/* PlyLoader::suggestedDimensions, PlyLoader.cpp:499-504 */
void svo_oracle_mesh_dims(void *mp, int side, int dims[3]) {
    mesh *m = (mesh *)mp;
    v3 s = mul3(sub3(m->upper, m->lower), (float)(side - 2));
    dims[0] = (int)s.x + 2;
    dims[1] = (int)s.y + 2;
    dims[2] = (int)s.z + 2;
}

int svo_oracle_mesh_setup(void *mp, int side, int block, const int dims[3], int threads) {
    mesh *m = (mesh *)mp;
    m->counts = (uint8_t *)calloc((size_t)block * block * block, 1);
    if (!m->counts) return -3;
    return setup_blocks(m, side, block, dims[0], dims[1], dims[2], threads);
}

/* PlyLoader::convertToVolume, PlyLoader.cpp:506-534, into out (w*h*d words
 * of suggestedDimensions(side)): the slab height is the budget over w*h
 * bytes (blockMemRequirement counts one byte per cell), the slab is the
 * block of setupBlockProcessing, and processBlock runs slab after slab into
 * one buffer that is never cleared between slabs (the reference reuses
 * `data`), each slab's first min(slab, d - z) slices written out.  Returns -1
 * when the budget holds no slice (the reference's ASSERT), -3 on allocation
 * failure. */
int svo_oracle_mesh_to_volume(void *mp, int side, uint64_t mem, int threads, uint32_t *out) {
    mesh *m = (mesh *)mp;
    int dims[3];
    svo_oracle_mesh_dims(mp, side, dims);
    const int w = dims[0], h = dims[1], d = dims[2];
    const uint64_t slice_cost = (uint64_t)w * (uint64_t)h;
    int slice = (int)(mem / slice_cost);
    if (slice > d) slice = d;
    if (slice == 0) return -1;
    const size_t cells = (size_t)w * h * slice;
    uint32_t *data = (uint32_t *)calloc(cells, 4);
    free(m->counts);
    m->counts = (uint8_t *)calloc(cells, 1);
    free(m->offsets); m->offsets = NULL;
    free(m->lists); m->lists = NULL;
    if (!data || !m->counts) { free(data); return -3; }
    int rc = setup_blocks3(m, side, w, h, slice, w, h, d, threads);
    if (rc) { free(data); return rc; }
    for (int z = 0; z < d; z += slice) {
        svo_oracle_mesh_process_block(mp, data, 0, 0, z, w, h, slice);
        const int nz = slice < d - z ? slice : d - z;
        memcpy(out + (size_t)w * h * z, data, (size_t)w * h * nz * 4);
    }
    free(data);
    return 0;
}

int svo_oracle_mesh_num_tris(void *mp) { return ((mesh *)mp)->ntris; }

void svo_oracle_mesh_destroy(void *mp) {
    mesh *m = (mesh *)mp;
    if (!m) return;
    free(m->tris); free(m->offsets); free(m->lists); free(m->counts);
    free(m);
}
