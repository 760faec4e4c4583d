/*
 * render_oracle.c — CPU restatement of the viewer's frame loop:
 * renderBatch + renderTile (Main.cpp:92-202) without SDL.
 *
 * TEST INFRASTRUCTURE ONLY (see svo_oracle.h).  The frame is cut into
 * n_strips horizontal strips as Main.cpp:349-361 cuts it over its threads
 * (each strip keeps its own corner grid and running dx/dy sums, so the
 * pixels depend on the strip layout); per strip, level-of-detail corner
 * rays every 8 pixels give a depth, each 8x8 tile whose four corners are not
 * all misses is traced from pos + dir * max(minT - 0.03, 0), shaded and
 * packed as RGBA8; pixels of skipped tiles stay 0.  The raymarch, invSqrt
 * and shade are this directory's restatements, pinned to the reference.
 * The whole frame is pinned to the reference's own renderBatch and
 * renderTile, compiled from Main.cpp's text (ref_render.cpp), at the
 * viewer's 1280 x 720 in 16 strips (tests/test_oracle_vs_reference.py and
 * the committed frames in tests/golden/frames.npz).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "svo_oracle.h"

static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline float smax(float a, float b) { return (a < b) ? b : a; }

enum { TILE = 8 };

typedef struct {
    const uint32_t *oct;
    uint64_t nwords;
    float a[9];  /* tform a11 a12 a13 a21 ... a33 */
    float pos[3];
    float light[3];
    int W, H, stride, pixel_stride;
    float scale, aspect, tile_scale, zx, zy, zz, coarse;
    uint32_t *out;
} frame;

/* Main.cpp:92-137 */
static void render_tile(const frame *f, int x0, int y0, int x1, int y1, float minT) {
    float dy = f->aspect - (float)y0 * f->scale;
    for (int y = y0; y < y1; ++y, dy -= f->scale) {
        float dx = -1.0f + (float)x0 * f->scale;
        for (int x = x0; x < x1; ++x, dx += f->scale) {
            int cx = x - ((x - x0) % f->pixel_stride);
            int cy = y - ((y - y0) % f->pixel_stride);
            if (cx != x || cy != y) {
                f->out[x + (size_t)y * f->W] = f->out[cx + (size_t)cy * f->W];
                continue;
            }
            float d[3] = {dx * f->a[0] + dy * f->a[1] + f->zx, dx * f->a[3] + dy * f->a[4] + f->zy,
                          dx * f->a[6] + dy * f->a[7] + f->zz};
            float s = svo_oracle_inv_sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            d[0] *= s;
            d[1] *= s;
            d[2] *= s;
            float o[3] = {f->pos[0] + d[0] * minT, f->pos[1] + d[1] * minT, f->pos[2] + d[2] * minT};
            uint32_t word = 0;
            float t = 0.0f;
            float col = 0.0f;
            if (svo_oracle_raymarch(f->oct, f->nwords, o, d, 0.0f, &word, &t, NULL, NULL) == 1)
                col = svo_oracle_shade(word, d, f->light);
            /* uint32(std::min(col, 1.0f)*255.0): the product is a double */
            uint32_t c = (uint32_t)((double)smin(col, 1.0f) * 255.0);
            f->out[x + (size_t)y * f->W] = c | (c << 8) | (c << 16) | 0xFF000000u;
        }
    }
}

/* Main.cpp:139-202 for rows [y0, y1) */
static void render_batch(const frame *f, int y0, int y1) {
    const float miss = 1e10f;
    const int x0 = 0, x1 = f->W;
    const int tilesX = (x1 - x0 - 1) / TILE + 2, tilesY = (y1 - y0 - 1) / TILE + 2;
    float *depth = (float *)malloc((size_t)tilesX * tilesY * sizeof(float));
    if (!depth) return;
    if (y1 > y0) memset(f->out + (size_t)y0 * f->W, 0, (size_t)(y1 - y0) * f->W * sizeof(uint32_t));
    float dy = f->aspect - (float)y0 * f->scale;
    for (int y = 0, idx = 0; y < tilesY; y++, dy -= f->tile_scale) {
        float dx = -1.0f + (float)x0 * f->scale;
        for (int x = 0; x < tilesX; x++, dx += f->tile_scale, idx++) {
            float d[3] = {dx * f->a[0] + dy * f->a[1] + f->zx, dx * f->a[3] + dy * f->a[4] + f->zy,
                          dx * f->a[6] + dy * f->a[7] + f->zz};
            float s = svo_oracle_inv_sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            d[0] *= s;
            d[1] *= s;
            d[2] *= s;
            uint32_t word = 0;
            float t = 0.0f;
            depth[idx] = svo_oracle_raymarch(f->oct, f->nwords, f->pos, d, f->coarse, &word, &t, NULL, NULL) ? t : miss;
            if (x > 0 && y > 0) {
                float minT = smin(smin(depth[idx], depth[idx - 1]), smin(depth[idx - tilesX], depth[idx - tilesX - 1]));
                if (minT != miss) {
                    int tx0 = (x - 1) * TILE + x0, ty0 = (y - 1) * TILE + y0;
                    int tx1 = tx0 + TILE < x1 ? tx0 + TILE : x1;
                    int ty1 = ty0 + TILE < y1 ? ty0 + TILE : y1;
                    render_tile(f, tx0, ty0, tx1, ty1, smax(minT - 0.03f, 0.0f));
                }
            }
        }
    }
    free(depth);
}

typedef struct {
    const frame *f;
    int first, step, n_strips;
} worker;

static void *run_strips(void *p) {
    worker *w = (worker *)p;
    for (int i = w->first; i < w->n_strips; i += w->step) {
        int y0 = i * w->f->stride, y1 = (i + 1) * w->f->stride;
        if (y1 > w->f->H) y1 = w->f->H;
        render_batch(w->f, y0, y1);
    }
    return NULL;
}

int svo_oracle_render_frame(const uint32_t *oct, uint64_t nwords, const float rot[9], const float pos[3],
                            float plane_dist, int W, int H, int n_strips, int pixel_stride, uint32_t *out,
                            int threads) {
    if (W < 1 || H < 1 || n_strips < 1 || pixel_stride < 1) return -1;
    frame f;
    f.oct = oct;
    f.nwords = nwords;
    memcpy(f.a, rot, sizeof(f.a));
    memcpy(f.pos, pos, sizeof(f.pos));
    f.W = W;
    f.H = H;
    f.pixel_stride = pixel_stride;
    f.out = out;
    f.stride = (H - 1) / n_strips + 1;                      /* Main.cpp:349 */
    f.scale = 2.0f / (float)W;                             /* :151 */
    f.tile_scale = (float)TILE * f.scale;                  /* :152 */
    f.aspect = (float)H / (float)W;                        /* :62 */
    f.zx = plane_dist * rot[2];                            /* :154 */
    f.zy = plane_dist * rot[5];
    f.zz = plane_dist * rot[8];
    f.coarse = 2.0f * (float)TILE / (plane_dist * (float)H); /* :155 */
    /* light = (tform * Vec3(-1, 1, -1)).normalize() with tform's translation
     * zeroed (:147, :158; Mat4::operator* adds a14 = 0) */
    float l[3] = {rot[0] * -1.0f + rot[1] * 1.0f + rot[2] * -1.0f + 0.0f,
                  rot[3] * -1.0f + rot[4] * 1.0f + rot[5] * -1.0f + 0.0f,
                  rot[6] * -1.0f + rot[7] * 1.0f + rot[8] * -1.0f + 0.0f};
    float inv = 1.0f / sqrtf(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
    f.light[0] = l[0] * inv;
    f.light[1] = l[1] * inv;
    f.light[2] = l[2] * inv;
    if (threads < 1) threads = 1;
    if (threads > n_strips) threads = n_strips;
    pthread_t th[64];
    worker w[64];
    if (threads > 64) threads = 64;
    for (int i = 0; i < threads; ++i) {
        w[i].f = &f;
        w[i].first = i;
        w[i].step = threads;
        w[i].n_strips = n_strips;
    }
    for (int i = 1; i < threads; ++i) pthread_create(&th[i], NULL, run_strips, &w[i]);
    run_strips(&w[0]);
    for (int i = 1; i < threads; ++i) pthread_join(th[i], NULL);
    return 0;
}

/* 1 / std::tan(float(M_PI) / 6.0f) (Main.cpp:153), the float overload. */
float svo_oracle_plane_dist(void) { return 1.0f / tanf(3.14159265358979323846f / 6.0f); }
