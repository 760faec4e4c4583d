/*
 * ref_render.cpp — the reference viewer's frame computed by the reference's
 * own code: BatchData, shade, renderTile and renderBatch (Main.cpp:71-202),
 * whose text the Makefile copies out of Main.cpp into _ref/main_render.inc
 * at build time.  Main.cpp as a whole needs SDL for its window and event
 * loop, so only these functions are compiled; the globals they read are
 * given here (the viewer's values, Main.cpp:56-69), with the back buffer as
 * a plain block of 1280 x 720 RGBA8 pixels.
 *
 * TEST INFRASTRUCTURE ONLY: pins oracle/render_oracle.c (and through it the
 * GPU frame renderer) to the reference.  Nothing in the library uses it.
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "Util.hpp"
#include "VoxelOctree.hpp"
#include "math/Mat4.hpp"
#include "math/MatrixStack.hpp"
#include "math/Vec3.hpp"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

namespace {

const int NumThreads = 16;
const int GWidth = 1280;
const int GHeight = 720;
const float AspectRatio = GHeight / (float)GWidth;
const int TileSize = 8;

struct PixelBlock {
    void *pixels;
    int pitch;
};
PixelBlock *backBuffer;
std::atomic<bool> renderHalfSize;

#include "main_render.inc"

}  // namespace

/* One frame at the viewer's 1280 x 720 in its 16 strips (the strip set-up of
 * Main.cpp:349-361, run strip after strip: each strip writes only its own
 * rows).  The camera is the viewer's matrix stacks with MODEL = identity and
 * VIEW = [rot | trans], so renderBatch's inverse model-view matrix is
 * [rot | trans] and its eye position trans + center + 1.  out: 1280 * 720
 * pixels, row-major. */
extern "C" int ref_render_frame(void *tree, const float rot[9], const float trans[3], int half_size, uint32_t *out) {
    VoxelOctree *oct = static_cast<VoxelOctree *>(tree);
    MatrixStack::set(MODEL_STACK, Mat4());
    MatrixStack::set(VIEW_STACK, Mat4(rot[0], rot[1], rot[2], trans[0], rot[3], rot[4], rot[5], trans[1], rot[6],
                                      rot[7], rot[8], trans[2], 0.0f, 0.0f, 0.0f, 1.0f));
    PixelBlock block = {out, GWidth * 4};
    backBuffer = &block;
    renderHalfSize = half_size != 0;
    const int stride = (GHeight - 1) / NumThreads + 1;
    for (int i = 0; i < NumThreads; i++) {
        BatchData d;
        d.id = i;
        d.tree = oct;
        d.x0 = 0;
        d.x1 = GWidth;
        d.y0 = i * stride;
        d.y1 = std::min((i + 1) * stride, GHeight);
        d.tilesX = (d.x1 - d.x0 - 1) / TileSize + 2;
        d.tilesY = (d.y1 - d.y0 - 1) / TileSize + 2;
        std::vector<float> depth((size_t)d.tilesX * d.tilesY);
        d.depthBuffer = depth.data();
        renderBatch(&d);
    }
    backBuffer = nullptr;
    return 0;
}
