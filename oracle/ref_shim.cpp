/*
 * Test-oracle shim over the reference implementation, compiled in place.
 *
 * This file is test infrastructure.  It is compiled together with the
 * reference's own sources (VoxelOctree.cpp, VoxelData.cpp, PlyLoader.cpp,
 * thread/*.cpp and the vendored lz4/plyfile/tribox3 C files) by
 * oracle/Makefile into oracle/_ref/libsvo_ref.so, and only tests and the
 * golden-fixture script load it.  It exposes the reference's behaviour
 * through a flat C ABI so that Python tests can call it with ctypes:
 *
 *   - VoxelOctree(const char *path)           VoxelOctree.cpp:57-90
 *   - VoxelOctree::save                       VoxelOctree.cpp:92-123
 *   - VoxelOctree(VoxelData *)                VoxelOctree.cpp:125-137
 *   - VoxelData(const char *path, size_t mem) VoxelData.cpp:37-48
 *   - VoxelData(PlyLoader *, int, size_t)     VoxelData.cpp:50-56
 *   - PlyLoader::convertToVolume              PlyLoader.cpp:506-534 (without its file)
 *   - VoxelOctree::raymarch                   VoxelOctree.cpp:207-346
 *   - compressMaterial / decompressMaterial   Util.hpp:64-100
 *   - triBoxOverlap                           third-party/tribox3.c:132-206
 *
 * The octree words are private members of VoxelOctree; the shim reads them
 * through member pointers formed by explicit template instantiation, where
 * access checking does not apply (C++11 [temp.explicit]/12).
 */
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include <memory>

#include "VoxelOctree.hpp"
#include "VoxelData.hpp"
#include "PlyLoader.hpp"
#include "Util.hpp"
#include "thread/ThreadUtils.hpp"
#include "third-party/tribox3.h"

namespace {
template <typename Tag, typename Tag::type M>
struct MemberAccess {
    friend typename Tag::type member(Tag) { return M; }
};
struct OctreeWordsTag {
    typedef std::unique_ptr<uint32[]> VoxelOctree::*type;
    friend type member(OctreeWordsTag);
};
struct OctreeSizeTag {
    typedef uint64 VoxelOctree::*type;
    friend type member(OctreeSizeTag);
};
template struct MemberAccess<OctreeWordsTag, &VoxelOctree::_octree>;
template struct MemberAccess<OctreeSizeTag, &VoxelOctree::_octreeSize>;
}

extern "C" {

int ref_start_threads(int n) {
    ThreadUtils::startThreads(n);
    return 0;
}

void *ref_build_voxel_file(const char *voxel_path, uint64_t mem) {
    std::unique_ptr<VoxelData> data(new VoxelData(voxel_path, size_t(mem)));
    return new VoxelOctree(data.get());
}

void *ref_build_ply(const char *ply_path, int side, uint64_t mem) {
    std::unique_ptr<PlyLoader> loader(new PlyLoader(ply_path));
    std::unique_ptr<VoxelData> data(new VoxelData(loader.get(), side, size_t(mem)));
    return new VoxelOctree(data.get());
}

int ref_ply_to_voxel_file(const char *ply_path, const char *voxel_path, int side, uint64_t mem) {
    std::unique_ptr<PlyLoader> loader(new PlyLoader(ply_path));
    loader->convertToVolume(voxel_path, side, size_t(mem));
    return 0;
}

// PlyLoader::convertToVolume (PlyLoader.cpp:506-534) into `out` instead of
// a file: the same suggestedDimensions, slab height (budget / w*h bytes),
// setupBlockProcessing with the slab as the block, and processBlock slab
// after slab into one buffer that is reused without clearing, as the
// reference reuses `data`.  convertToVolume never calls isBlockEmpty, so
// processBlock's progress line divides by a zero block count (SIGFPE on
// x86-64; AArch64 integer division gives 0 and the conversion completes).
// One isBlockEmpty call on the first slab that holds triangles makes that
// count nonzero; it only feeds the progress line.  The reference's buffer
// comes from new[] uninitialised (fresh zero pages for large volumes); here
// it starts zeroed.  dims gets w, h, d; with out == NULL nothing else runs.
// Returns -1 when the budget holds no slice (the reference's ASSERT).
int ref_ply_volume(const char *ply_path, int side, uint64_t mem, int *dims, uint32_t *out) {
    std::unique_ptr<PlyLoader> loader(new PlyLoader(ply_path));
    int w, h, d;
    loader->suggestedDimensions(side, w, h, d);
    dims[0] = w;
    dims[1] = h;
    dims[2] = d;
    if (!out) return 0;
    size_t sliceCost = loader->blockMemRequirement(w, h, 1);
    int sliceZ = std::min((int)(size_t(mem) / sliceCost), d);
    if (sliceZ == 0) return -1;
    std::vector<uint32> data(size_t(w) * size_t(h) * size_t(sliceZ), 0u);
    loader->setupBlockProcessing(side, w, h, sliceZ, w, h, d);
    bool any = false;
    for (int z = 0; z < d && !any; z += sliceZ) any = !loader->isBlockEmpty(0, 0, z);
    for (int z = 0; z < d; z += sliceZ) {
        if (any) loader->processBlock(data.data(), 0, 0, z, w, h, sliceZ);
        size_t n = size_t(w) * size_t(h) * size_t(std::min(sliceZ, d - z));
        std::memcpy(out + size_t(w) * size_t(h) * size_t(z), data.data(), n * sizeof(uint32));
    }
    loader->teardownBlockProcessing();
    return 0;
}

void *ref_load(const char *oct_path) {
    return new VoxelOctree(oct_path);
}

int ref_save(void *tree, const char *oct_path) {
    static_cast<VoxelOctree *>(tree)->save(oct_path);
    return 0;
}

void ref_free(void *tree) {
    delete static_cast<VoxelOctree *>(tree);
}

uint64_t ref_num_words(void *tree) {
    return static_cast<VoxelOctree *>(tree)->*member(OctreeSizeTag());
}

const uint32_t *ref_words(void *tree) {
    return (static_cast<VoxelOctree *>(tree)->*member(OctreeWordsTag())).get();
}

void ref_center(void *tree, float *c) {
    Vec3 v = static_cast<VoxelOctree *>(tree)->center();
    c[0] = v.x; c[1] = v.y; c[2] = v.z;
}

/* rays: 6 floats per ray (ox, oy, oz, dx, dy, dz).  hit/t/word may be NULL.
 * Work is interleaved over `threads` std::threads in chunks of 1024 rays. */
void ref_raymarch(void *tree, const float *rays, uint64_t n, float rayScale,
                  uint8_t *hit, float *t, uint32_t *word, int threads) {
    VoxelOctree *oct = static_cast<VoxelOctree *>(tree);
    const uint64_t chunk = 1024;
    auto body = [&](int id) {
        for (uint64_t base = uint64_t(id) * chunk; base < n; base += uint64_t(threads) * chunk) {
            uint64_t end = base + chunk < n ? base + chunk : n;
            for (uint64_t i = base; i < end; ++i) {
                const float *r = rays + 6 * i;
                uint32 w = 0;
                float tt = 0.0f;
                bool h = oct->raymarch(Vec3(r[0], r[1], r[2]), Vec3(r[3], r[4], r[5]), rayScale, w, tt);
                if (hit) hit[i] = h ? 1 : 0;
                if (t) t[i] = h ? tt : 0.0f;
                if (word) word[i] = h ? w : 0;
            }
        }
    };
    if (threads <= 1) {
        threads = 1;
        body(0);
        return;
    }
    std::vector<std::thread> pool;
    for (int k = 0; k < threads; ++k)
        pool.emplace_back(body, k);
    for (auto &th : pool)
        th.join();
}

uint32_t ref_compress_material(const float *n, float shade) {
    return compressMaterial(Vec3(n[0], n[1], n[2]), shade);
}

void ref_decompress_material(uint32_t w, float *n, float *shade) {
    Vec3 v;
    float s;
    decompressMaterial(w, v, s);
    n[0] = v.x; n[1] = v.y; n[2] = v.z;
    *shade = s;
}

float ref_inv_sqrt(float x) {
    return invSqrt(x);
}

int ref_tri_box_overlap(const float *center, const float *half, const float *verts9) {
    float c[3] = {center[0], center[1], center[2]};
    float h[3] = {half[0], half[1], half[2]};
    float v[3][3];
    std::memcpy(v, verts9, sizeof(v));
    return triBoxOverlap(c, h, v);
}

} /* extern "C" */
