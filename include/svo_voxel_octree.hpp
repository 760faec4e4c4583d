// svo_voxel_octree.hpp — a VoxelOctree-shaped C++ class over the C ABI of
// svo.h, for code written against the reference's src/VoxelOctree.hpp:37-58.
//
// Header-only; link with -lsvo_gb300.  The class is a template over the
// caller's 3-vector type (any type with float members x, y, z and a
// (x, y, z) constructor).  Included after the reference's math/Vec3.hpp it
// also defines `VoxelOctreeGpu` for the reference's own Vec3, so that
//
//   #include "math/Vec3.hpp"
//   #include "svo_voxel_octree.hpp"
//   VoxelOctreeGpu tree("models/XYZRGB-Dragon.oct");
//
// replaces `VoxelOctree tree("models/XYZRGB-Dragon.oct");`.
//
// Errors: the reference reports none (a failed fopen leaves a broken object,
// VoxelOctree.cpp:60); this class throws std::runtime_error with
// svo_last_error()'s message instead.
#ifndef SVO_VOXEL_OCTREE_HPP_
#define SVO_VOXEL_OCTREE_HPP_

#include <stddef.h>
#include <stdint.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "svo.h"

template <class Vec3T>
class BasicVoxelOctreeGpu {
    svo_octree *_h;

    static void check(int rc) {
        if (rc != SVO_OK) throw std::runtime_error(std::string(svo_last_error()));
    }

    BasicVoxelOctreeGpu(const BasicVoxelOctreeGpu &);
    BasicVoxelOctreeGpu &operator=(const BasicVoxelOctreeGpu &);

public:
    // VoxelOctree(const char *path): load a .oct file (VoxelOctree.cpp:57-90).
    explicit BasicVoxelOctreeGpu(const char *path) : _h(0) { check(svo_octree_load(path, &_h)); }

    // VoxelOctree(VoxelData*) over VoxelData(path, mem), a .voxel file
    // (VoxelOctree.cpp:125-205, VoxelData.cpp:37-48).
    BasicVoxelOctreeGpu(const char *voxelPath, size_t mem) : _h(0) {
        check(svo_octree_build_voxel_file(voxelPath, mem, 0, &_h));
    }

    // VoxelOctree(VoxelData*) over VoxelData(new PlyLoader(plyPath), side, mem)
    // (VoxelData.cpp:50-56).  `threads` is the size the reference's thread pool
    // would have: its voxelization depends on it (PlyLoader.cpp:381-405).
    BasicVoxelOctreeGpu(const char *plyPath, int side, int threads, size_t mem) : _h(0) {
        check(svo_octree_build_ply(plyPath, side, threads, mem, 0, &_h));
    }

    ~BasicVoxelOctreeGpu() { svo_octree_destroy(_h); }

    // VoxelOctree::save (VoxelOctree.cpp:92-123).
    void save(const char *path) const { check(svo_octree_save(_h, path)); }

    // VoxelOctree::center (VoxelOctree.hpp:55-57).
    Vec3T center() const {
        float c[3];
        check(svo_octree_center(_h, c));
        return Vec3T(c[0], c[1], c[2]);
    }

    // VoxelOctree::raymarch (VoxelOctree.cpp:207-346) with its signature:
    // one ray, one GPU round trip.  As in the reference, `normal` is left
    // unset on a level-of-detail exit (rayScale > 0) and nothing is written
    // on a miss.
    bool raymarch(const Vec3T &o, const Vec3T &d, float rayScale, uint32_t &normal, float &t) const {
        float r[6] = {o.x, o.y, o.z, d.x, d.y, d.z};
        uint8_t h = 0;
        float tt = 0.0f;
        uint32_t w = 0;
        svo_trace_out out = {&h, &tt, 0, &w, 0, 0};
        const float light[3] = {0.0f, 0.0f, 1.0f};
        check(svo_trace_host(_h, r, 1, rayScale, light, &out));
        if (h == 0) return false;
        t = tt;
        if (h == 1) normal = w;
        return true;
    }

    // The same for a batch of rays (6 floats per ray: o then d), one call:
    // hit is 0 (miss), 1 (hit, normal set) or 2 (level-of-detail exit).
    void raymarch(const std::vector<float> &rays, float rayScale, std::vector<uint8_t> &hit,
                  std::vector<uint32_t> &normal, std::vector<float> &t) const {
        size_t n = rays.size() / 6;
        hit.resize(n);
        normal.resize(n);
        t.resize(n);
        if (n == 0) return;
        svo_trace_out out = {&hit[0], &t[0], 0, &normal[0], 0, 0};
        const float light[3] = {0.0f, 0.0f, 1.0f};
        check(svo_trace_host(_h, &rays[0], n, rayScale, light, &out));
    }

    // The handle, for the library's other entry points (svo_trace_image,
    // svo_render_frame, svo_batch_*).
    svo_octree *handle() const { return _h; }
};

#ifdef MATH_VEC3_HPP_
typedef BasicVoxelOctreeGpu<Vec3> VoxelOctreeGpu;
#endif

#endif  // SVO_VOXEL_OCTREE_HPP_
