// Exercises include/svo_voxel_octree.hpp the way the reference's code would
// use VoxelOctree (src/VoxelOctree.hpp:37-58), linked against libsvo_gb300.so.
//
//   voxel_octree_main host <in.oct> <out.oct>
//       .oct read/write through the C ABI (no GPU), and the class's error
//       path: loading a missing file throws.
//   voxel_octree_main gpu <in.oct> <saved.oct> <rays.bin> <results.bin>
//       VoxelOctreeGpu(path), center(), save(); the batch raymarch at
//       rayScale 0 and 0.02, and the one-ray raymarch for every ray at
//       rayScale 0; results written as raw arrays for the test to compare.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "svo_voxel_octree.hpp"

struct Vec3 {  // stands in for the reference's math/Vec3.hpp
    float x, y, z;
    Vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
typedef BasicVoxelOctreeGpu<Vec3> VoxelOctreeGpu;

static int host_mode(const char *in, const char *out) {
    uint32_t *words = 0;
    uint64_t n = 0;
    float c[3];
    if (svo_oct_read(in, &words, &n, c) != SVO_OK) {
        fprintf(stderr, "read: %s\n", svo_last_error());
        return 1;
    }
    if (svo_oct_write(out, words, n, c) != SVO_OK) {
        fprintf(stderr, "write: %s\n", svo_last_error());
        return 1;
    }
    printf("words %llu center %.9g %.9g %.9g\n", (unsigned long long)n, c[0], c[1], c[2]);
    svo_free(words);
    try {
        VoxelOctreeGpu missing("/nonexistent/dir/missing.oct");
        printf("no error\n");
        return 1;
    } catch (const std::runtime_error &e) {
        printf("error: %s\n", e.what());
    }
    return 0;
}

static int gpu_mode(const char *in, const char *saved, const char *rays_path, const char *results) {
    FILE *f = fopen(rays_path, "rb");
    if (!f) return 1;
    fseek(f, 0, SEEK_END);
    long bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<float> rays(bytes / sizeof(float));
    if (fread(&rays[0], 1, bytes, f) != (size_t)bytes) return 1;
    fclose(f);
    size_t n = rays.size() / 6;

    VoxelOctreeGpu tree(in);
    Vec3 c = tree.center();
    printf("center %.9g %.9g %.9g\n", c.x, c.y, c.z);
    tree.save(saved);

    std::vector<uint8_t> hit, lod_hit;
    std::vector<uint32_t> normal, lod_normal;
    std::vector<float> t, lod_t;
    tree.raymarch(rays, 0.0f, hit, normal, t);
    tree.raymarch(rays, 0.02f, lod_hit, lod_normal, lod_t);
    // the reference's one-ray signature; a miss leaves normal and t unset
    std::vector<uint8_t> one_hit(n);
    std::vector<uint32_t> one_normal(n, 0);
    std::vector<float> one_t(n, 0.0f);
    for (size_t i = 0; i < n; ++i) {
        const float *r = &rays[6 * i];
        one_hit[i] = tree.raymarch(Vec3(r[0], r[1], r[2]), Vec3(r[3], r[4], r[5]), 0.0f, one_normal[i], one_t[i]);
    }
    FILE *o = fopen(results, "wb");
    if (!o) return 1;
    fwrite(&hit[0], 1, n, o);
    fwrite(&t[0], 4, n, o);
    fwrite(&normal[0], 4, n, o);
    fwrite(&lod_hit[0], 1, n, o);
    fwrite(&lod_t[0], 4, n, o);
    fwrite(&one_hit[0], 1, n, o);
    fwrite(&one_t[0], 4, n, o);
    fwrite(&one_normal[0], 4, n, o);
    fclose(o);
    return 0;
}

int main(int argc, char **argv) {
    if (argc == 4 && !strcmp(argv[1], "host")) return host_mode(argv[2], argv[3]);
    if (argc == 6 && !strcmp(argv[1], "gpu")) {
        try {
            return gpu_mode(argv[2], argv[3], argv[4], argv[5]);
        } catch (const std::runtime_error &e) {
            fprintf(stderr, "error: %s\n", e.what());
            return 2;
        }
    }
    fprintf(stderr, "usage: %s host <in.oct> <out.oct> | gpu <in.oct> <saved.oct> <rays.bin> <results.bin>\n",
            argv[0]);
    return 64;
}
