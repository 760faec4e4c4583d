/*
 * svo_oracle — CPU restatement of the reference's octree hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Tests, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load liboracle.so as the checker
 * or as the timed CPU baseline.  The product library never links or calls it.
 *
 * Every function restates one reference function step for step (same float
 * operation order, compiled without FP contraction) and cites it by
 * file:line within the reference project.
 */
#ifndef SVO_ORACLE_H
#define SVO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Util.hpp:47-58 (Quake III inverse square root with one Newton step). */
float svo_oracle_inv_sqrt(float x);
/* Util.hpp:64-84. */
uint32_t svo_oracle_compress_material(const float n[3], float shade);
/* Util.hpp:86-100. */
void svo_oracle_decompress_material(uint32_t word, float n[3], float *shade);
/* Main.cpp:81-90: grey value (the reference returns it in all three channels). */
float svo_oracle_shade(uint32_t word, const float dir[3], const float light[3]);

/* VoxelOctree.cpp:207-346.  Returns 0 on a miss, 1 on a leaf hit, 2 on a
 * level-of-detail exit (rayScale > 0, VoxelOctree.cpp:265-268).
 * word: the leaf payload (`normal` in the reference), written on a leaf hit.
 * t:    written on any hit.
 * leaf: index of the leaf word in `oct` (VoxelOctree.cpp:282), leaf hits only.
 * loads: incremented once per octree word read (descriptor :254, far word
 *        :279, leaf word :282); may be NULL. */
int svo_oracle_raymarch(const uint32_t *oct, uint64_t nwords, const float o[3], const float d[3],
                        float rayScale, uint32_t *word, float *t, uint64_t *leaf, uint64_t *loads);

/* Batch form over `threads` pthreads, rays = 6 floats (o, d) per ray.
 * Outputs (each may be NULL): hit (0/1/2), t (+inf on miss), leaf index
 * (0xFFFFFFFF when no leaf), leaf word (0 when no leaf), grey shade
 * (svo_oracle_shade with `light`, 0 when no leaf) and per-ray load counts. */
void svo_oracle_raymarch_batch(const uint32_t *oct, uint64_t nwords, const float *rays, uint64_t nrays,
                               float rayScale, const float light[3], uint8_t *hit, float *t,
                               uint32_t *leaf, uint32_t *word, float *grey, uint32_t *loads, int threads);

/* VoxelOctree(VoxelData*) (VoxelOctree.cpp:125-205) over VoxelData(path, mem)
 * (VoxelData.cpp:37-48, 211-291) with the .voxel payload given in memory:
 * grid = w*h*d words, x fastest, 0 = empty.  On success returns 0 and
 * *words (free with svo_oracle_free), *nwords, center[3].
 * Returns -1 when `mem` is too small (the reference exits the process),
 * -2 when the virtual side is < 2 (the reference recurses without end),
 * -3 on allocation failure. */
int svo_oracle_build_dense(const uint32_t *grid, int w, int h, int d, uint64_t mem,
                           uint32_t **words, uint64_t *nwords, float center[3]);

/* Cache-block edge M that VoxelData::init (VoxelData.cpp:211-262) picks for
 * the given dims, memory budget and per-cell cost (4 for .voxel input,
 * 5 for the PLY path); 0 when no block fits. */
uint64_t svo_oracle_cache_block(int w, int h, int d, uint64_t mem, uint64_t cell_cost);

/* VoxelOctree(const char*) payload decode (VoxelOctree.cpp:57-90): header
 * float center[3], uint64 nWords, then per 64 MiB of payload a uint64
 * compressed size and an LZ4 block that may reference earlier output.
 * Returns 0 on success, <0 on a truncated or corrupt stream. */
int svo_oracle_oct_decode(const uint8_t *bytes, uint64_t len, uint32_t **words, uint64_t *nwords,
                          float center[3]);

void svo_oracle_free(void *p);

/* scene_build.c: the synthetic scene of scenes.py on host threads.  box: 6
 * ints per sphere (x0, x1, y0, y1, z0, z1), params: 4 floats (cx, cy, cz, r);
 * heights may be NULL.  Returns Morton-ordered keys and payload words
 * (free both with svo_oracle_free). */
int svo_oracle_scene_voxels(int side, const float *heights, float thickness, const int *box, const float *params,
                            int n_spheres, int threads, uint64_t **keys, uint32_t **payload, uint64_t *n_voxels);

/* Octree words of VoxelOctree(VoxelData*) for a cube of edge 2^log_side
 * given its voxels in ascending Morton order (equal power-of-two dims only,
 * where the reference's VoxelData corner cases do not arise). */
int svo_oracle_build_sorted(const uint64_t *keys, const uint32_t *payload, uint64_t n, int log_side,
                            uint32_t **words, uint64_t *n_words);

/* ply_oracle.c: the reference's mesh path.  svo_oracle_mesh_create takes a
 * parsed PLY (positions, optional vertex normals and colours as floats,
 * faces as [count, idx...] runs) and restates PlyLoader's rescale and
 * triangulation; svo_oracle_build_mesh then runs VoxelData(PlyLoader*,
 * side, mem) with `threads` sub-block partitions and VoxelOctree(VoxelData*).
 * Returns 0, or -1 (mem too small), -2 (side < 2), -3 (allocation),
 * -5 (a triangle's block cell lies outside the block grid). */
void *svo_oracle_mesh_create(const float *pos, const float *nrm, const float *col, int n_verts, const int *faces,
                             int n_faces);
void svo_oracle_mesh_dims(void *mesh, int side, int dims[3]);
int svo_oracle_mesh_num_tris(void *mesh);
void svo_oracle_mesh_destroy(void *mesh);
int svo_oracle_build_mesh(void *mesh, int side, int threads, uint64_t mem, uint32_t **words, uint64_t *nwords,
                          float center[3]);
/* PlyLoader::convertToVolume (the builder's --mode 1) into out: w*h*d words
 * of svo_oracle_mesh_dims(side), x fastest.  Returns 0, -1 (mem holds no
 * slice), -3 (allocation), -5 (as above). */
int svo_oracle_mesh_to_volume(void *mesh, int side, uint64_t mem, int threads, uint32_t *out);
/* render_oracle.c: the viewer's frame (Main.cpp:92-202, n_strips strips as
 * its threads cut it, pixel_stride 1 or the half-size 3), RGBA8 into out
 * (W*H words, row-major).  rot = tform a11..a33, pos = the camera position
 * in the octree frame, plane_dist = svo_oracle_plane_dist(). */
int svo_oracle_render_frame(const uint32_t *oct, uint64_t nwords, const float rot[9], const float pos[3],
                            float plane_dist, int W, int H, int n_strips, int pixel_stride, uint32_t *out,
                            int threads);
float svo_oracle_plane_dist(void);

/* Triangle/box overlap (separating axes), third-party/tribox3.c:132-206. */
int svo_oracle_tri_box_overlap(const float center[3], const float half[3], const float verts[9]);

#ifdef __cplusplus
}
#endif
#endif
