/*
 * svo.h — C ABI of the GB300 sparse-voxel-octree library (libsvo_gb300.so).
 *
 * Drop-in boundary for the reference's VoxelOctree hot path
 * (tunabrain/sparse-voxel-octrees, src/VoxelOctree.hpp:37-58):
 *   build (voxels -> 32-bit child-descriptor octree), .oct load/save, and the
 *   FP32 ESVO raymarch returning hit t, leaf payload word, leaf index and the
 *   viewer's shaded colour.
 *
 * Conventions
 *   - Every function returns an int status: SVO_OK (0) or a negative SVO_ERR_*.
 *     svo_last_error() returns a message for the calling thread's last failure.
 *   - No exceptions cross this boundary; no allocation is hidden from the
 *     caller except inside the opaque svo_octree handle and its staging pool.
 *   - `stream` is a cudaStream_t passed as void*; NULL selects the legacy
 *     default stream.  Functions taking device pointers are asynchronous with
 *     respect to the host on that stream; *_host functions return after their
 *     results are in host memory.
 *   - Octree words live in HBM for the lifetime of the handle; a host copy is
 *     made on demand (svo_octree_copy_words, svo_octree_save).
 *   - The word layout is the reference's: bits [31:18] child offset (or its
 *     high part when far), [17] far flag, [16] children carry far words,
 *     [15:8] valid mask, [7:0] non-leaf mask, child octant i on bit 128>>i,
 *     child slots in descending octant order, root at index 0.
 *
 * Limits: the GPU paths address at most 2^32-1 octree words and 2^32-1 rays
 * per call; the build accepts virtual sides 2..65536.
 */
#ifndef SVO_GB300_H
#define SVO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SVO_OK 0
#define SVO_ERR_INVALID (-1) /* bad argument (null pointer, bad size, bad option) */
#define SVO_ERR_IO (-2)      /* a file could not be opened, read or written */
#define SVO_ERR_FORMAT (-3)  /* truncated or corrupt .oct / .voxel / .ply stream */
#define SVO_ERR_MEMORY (-4)  /* host or device allocation failed, or `mem` budget below the minimum */
#define SVO_ERR_CUDA (-5)    /* a CUDA runtime call failed */
#define SVO_ERR_LIMIT (-6)   /* input beyond a documented limit */
#define SVO_ERR_DEVICE (-7)  /* a kernel raised its error flag (step cap or bounds check) */

typedef struct svo_octree svo_octree;
typedef void *svo_stream;

/* Message for the calling thread's last failing call ("" if none). */
const char *svo_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int svo_version(void);

/* ------------------------------------------------------------------ handle */

/* Replaces VoxelOctree::VoxelOctree(const char *path), VoxelOctree.cpp:57-90.
 * Reads the .oct header (float center[3], uint64 nWords) and the 64 MiB
 * LZ4 blocks, then uploads the words to the current device.  Unlike the
 * reference (which leaves a broken object when fopen fails) a missing or
 * corrupt file returns SVO_ERR_IO / SVO_ERR_FORMAT. */
int svo_octree_load(const char *path, svo_octree **out);

/* Replaces VoxelOctree::save(const char *path), VoxelOctree.cpp:92-123.
 * Same header and block framing; each 64 MiB block is LZ4-compressed
 * independently, which the reference's streaming decoder reads unchanged. */
int svo_octree_save(const svo_octree *oct, const char *path);

/* Host-only .oct codec (no device involved): svo_oct_read decodes a file
 * into a malloc'd word array (free it with svo_free); svo_oct_write encodes
 * host words.  svo_octree_load / svo_octree_save are these plus the upload /
 * download of the words. */
int svo_oct_read(const char *path, uint32_t **words, uint64_t *n_words, float center[3]);
int svo_oct_write(const char *path, const uint32_t *words, uint64_t n_words, const float center[3]);
void svo_free(void *p);

/* Wraps an existing word array (host memory) with its center; the words are
 * copied to the device.  Used to trace octrees produced elsewhere. */
int svo_octree_from_words(const uint32_t *words, uint64_t n_words, const float center[3], svo_octree **out);

/* The builds keep their freed scratch memory in a per-device pool of the
 * library for the next build; this returns that memory to the driver (after
 * a device synchronisation). */
int svo_trim_memory(void);

/* Frees the handle and its device memory. */
int svo_octree_destroy(svo_octree *oct);

/* Number of 32-bit words (VoxelOctree::_octreeSize, VoxelOctree.hpp:40). */
int svo_octree_num_words(const svo_octree *oct, uint64_t *n_words);

/* Index width of svo_trace / svo_trace_host: 32 (the default) or 64.
 * Octrees above 2^32-1 words always trace with 64-bit word indices (their far
 * offsets carry bits above 32, VoxelOctree.cpp:190-194, :277-280); 64 selects
 * that kernel for smaller octrees too, with identical results.  32 is refused
 * for octrees above 2^32-1 words.  Above 2^32-1 words svo_trace refuses the
 * 32-bit `leaf` output and the image, batched, load-count, frame and
 * leaf-shading entry points return SVO_ERR_LIMIT. */
int svo_octree_set_index_width(svo_octree *oct, int bits);

/* The traversal kernels walk a descriptor table (16 bytes per node: the
 * descriptor, its children's table position and its child block) that the
 * first trace call on a handle builds after checking every reachable node;
 * results are identical to the word traversal of VoxelOctree.cpp:252-339,
 * which runs instead where the table cannot be built (octrees over 2^32-1
 * words, or a node whose offsets leave the array) and inside graph capture
 * before the table exists.  enable = 0 selects the word traversal. */
int svo_octree_set_table(svo_octree *oct, int enable);

/* Builds the descriptor table now if the octree qualifies (synchronous) and
 * returns its entry count, or 0 when it does not qualify. */
int svo_octree_table_size(svo_octree *oct, uint64_t *entries);

/* Copies the words to host memory `dst` (n_words entries). */
int svo_octree_copy_words(const svo_octree *oct, uint32_t *dst, uint64_t n_words);

/* Device pointer to the resident words (valid until svo_octree_destroy). */
int svo_octree_device_words(const svo_octree *oct, const uint32_t **d_words);

/* Replaces VoxelOctree::center(), VoxelOctree.hpp:55-57. */
int svo_octree_center(const svo_octree *oct, float center[3]);

/* Reads and clears the handle's device error word.  Bit 0 is set when an
 * asynchronous svo_trace call had a ray stop at the traversal step cap or at
 * an out-of-range word index (only possible on a corrupt octree). */
int svo_octree_device_status(svo_octree *oct, uint32_t *flags);

/* Walks the octree from the root and checks the descriptor invariants
 * (offsets in range, far words present, leaf masks, no cycles).  Returns
 * SVO_OK and the number of descriptors and leaves, or SVO_ERR_FORMAT. */
int svo_octree_validate(const svo_octree *oct, uint64_t *n_descriptors, uint64_t *n_leaves);

/* ------------------------------------------------------------------- build */

/* Replaces VoxelOctree::VoxelOctree(VoxelData *) (VoxelOctree.cpp:125-205)
 * over VoxelData(const char *path, size_t mem) (VoxelData.cpp:37-48) on the
 * GPU: occupied-voxel extraction in Morton order, then a bottom-up level
 * pass (valid masks, subtree word counts, far-pointer decisions) and a
 * top-down placement pass that writes the reference's exact word stream.
 *   grid: w*h*d uint32 voxels, x fastest, 0 = empty (the .voxel payload,
 *         PlyLoader.cpp:521-528); host memory, or device memory when
 *         grid_on_device != 0.
 *   mem:  the reference's memory budget; it selects VoxelData's cache-block
 *         edge (VoxelData.cpp:211-244), which decides two corner cases of the
 *         reference's output that this build reproduces: a buffer of odd
 *         depth never marks its last z slice (VoxelData.cpp:163-170), and a
 *         cache block whose only voxels lie in that slice still appears as
 *         an empty descriptor.  Pass 1 << 30 for the reference's default.
 * Returns SVO_ERR_MEMORY when `mem` admits no cache block (the reference
 * exits the process) and SVO_ERR_INVALID when the virtual side is below 2. */
int svo_octree_build_dense(const uint32_t *grid, int w, int h, int d, uint64_t mem, int grid_on_device,
                           svo_stream stream, svo_octree **out);

/* Same as svo_octree_build_dense, reading a .voxel file (int32 w, h, d then
 * w*h*d uint32, x fastest), i.e. VoxelData(const char *path, size_t mem).
 * A grid larger than half the free device memory is not loaded whole: the
 * file is streamed in z slabs (as VoxelData reads it block by block,
 * VoxelData.cpp:177-209), only occupied voxels are kept on the device, and a
 * radix sort restores their Morton order; the words are the same. */
int svo_octree_build_voxel_file(const char *path, uint64_t mem, svo_stream stream, svo_octree **out);

/* svo_octree_build_voxel_file with the streamed form forced and slabs of
 * about slab_bytes of device memory (at least 16 slices): for a bounded
 * device footprint.  Needs a virtual side of at least 16. */
int svo_octree_build_voxel_file_streamed(const char *path, uint64_t mem, uint64_t slab_bytes, svo_stream stream,
                                         svo_octree **out);

/* No counterpart in the reference.  The GPU build of svo_octree_build_dense
 * for callers that cannot allocate device memory while they run: a host
 * application whose device memory is already handed to its own pool, or a
 * frame loop that must not take the device-wide synchronisation that
 * cudaMalloc / cudaFree imply.  This call allocates nothing: its working
 * memory is one fixed 32 MiB device arena inside the library (reserved on
 * every device that loads the library, until the process exits), and the
 * caller passes the device grid and a device buffer of `capacity` words for
 * the result.  On success *n_words holds the octree's word count and
 * center[3] its center; the words are byte-identical to svo_octree_build_dense.
 *   Limits: virtual side <= 256 and at most 262,144 occupied voxels;
 *   larger inputs, or an output buffer smaller than the octree (*n_words is
 *   still set), return SVO_ERR_LIMIT.
 *   The first call on a device looks up the arena's device address and
 *   keeps it for the process; make that first call before any stream capture
 *   on that device.  cudaDeviceReset between calls is not supported: the
 *   kept address would no longer be valid.
 *   All calls share the one arena, so calls that overlap on the GPU (from
 *   several host threads or streams at once) race and must be serialised by
 *   the caller.  The call returns after its work on `stream` is complete,
 *   on success and on error alike. */
int svo_octree_build_dense_noalloc(const uint32_t *d_grid, int w, int h, int d, uint64_t mem, uint32_t *d_words,
                                   uint64_t capacity, uint64_t *n_words, float center[3], svo_stream stream);

/* -------------------------------------------------------------- mesh build */

/* A triangle mesh on the current device: PlyLoader(const char *path)
 * (PlyLoader.cpp:66-79) after readVertices, rescaleVertices and
 * readTriangles (:122-224).  Vertex x y z [nx ny nz] [red green blue]
 * as FP32 (a missing colour channel is 255), polygons fan-triangulated,
 * flat face normals when the file has no normals. */
typedef struct svo_mesh svo_mesh;

/* Parses a PLY file (ascii, binary_little_endian or binary_big_endian, the
 * formats of the reference's plyfile reader, with its value conversions) on
 * the host and uploads the triangles.  SVO_ERR_FORMAT for a file the
 * reference cannot read (no vertex/face element, no vertex_indices), a face
 * index outside the vertex array or a non-finite vertex coordinate (the
 * reference's undefined cases); SVO_ERR_IO when the file cannot be read. */
int svo_mesh_load_ply(const char *path, svo_mesh **out);

/* The same from arrays: n_vertices positions (3 floats each), optional
 * normals and colours (3 floats each, NULL = absent / 255), and faces as
 * n_face_ints ints holding, per polygon, its vertex count then its indices. */
int svo_mesh_from_arrays(const float *positions, const float *normals, const float *colors, uint64_t n_vertices,
                         const int32_t *faces, uint64_t n_face_ints, svo_mesh **out);

/* Host only: the parse step of svo_mesh_load_ply, before rescaling.  On
 * success *positions, *colors (3 floats per vertex), *normals (3 floats per
 * vertex, or NULL when the file has none) and *triangles (3 indices per fan
 * triangle) are malloc'd arrays to release with svo_free; lower/upper are
 * PlyLoader's vertex bounds (PlyLoader.cpp:160-163). */
int svo_ply_parse(const char *path, float **positions, float **normals, float **colors, uint64_t *n_vertices,
                  int32_t **triangles, uint64_t *n_triangles, float lower[3], float upper[3]);

uint64_t svo_mesh_num_triangles(const svo_mesh *mesh);

/* PlyLoader::suggestedDimensions (PlyLoader.cpp:499-504): the volume
 * W, H, D for a side length. */
int svo_mesh_dimensions(const svo_mesh *mesh, int side, int dims[3]);

void svo_mesh_destroy(svo_mesh *mesh);

/* Replaces VoxelOctree(VoxelData *) over VoxelData(PlyLoader *, side, mem)
 * (VoxelData.cpp:50-56): the mesh voxelized on the GPU by the reference's
 * per-voxel triangle/box rule and running-average material blend, then the
 * octree built as svo_octree_build_dense does.  The reference's result
 * depends on its thread-pool size, which cuts each cache block into
 * `threads` sub-blocks with their own culled triangle lists
 * (PlyLoader.cpp:381-437), and on `mem`, which sets the cache block; both
 * are parameters here and the words match the reference's for the same
 * pair.  side in [5, 2^20].  Cache blocks are folded one after another
 * through one block buffer, as the reference does, only when a block's
 * dropped last slice lands in a later block's buffer volume, or when the
 * all-at-once form's scratch (16 bytes per cell of every brick a triangle
 * touches) would exceed half the free device memory; otherwise all blocks
 * are folded at once with no buffer.  Setting the environment
 * variable SVO_MESH_BLOCK_BUFFER=1 keeps the block-by-block path everywhere
 * (the words are the same; the tests run both). */
int svo_octree_build_mesh(const svo_mesh *mesh, int side, int threads, uint64_t mem, svo_stream stream,
                          svo_octree **out);

/* Replaces PlyLoader::convertToVolume(path, maxSize, memoryBudget)
 * (PlyLoader.cpp:506-534), the builder's --mode 1 (Main.cpp:312-324): the
 * mesh voxelized at suggestedDimensions(side) = w x h x d with a `threads`
 * thread pool's sub-block partition, written as a .voxel file (int32 w, h,
 * d, then w*h*d words, x fastest, 0 = empty) that svo_octree_build_voxel_file
 * and the reference's VoxelData(path, mem) read.  As the reference does,
 * the volume is processed in z-slabs of S = mem / (w*h) slices through one
 * w*h*S buffer (words and per-cell counts) that is never cleared between
 * slabs, so a cell blends with what the slab before left at the same place
 * and a slab with no triangles repeats the previous slab's words; each slab
 * contributes its first min(S, d - z) slices.  SVO_ERR_MEMORY when mem holds
 * no slice (the reference's ASSERT).  The reference's own
 * conversion stops with SIGFPE on x86-64: its progress line divides by a
 * block count only isBlockEmpty raises, which this path never calls.
 * svo_mesh_to_volume leaves the words in d_volume (device memory for the
 * w*h*d words of svo_mesh_dimensions); it works on `stream` and synchronises
 * it before returning, to read the conversion's error flags. */
int svo_mesh_to_volume(const svo_mesh *mesh, int side, int threads, uint64_t mem, uint32_t *d_volume,
                       svo_stream stream);
int svo_mesh_write_voxel_file(const svo_mesh *mesh, const char *path, int side, int threads, uint64_t mem,
                              svo_stream stream);

/* svo_mesh_load_ply + svo_octree_build_mesh + svo_mesh_destroy: the
 * builder's in-memory mode (Main.cpp -builder with a .ply input). */
int svo_octree_build_ply(const char *path, int side, int threads, uint64_t mem, svo_stream stream,
                         svo_octree **out);

/* ------------------------------------------------------------------- trace */

/* Per-ray outputs; any pointer may be NULL to skip that output.
 *   hit:   0 miss, 1 leaf hit, 2 level-of-detail exit (ray_scale > 0,
 *          VoxelOctree.cpp:265-268)
 *   t:     raymarch's t on a hit, +inf on a miss
 *   leaf:  index into the word array of the hit leaf's payload word
 *          (VoxelOctree.cpp:282), 0xFFFFFFFF when no leaf was hit
 *   word:  the leaf payload (raymarch's `normal` out-parameter), 0 when none
 *   rgb:   3 floats per ray, the viewer's shade() (Main.cpp:81-90) of the leaf
 *          word for the ray direction and `light`; 0 when no leaf was hit
 *   rgba8: the same colour as the viewer stores a traced pixel (renderTile,
 *          Main.cpp:126-131): c = uint32(min(shade, 1) * 255.0) with the
 *          product in double, packed c | c << 8 | c << 16 | 0xFF000000;
 *          0xFF000000 when no leaf was hit */
typedef struct svo_trace_out {
    uint8_t *hit;
    float *t;
    uint32_t *leaf;
    uint32_t *word;
    float *rgb;
    uint32_t *rgba8;
} svo_trace_out;

/* Replaces a loop of VoxelOctree::raymarch(o, d, rayScale, normal, t)
 * (VoxelOctree.cpp:207-346) over n rays, one GPU launch.  rays: 6 floats per
 * ray (ox, oy, oz, dx, dy, dz) in the octree's [1,2]^3 frame, d normalised
 * by the caller as in the reference; light: 3 floats (host memory).  All
 * array pointers are device pointers; asynchronous on `stream`. */
int svo_trace(const svo_octree *oct, const float *rays, uint64_t n, float ray_scale, const float light[3],
              const svo_trace_out *out, svo_stream stream);

/* Same as svo_trace with host arrays: rays are copied in and results out
 * through the handle's four staging buffers in chunks of about 4 M rays, on
 * internal copy-in, copy-out and per-buffer trace streams, so copies overlap
 * tracing.  Returns when results are on the host (after any work queued
 * earlier by the asynchronous forms below). */
int svo_trace_host(svo_octree *oct, const float *rays, uint64_t n, float ray_scale, const float light[3],
                   const svo_trace_out *out);

/* svo_trace for rays stored as a row-major width x height image: the same
 * per-ray results, traced by one persistent launch in 8x4-pixel tiles so a
 * warp's rays are neighbours (about 13% faster than svo_trace on camera rays).
 * Outputs are indexed y*width + x.  The launch uses a work counter owned by
 * the handle, so svo_trace_image calls on one handle that could overlap on
 * the GPU (different streams) must be ordered by the caller. */
int svo_trace_image(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height, float ray_scale,
                    const float light[3], const svo_trace_out *out, svo_stream stream);

/* svo_trace_image with host arrays, staged in chunks of whole rows with
 * copies overlapped with tracing.  Returns when results are on the host. */
int svo_trace_image_host(svo_octree *oct, const float *rays, uint32_t width, uint32_t height, float ray_scale,
                         const float light[3], const svo_trace_out *out);

/* No counterpart in the reference (whose raymarch is one blocking call per
 * ray).  svo_trace_host and svo_trace_image_host without the wait: the call
 * queues its copies and traces on the handle's host pipeline and returns.
 * Calls on one handle run in call order through that pipeline, so a second
 * call's input copies overlap the first call's traces.  The rays must stay
 * unchanged, and the outputs unread, until svo_octree_synchronize(oct)
 * returns; with page-locked host memory the copies run asynchronously, with
 * pageable memory the CUDA runtime stages them and the call returns later.
 * Traversal faults (corrupt octrees) are reported by svo_octree_synchronize. */
int svo_trace_host_async(svo_octree *oct, const float *rays, uint64_t n, float ray_scale, const float light[3],
                         const svo_trace_out *out);
int svo_trace_image_host_async(svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                               float ray_scale, const float light[3], const svo_trace_out *out);

/* Waits until every host trace queued on the handle (svo_trace_host_async,
 * svo_trace_image_host_async) has its results on the host. */
int svo_octree_synchronize(svo_octree *oct);

/* Device-side load counter for the roofline: for each ray, the number of
 * octree words the reference's raymarch reads (descriptor fetches at
 * VoxelOctree.cpp:254, far words at :279, the leaf word at :282).  Slower
 * than svo_trace; not for timing. */
int svo_trace_count_loads(const svo_octree *oct, const float *rays, uint64_t n, float ray_scale,
                          uint32_t *loads, svo_stream stream);

/* The viewer's frame, headless: renderBatch + renderTile (Main.cpp:92-202)
 * with its beam prepass.  The frame is cut into n_strips horizontal strips
 * as the viewer cuts it over its threads (NumThreads = 16, Main.cpp:47,
 * 349-361); per strip, level-of-detail corner rays every 8 pixels
 * (coarseScale = 16 / (planeDist * height)) bound each 8x8 tile's start
 * distance, tiles whose four corners all miss stay 0, and every other pixel
 * is traced from pos + dir * max(minT - 0.03, 0) and written as the
 * viewer's RGBA8 (0xFF000000 | grey * 0x010101).  pixel_stride 3 is the
 * viewer's half-size mode (renderHalfSize).  rot = the viewer's
 * INV_MODELVIEW rotation a11..a33 (row-major), pos = its camera position in
 * the octree frame (tform * 0 + center + 1, Main.cpp:145); the headlight is
 * derived from rot as the viewer does (:158).  rgba: width*height device
 * words, row-major.  Asynchronous on `stream`; rays that stop at a bounds
 * check set the handle's error word. */
int svo_render_frame(const svo_octree *oct, const float rot[9], const float pos[3], uint32_t width, uint32_t height,
                     uint32_t n_strips, uint32_t pixel_stride, uint32_t *rgba, svo_stream stream);

/* ---------------------------------------------------- differentiable shading */

/* No counterpart in the reference.  The viewer's shade() (Main.cpp:81-90)
 * with FP32 per-leaf parameters instead of the packed leaf word:
 *   n = p/|p| (p = leaf_normal[3*i..]),  rgb_k = c_k 0.9 |l.n| + 0.2 max(l.r, 0)^2,
 *   r = d - 2 (n.d) n,  c = leaf_rgb[3*i..],
 * for the leaf i a ray hits (i = the word index svo_trace reports as `leaf`;
 * the arrays hold 3 floats per octree word, only leaf entries are used).
 * Rays are a stack of n_views row-major images of width x height, all device
 * memory; view v (rows [v*height, (v+1)*height)) uses lights[3*v..] (device).
 *
 * svo_diff_forward traces every ray (the unchanged discrete raymarch) and
 * writes rgb (3 floats per ray, 0 on a miss) and, when hit_leaf != NULL, the
 * hit leaf's word index per ray (0xFFFFFFFF on a miss). */
int svo_diff_forward(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height, uint32_t n_views,
                     const float *lights, const float *leaf_rgb, const float *leaf_normal, uint32_t *hit_leaf,
                     float *rgb, svo_stream stream);

/* Adjoint of svo_diff_forward: adds dL/dleaf_rgb and dL/dleaf_normal for
 * the given dL/drgb (3 floats per ray) into grad_rgb / grad_normal (same
 * layout as the parameters; zero them first for a fresh gradient).  Hit
 * leaves come from hit_leaf, or, when hit_leaf == NULL, from re-tracing the
 * rays (no per-ray buffer kept between the passes).  Lanes of a warp hitting
 * the same leaf are summed in registers before one set of atomics per leaf;
 * the summation order across warps is not fixed. */
int svo_diff_backward(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height, uint32_t n_views,
                      const float *lights, const float *leaf_rgb, const float *leaf_normal, const uint32_t *hit_leaf,
                      const float *d_rgb, float *grad_rgb, float *grad_normal, svo_stream stream);

/* No counterpart in the reference.  svo_diff_backward for the L2 loss
 *   L = loss_scale / 2 * sum over rays and channels of (rgb - target)^2,
 * with dL/drgb = loss_scale (rgb - target) formed inside the adjoint from the
 * forward pass's rgb output (same parameters) and target (3 floats per ray,
 * device) instead of a d_rgb array.  Optional:
 *   loss_sum (device double): += sum of (rgb - target)^2 over all rays,
 *     misses included (their rgb is 0);
 *   touched / leaf_list / leaf_count (all or none): a record of the leaves
 *     that have received a gradient.  touched holds one bit per octree word
 *     ((n_words + 31) / 32 uint32, zeroed before the first call),
 *     leaf_list leaf_capacity >= n_words entries, leaf_count one uint32
 *     (zeroed with touched).  A leaf whose bit is clear gets its bit set and
 *     is appended to leaf_list; the record grows over calls and is what
 *     svo_adam_step_leaves updates. */
int svo_diff_backward_l2(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                         uint32_t n_views, const float *lights, const float *leaf_rgb, const float *leaf_normal,
                         const uint32_t *hit_leaf, const float *rgb, const float *target, float loss_scale,
                         float *grad_rgb, float *grad_normal, double *loss_sum, uint32_t *touched,
                         uint32_t *leaf_list, uint32_t *leaf_count, uint64_t leaf_capacity, svo_stream stream);

/* The same three calls with the leaves' parameters and gradients at
 * param_stride floats apart (>= 3) instead of 3: leaf i's colour is
 * leaf_rgb[param_stride*i ..], its normal leaf_normal[param_stride*i ..],
 * and the gradients are laid out the same way.  With param_stride = 8 and
 * leaf_normal = leaf_rgb + 3 (and grad_normal = grad_rgb + 3), a leaf's
 * colour and normal share one 32-byte record, so each gather and each
 * leaf's set of gradient atomics touches one memory sector instead of two;
 * svo_adam_step_leaves with width 8 then updates whole records (the two
 * unused floats get no gradient and stay as they are).  The results are
 * those of the 3-float layout. */
int svo_diff_forward_stride(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                            uint32_t n_views, const float *lights, const float *leaf_rgb, const float *leaf_normal,
                            uint32_t param_stride, uint32_t *hit_leaf, float *rgb, svo_stream stream);
int svo_diff_backward_stride(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                             uint32_t n_views, const float *lights, const float *leaf_rgb, const float *leaf_normal,
                             uint32_t param_stride, const uint32_t *hit_leaf, const float *d_rgb, float *grad_rgb,
                             float *grad_normal, svo_stream stream);
int svo_diff_backward_l2_stride(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                                uint32_t n_views, const float *lights, const float *leaf_rgb,
                                const float *leaf_normal, uint32_t param_stride, const uint32_t *hit_leaf,
                                const float *rgb, const float *target, float loss_scale, float *grad_rgb,
                                float *grad_normal, double *loss_sum, uint32_t *touched, uint32_t *leaf_list,
                                uint32_t *leaf_count, uint64_t leaf_capacity, svo_stream stream);

/* No counterpart in the reference.  One Adam step (no weight decay, no
 * amsgrad) over n parameters in one pass: exp_avg = beta1 exp_avg + (1 -
 * beta1) g, exp_avg_sq = beta2 exp_avg_sq + (1 - beta2) g^2, params -=
 * lr / (1 - beta1^step) * exp_avg / (sqrt(exp_avg_sq) / sqrt(1 - beta2^step)
 * + eps); with zero_grad != 0 the gradients are zeroed in the same pass for
 * the next svo_diff_backward accumulation.  All arrays are device memory;
 * asynchronous on `stream`.  step >= 1 counts this update. */
int svo_adam_step(float *params, float *grads, float *exp_avg, float *exp_avg_sq, uint64_t n, float lr, float beta1,
                  float beta2, float eps, int step, int zero_grad, svo_stream stream);

/* No counterpart in the reference.  svo_adam_step restricted to the leaves in
 * leaf_list (the first *leaf_count entries, at most leaf_capacity; the count
 * is read on the device): values [leaf*width, leaf*width + width) of each
 * array, n_values in all.  When the list holds every leaf that has ever had
 * a gradient (svo_diff_backward_l2's record) and the moments started at
 * zero, the results are identical to svo_adam_step over all n_values: an
 * unlisted value has g = m = v = 0, which the dense update leaves as it is. */
int svo_adam_step_leaves(float *params, float *grads, float *exp_avg, float *exp_avg_sq, uint64_t n_values,
                         uint32_t width, const uint32_t *leaf_list, const uint32_t *leaf_count,
                         uint64_t leaf_capacity, float lr, float beta1, float beta2, float eps, int step,
                         int zero_grad, svo_stream stream);

/* ----------------------------------------------------------------- batched */

/* One (octree, view) pair of a batched trace.  A view is either
 *   - an image: width x height pixels, rays from `rays` (device, row-major
 *     width*height records) or, when rays == NULL, generated in the kernel
 *     from `camera` with the viewer's formula (Main.cpp:149-176):
 *     camera = {a11..a33 (row-major rotation), px, py, pz (position),
 *     2/width, height/width, zx, zy, zz} with (zx, zy, zz) = (a13, a23, a33)
 *     / tan(pi/6); outputs are indexed y*width + x;
 *   - or linear: width == 0, n_rays rays from `rays`, outputs by ray index.
 * Each view has its own ray_scale, light and device outputs. */
typedef struct svo_view {
    const svo_octree *octree;
    const float *rays;
    uint64_t n_rays;
    uint32_t width, height;
    float camera[17];
    float ray_scale;
    float light[3];
    svo_trace_out out;
} svo_view;

/* Launch shape of the persistent traversal kernel (see svo_batch_autotune). */
typedef struct svo_trace_config {
    int block_threads;   /* threads per CTA, multiple of 32, <= 1024 */
    int blocks_per_sm;   /* persistent grid = SM count x blocks_per_sm */
    int refill_idle;     /* a warp refills its idle lanes once this many (1..32) are idle; 0 = no
                            refill: a warp takes its next 32 slots once all its lanes finish */
    int steps_per_round; /* traversal steps between refill checks */
    int tile_w;          /* image tile width in pixels: 4, 8, 16 or 32 (tile = tile_w x 32/tile_w) */
    int chunk;           /* ray slots a warp takes from the work queue at once (multiple of 32) */
    int cache_entries;   /* descriptor-table entries (the top levels) of its current octree each warp
                            keeps in shared memory: 0 = none, else a multiple of 32 up to 512, at most
                            64 KB per CTA; plain-tile schedule (refill_idle 0) over tables only */
    int reg_cap;         /* lane-refill kernel build: 0 = default (64 registers per thread, 4 CTAs of 256
                            per SM), 48 = at most 48 registers (5 CTAs, a few spilled values) */
} svo_trace_config;

typedef struct svo_batch svo_batch;

/* No counterpart in the reference (its viewer renders one octree per frame
 * on host threads, Main.cpp:139-262).  Records the views and uploads the job
 * table; the octrees and output buffers must outlive the batch. */
int svo_batch_create(const svo_view *views, int n_views, svo_batch **out);
int svo_batch_default_config(svo_trace_config *cfg);
/* Number of work-queue slots (rays plus padding of partial pixel tiles). */
int svo_batch_num_slots(svo_batch *b, uint64_t *slots);
/* One persistent launch over every view (asynchronous on `stream`). */
int svo_batch_trace(svo_batch *b, const svo_trace_config *cfg, svo_stream stream);
/* Captures the queue reset and the launch into a CUDA graph owned by the
 * batch; svo_batch_launch_graph replays it on any stream. */
int svo_batch_capture_graph(svo_batch *b, const svo_trace_config *cfg);
int svo_batch_launch_graph(svo_batch *b, svo_stream stream);
/* Times candidate launch shapes (block size, refill threshold, steps per
 * round, tile width, rays per queue access, table cache depth, register
 * budget) on this batch and returns the fastest; results are
 * cached per device and workload in a JSON-lines file ($SVO_AUTOTUNE_CACHE,
 * default ~/.cache/svo_gb300_autotune.jsonl; SVO_AUTOTUNE_FORCE=1 re-times).
 * *best_ms is -1 when the cache answered.  Synchronises `stream`. */
int svo_batch_autotune(svo_batch *b, svo_trace_config *best, float *best_ms, svo_stream stream);
/* Reads and clears the batch's device error word (as svo_octree_device_status). */
int svo_batch_status(svo_batch *b, uint32_t *flags);
int svo_batch_destroy(svo_batch *b);

#ifdef __cplusplus
}
#endif

#endif /* SVO_GB300_H */
