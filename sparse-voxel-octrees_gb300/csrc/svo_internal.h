// svo_internal.h — host-side internals shared by the library's translation units.
#pragma once

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "svo.h"

// The opaque handle behind svo_octree*.
struct svo_octree {
    uint32_t *d_words = nullptr;  // resident octree words (HBM)
    uint64_t n_words = 0;
    float center[3] = {0.0f, 0.0f, 0.0f};
    int device = 0;
    // One device control block: kQueues work counters, then d_status.
    uint32_t *d_status = nullptr;  // device error word: bit 0 = a ray ended with kFault
    unsigned long long *d_queue = nullptr;  // work counters: [0] svo_trace_image and the differentiable
                                            // launches, [1 + b] svo_trace_image_host's trace stream b
    int index_bits = 32;  // 64: svo_trace uses 64-bit word indices even when n_words fits 32 bits

    // Descriptor table of the table traversal (octree_table.cu), built by the
    // first trace call that can use it; a cache of the immutable words.
    mutable uint4 *d_tab = nullptr;
    mutable uint64_t n_tab = 0;
    mutable std::atomic<int> tab_state{0};  // 0 not built yet, 1 built, -1 the octree does not qualify
    bool use_table = true;
    mutable std::mutex tab_mtx;

    // Host-buffer pipeline of svo_trace_host and svo_trace_image_host: one
    // device staging arena split into kStageBuffers buffers, a copy-in and a
    // copy-out stream, one trace stream per buffer, and per-buffer events
    // (inputs landed, trace done, outputs copied).
    static constexpr int kStageBuffers = 4;  // stage_used has one flag per buffer
    static constexpr int kQueues = 1 + kStageBuffers;
    std::mutex staging_mtx;
    void *stage_dev = nullptr;
    size_t stage_dev_bytes = 0;
    uint64_t stage_cap = 0;       // rays per staging buffer (the arena's layout)
    uint64_t stage_seq = 0;       // chunks enqueued so far: chunk k uses buffer k % kStageBuffers
    bool stage_used[4] = {};      // the buffer holds an earlier chunk (its events are waited on)
    bool stage_pending = false;   // enqueued work not yet drained (svo_octree_synchronize)
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaStream_t stage_trace[kStageBuffers] = {};
    cudaEvent_t stage_in[kStageBuffers] = {}, stage_traced[kStageBuffers] = {}, stage_out[kStageBuffers] = {};
};

namespace svo {

// Octrees above 2^32-1 words need 64-bit word indices: far offsets then carry
// bits above 32 in the descriptor's top 14 bits (VoxelOctree.cpp:190-194).
constexpr uint64_t kMaxNarrowWords = 0xFFFFFFFFull;
inline bool wide_octree(const svo_octree *o) { return o->n_words > kMaxNarrowWords; }

// Records a formatted message for svo_last_error() and returns `code`.
int set_error(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
void clear_error();

#define SVO_CUDA_TRY(call)                                   \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return ::svo::cuda_fail(_e, #call); \
    } while (0)

// LZ4 block format (independent blocks; decoder accepts history before pos0).
size_t lz4_compress_bound(size_t n);
size_t lz4_compress_block(const uint8_t *src, size_t n, uint8_t *dst, size_t cap);
int lz4_decompress_block(const uint8_t *src, size_t src_len, uint8_t *out, size_t pos0, size_t out_len);

// Stream-ordered scratch from the library's per-device pool (mem_pool.cpp);
// release with cudaFreeAsync.
cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t st);

// VoxelData::init cache-block search (VoxelData.cpp:211-244): log2 of the
// cache-block edge, or -1 when no partition fits `mem`.
int cache_block_log2(int w, int h, int d, uint64_t mem, uint64_t cell_cost);

// GPU build from a device-resident dense grid (build.cu).  On success the
// caller owns *d_words (cudaFree).
int build_dense_device(const uint32_t *d_grid, int w, int h, int d, int log_side, int log_block, cudaStream_t st,
                       uint32_t **d_words, uint64_t *n_words);

// Phases 2-3 of the build (build.cu) from voxels already in ascending Morton
// order: d_keys are Morton codes over a 2^log_side cube, d_payload the leaf
// words.  d_topflag (one byte per cache block, Morton-indexed) is required
// when log_block < log_side and marks blocks that exist without children.
int build_from_sorted_device(const uint64_t *d_keys, const uint32_t *d_payload, uint64_t n, int log_side,
                             int log_block, const uint8_t *d_topflag, cudaStream_t st, uint32_t **d_words,
                             uint64_t *n_words);

// The .voxel build streamed in z slabs of about slab_bytes (voxel_stream.cu);
// fp is positioned after the 12-byte header.
int build_voxel_file_streamed(FILE *fp, int w, int h, int d, uint64_t mem, uint64_t slab_bytes, cudaStream_t st,
                              uint32_t **d_words, uint64_t *n_words, float center[3]);

// Trace launchers (trace.cu).
int launch_trace(const svo_octree *oct, const float *d_rays, uint64_t n, float ray_scale, const float light[3],
                 const svo_trace_out &out, cudaStream_t st);
int launch_trace_image(const svo_octree *oct, const float *d_rays, uint32_t width, uint32_t height, float ray_scale,
                       const float light[3], const svo_trace_out &out, cudaStream_t st, int queue = 0);
int launch_count_loads(const svo_octree *oct, const float *d_rays, uint64_t n, float ray_scale, uint32_t *loads,
                       cudaStream_t st);

// Creates a handle around device words (takes ownership).
int make_handle(uint32_t *d_words, uint64_t n_words, const float center[3], svo_octree **out);

// The handle's descriptor table (octree_table.cu), built on first use; null
// when the octree does not qualify (over 2^32-1 words, or a reachable node
// that fails the checks), when the table is switched off, or while `caller`
// is being captured into a graph.  Synchronous the first time.
const uint4 *octree_table(const svo_octree *oct, cudaStream_t caller);

}  // namespace svo
