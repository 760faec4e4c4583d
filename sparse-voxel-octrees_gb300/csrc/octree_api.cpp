// octree_api.cpp — the C ABI (include/svo.h): handle lifetime, .oct and
// .voxel I/O, build and trace entry points, validation, errors.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <functional>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "svo_internal.h"

namespace svo {

namespace {
thread_local std::string g_last_error;
constexpr uint64_t kOctBlock = 64ull * 1024 * 1024;  // VoxelOctree.cpp:55
constexpr uint64_t kStageRays = 1ull << 22;          // rays per staging chunk
}  // namespace

int set_error(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return set_error(SVO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

void clear_error() { g_last_error.clear(); }

// Util.hpp:102-106
static int round_to_pow2(int x) {
    int y;
    for (y = 1; y < x; y *= 2) {
    }
    return y;
}

static int log2_exact(uint64_t v) {
    int r = 0;
    while ((1ull << r) < v) ++r;
    return r;
}

static uint64_t pyramid_cells(int levels) {  // VoxelData.cpp:65-74
    uint64_t r = 0, s = 1;
    for (int i = 0; i < levels; ++i) {
        r += s;
        s *= 8;
    }
    return r;
}

int cache_block_log2(int w, int h, int d, uint64_t mem, uint64_t cell_cost) {
    int side = std::max(round_to_pow2(w), std::max(round_to_pow2(h), round_to_pow2(d)));
    int hb = log2_exact((uint64_t)side);
    int largest = -1;
    for (int i = hb; i >= 0; --i) {  // VoxelData.cpp:221-235
        int low = hb - i;
        uint64_t cost = pyramid_cells(i + 1) + pyramid_cells(low) + ((uint64_t)1 << (uint64_t)(low * 3)) * cell_cost;
        if (cost < mem) largest = hb - i;
    }
    return largest;
}

}  // namespace svo
extern "C" int svo_octree_destroy(svo_octree *oct);
namespace svo {

int make_handle(uint32_t *d_words, uint64_t n_words, const float center[3], svo_octree **out) {
    std::unique_ptr<svo_octree> h(new svo_octree());
    h->d_words = d_words;
    h->n_words = n_words;
    std::memcpy(h->center, center, sizeof(h->center));
    cudaGetDevice(&h->device);
    // One control block: the work counters, then the error word.
    const size_t ctrl_bytes = svo_octree::kQueues * sizeof(unsigned long long) + 8;
    void *ctrl = nullptr;
    cudaError_t e = cudaMalloc(&ctrl, ctrl_bytes);
    if (e != cudaSuccess) {
        cudaFree(d_words);
        h->d_words = nullptr;
        return cuda_fail(e, "cudaMalloc(control block)");
    }
    h->d_queue = static_cast<unsigned long long *>(ctrl);
    h->d_status = reinterpret_cast<uint32_t *>(static_cast<char *>(ctrl) +
                                               svo_octree::kQueues * sizeof(unsigned long long));
    e = cudaMemset(ctrl, 0, ctrl_bytes);
    if (e != cudaSuccess) {
        svo_octree_destroy(h.release());
        return cuda_fail(e, "cudaMemset(control block)");
    }
    *out = h.release();
    return SVO_OK;
}

static int upload_words(const uint32_t *words, uint64_t n, const float center[3], svo_octree **out) {
    if (n == 0) return set_error(SVO_ERR_FORMAT, "octree has no words");
    uint32_t *d = nullptr;
    SVO_CUDA_TRY(cudaMalloc((void **)&d, n * sizeof(uint32_t)));
    cudaError_t e = cudaMemcpy(d, words, n * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "upload octree words");
    }
    return make_handle(d, n, center, out);
}

static int ensure_staging(svo_octree *oct, size_t dev_bytes) {
    if (oct->stage_dev_bytes >= dev_bytes) return SVO_OK;
    if (oct->stage_dev) cudaFree(oct->stage_dev);
    oct->stage_dev = nullptr;
    oct->stage_dev_bytes = 0;
    SVO_CUDA_TRY(cudaMalloc(&oct->stage_dev, dev_bytes));
    oct->stage_dev_bytes = dev_bytes;
    return SVO_OK;
}

static int check_device_status(const svo_octree *oct) {
    uint32_t flags = 0;
    SVO_CUDA_TRY(cudaMemcpy(&flags, oct->d_status, sizeof(flags), cudaMemcpyDeviceToHost));
    if (flags) {
        cudaMemset(oct->d_status, 0, sizeof(uint32_t));
        return set_error(SVO_ERR_DEVICE, "a ray hit the traversal step cap or an out-of-range word index "
                                         "(corrupt octree?)");
    }
    return SVO_OK;
}

// Chunk plan (in units of rays or rows) for the host pipelines: chunks of
// `target` rounded down to a multiple of `align`, the remainder last.  Both
// directions of the host link are busy in the steady state, so the copies,
// not the traces, bound a call; shorter chunks at the ends (to shorten the
// unoverlapped first copy-in and last copy-out) measured slower on GB300.
// Results do not depend on the plan: every ray is traced on its own.
static std::vector<uint64_t> plan_chunks(uint64_t total, uint64_t target, uint64_t align) {
    const uint64_t t = std::max(align, target / align * align);
    std::vector<uint64_t> plan;
    for (uint64_t s = 0; s < total; s += t) plan.push_back(std::min(t, total - s));
    return plan;
}

// The host-buffer pipeline of svo_trace_host and svo_trace_image_host (and
// their asynchronous forms).  Chunk k's rays go in on the copy-in stream into
// staging buffer k % B, are traced on that buffer's trace stream (each with
// its own work counter, so one chunk's persistent launch fills the tail of the
// previous one) and come out on the copy-out stream.  A buffer's rays are
// overwritten only after its previous trace, and its results only after their
// copy-out.  With two buffers a buffer's whole cycle (copy in, trace, copy
// out) paced the copy-in stream; with four, the copy-in stream runs back to
// back, which the host link's transfer rate then bounds.  The chunk counter
// carries over from call to call, so an asynchronous call's copies queue
// behind the previous call's and overlap its traces.
//
// Waits for every enqueued chunk, then reports traversal faults.  Called with
// staging_mtx held.
static int host_drain(svo_octree *oct) {
    if (!oct->stage_pending) return SVO_OK;
    cudaError_t e = cudaSuccess;
    auto drain = [&](cudaStream_t q) {
        const cudaError_t eq = cudaStreamSynchronize(q);
        if (e == cudaSuccess) e = eq;
    };
    drain(oct->copy_in);
    for (int k = 0; k < svo_octree::kStageBuffers; ++k) drain(oct->stage_trace[k]);
    drain(oct->copy_out);
    oct->stage_pending = false;
    if (e != cudaSuccess) return cuda_fail(e, "host trace pipeline");
    return check_device_status(oct);
}

// Enqueues the chunks of `plan` (rays from `rays`, results to `out`, all host
// memory); launch(d_rays, rays, outputs, stream, buffer) enqueues one chunk's
// trace.  Called with staging_mtx held.  On an error, everything enqueued so
// far is drained before returning.
template <typename Launch>
static int host_enqueue(svo_octree *oct, const float *rays, const std::vector<uint64_t> &plan,
                        const svo_trace_out &out, Launch launch) {
    constexpr int B = svo_octree::kStageBuffers;
    uint64_t need = 0;
    for (uint64_t m : plan) need = std::max(need, m);
    // Per buffer: rays 24 B, hit 1, t 4, leaf 4, word 4, rgb 12, rgba8 4 (256-byte aligned arrays).
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    auto buf_bytes = [&](uint64_t C) { return al(C * 24) + al(C) + al(C * 4) * 4 + al(C * 12); };
    if (need > oct->stage_cap) {
        // a larger arena: nothing may still be using the old one
        int rc = host_drain(oct);
        if (rc) return rc;
        rc = ensure_staging(oct, B * buf_bytes(need));
        if (rc) return rc;
        oct->stage_cap = need;
        for (bool &u : oct->stage_used) u = false;
    }
    const uint64_t C = oct->stage_cap;
    const size_t buf = buf_bytes(C);
    if (!oct->copy_in) {
        SVO_CUDA_TRY(cudaStreamCreateWithFlags(&oct->copy_in, cudaStreamNonBlocking));
        SVO_CUDA_TRY(cudaStreamCreateWithFlags(&oct->copy_out, cudaStreamNonBlocking));
        for (int k = 0; k < B; ++k) {
            SVO_CUDA_TRY(cudaStreamCreateWithFlags(&oct->stage_trace[k], cudaStreamNonBlocking));
            SVO_CUDA_TRY(cudaEventCreateWithFlags(&oct->stage_in[k], cudaEventDisableTiming));
            SVO_CUDA_TRY(cudaEventCreateWithFlags(&oct->stage_traced[k], cudaEventDisableTiming));
            SVO_CUDA_TRY(cudaEventCreateWithFlags(&oct->stage_out[k], cudaEventDisableTiming));
        }
    }
    cudaStream_t si = oct->copy_in, so = oct->copy_out;
    oct->stage_pending = true;
    auto enqueue = [&]() -> int {
        uint64_t c0 = 0;
        for (size_t j = 0; j < plan.size(); c0 += plan[j], ++j) {
            const int h = (int)(oct->stage_seq++ % (uint64_t)B);
            const bool reused = oct->stage_used[h];
            oct->stage_used[h] = true;
            const uint64_t m = plan[j];
            cudaStream_t sk = oct->stage_trace[h];
            uint8_t *base = (uint8_t *)oct->stage_dev + h * buf;
            float *d_rays = (float *)base;
            uint8_t *d_hit = base + al(C * 24);
            float *d_t = (float *)(d_hit + al(C));
            uint32_t *d_leaf = (uint32_t *)((uint8_t *)d_t + al(C * 4));
            uint32_t *d_word = (uint32_t *)((uint8_t *)d_leaf + al(C * 4));
            float *d_rgb = (float *)((uint8_t *)d_word + al(C * 4));
            uint32_t *d_rgba8 = (uint32_t *)((uint8_t *)d_rgb + al(C * 12));
            if (reused) SVO_CUDA_TRY(cudaStreamWaitEvent(si, oct->stage_traced[h], 0));
            SVO_CUDA_TRY(cudaMemcpyAsync(d_rays, rays + 6 * c0, m * 24, cudaMemcpyHostToDevice, si));
            SVO_CUDA_TRY(cudaEventRecord(oct->stage_in[h], si));
            SVO_CUDA_TRY(cudaStreamWaitEvent(sk, oct->stage_in[h], 0));
            if (reused) SVO_CUDA_TRY(cudaStreamWaitEvent(sk, oct->stage_out[h], 0));
            svo_trace_out o;
            o.hit = out.hit ? d_hit : nullptr;
            o.t = out.t ? d_t : nullptr;
            o.leaf = out.leaf ? d_leaf : nullptr;
            o.word = out.word ? d_word : nullptr;
            o.rgb = out.rgb ? d_rgb : nullptr;
            o.rgba8 = out.rgba8 ? d_rgba8 : nullptr;
            int rc = launch(d_rays, m, o, sk, h);
            if (rc) return rc;
            SVO_CUDA_TRY(cudaEventRecord(oct->stage_traced[h], sk));
            SVO_CUDA_TRY(cudaStreamWaitEvent(so, oct->stage_traced[h], 0));
            if (out.hit) SVO_CUDA_TRY(cudaMemcpyAsync(out.hit + c0, d_hit, m, cudaMemcpyDeviceToHost, so));
            if (out.t) SVO_CUDA_TRY(cudaMemcpyAsync(out.t + c0, d_t, m * 4, cudaMemcpyDeviceToHost, so));
            if (out.leaf) SVO_CUDA_TRY(cudaMemcpyAsync(out.leaf + c0, d_leaf, m * 4, cudaMemcpyDeviceToHost, so));
            if (out.word) SVO_CUDA_TRY(cudaMemcpyAsync(out.word + c0, d_word, m * 4, cudaMemcpyDeviceToHost, so));
            if (out.rgb) SVO_CUDA_TRY(cudaMemcpyAsync(out.rgb + 3 * c0, d_rgb, m * 12, cudaMemcpyDeviceToHost, so));
            if (out.rgba8)
                SVO_CUDA_TRY(cudaMemcpyAsync(out.rgba8 + c0, d_rgba8, m * 4, cudaMemcpyDeviceToHost, so));
            SVO_CUDA_TRY(cudaEventRecord(oct->stage_out[h], so));
        }
        return SVO_OK;
    };
    const int rc = enqueue();
    if (rc) {
        // Every stream is drained when a chunk failed to enqueue: the staging
        // buffers must be idle before the next call reuses them.  The error
        // recorded by the failed step is the one reported.
        oct->stage_pending = true;
        for (cudaStream_t q : {si, so}) cudaStreamSynchronize(q);
        for (int k = 0; k < B; ++k) cudaStreamSynchronize(oct->stage_trace[k]);
        oct->stage_pending = false;
    }
    return rc;
}

}  // namespace svo

using namespace svo;

extern "C" {

const char *svo_last_error(void) { return g_last_error.c_str(); }

int svo_version(void) { return 100; }

void svo_free(void *p) { free(p); }

// .oct read: the file is mapped, its block table indexed, and the blocks
// decoded on worker threads straight into the word array.  Blocks written by
// svo_oct_write are independent; the reference writes with
// LZ4_compress_continue (VoxelOctree.cpp:96-119), whose blocks may copy from
// the previous 64 KiB of output, so a block that reaches back fails its
// independent attempt and is decoded afterwards, in order, with that history.
int svo_oct_read(const char *path, uint32_t **words_out, uint64_t *n_out, float center[3]) {
    if (!path || !words_out || !n_out || !center) return set_error(SVO_ERR_INVALID, "null argument");
    int fd = open(path, O_RDONLY);
    if (fd < 0) return set_error(SVO_ERR_IO, "cannot open %s", path);
    struct stat st;
    if (fstat(fd, &st) != 0) {
        close(fd);
        return set_error(SVO_ERR_IO, "cannot size %s", path);
    }
    const size_t fsize = (size_t)st.st_size;
    if (fsize < 20) {
        close(fd);
        return set_error(SVO_ERR_FORMAT, "%s: truncated header", path);
    }
    void *mp = mmap(nullptr, fsize, PROT_READ, MAP_PRIVATE, fd, 0);
    close(fd);
    if (mp == MAP_FAILED) return set_error(SVO_ERR_IO, "cannot map %s", path);
    std::unique_ptr<void, std::function<void(void *)>> mguard(mp, [fsize](void *q) { munmap(q, fsize); });
    const uint8_t *file = (const uint8_t *)mp;
    uint64_t n = 0;
    std::memcpy(center, file, 12);
    std::memcpy(&n, file + 12, 8);
    if (n == 0 || n > (1ull << 36))
        return set_error(n ? SVO_ERR_LIMIT : SVO_ERR_FORMAT, "%s: unsupported word count %llu", path,
                         (unsigned long long)n);
    struct Block {
        size_t src;
        uint64_t csize, off, len;
    };
    std::vector<Block> blocks;
    size_t pos = 20;
    for (uint64_t off = 0; off < n * 4; off += kOctBlock) {
        uint64_t csize = 0;
        if (fsize - pos < 8) return set_error(SVO_ERR_FORMAT, "%s: truncated block header", path);
        std::memcpy(&csize, file + pos, 8);
        pos += 8;
        if (csize > lz4_compress_bound(kOctBlock)) return set_error(SVO_ERR_FORMAT, "%s: bad block size", path);
        if (fsize - pos < csize) return set_error(SVO_ERR_FORMAT, "%s: truncated block", path);
        blocks.push_back({pos, csize, off, std::min<uint64_t>(n * 4 - off, kOctBlock)});
        pos += csize;
    }
    uint32_t *words = (uint32_t *)malloc(n * sizeof(uint32_t));
    if (!words) return set_error(SVO_ERR_MEMORY, "cannot allocate %llu words", (unsigned long long)n);
    std::unique_ptr<uint32_t, void (*)(void *)> wguard(words, free);
    uint8_t *dst = reinterpret_cast<uint8_t *>(words);
    // independent attempts in parallel (no history: pos0 = 0 at the block start)
    std::vector<uint8_t> done(blocks.size(), 0);
    std::atomic<size_t> next{0};
    const unsigned nt = std::max(1u, std::min<unsigned>(std::min(std::thread::hardware_concurrency(), 16u),
                                                        (unsigned)blocks.size()));
    auto worker = [&] {
        for (size_t k; (k = next.fetch_add(1)) < blocks.size();) {
            const Block &b = blocks[k];
            done[k] = lz4_decompress_block(file + b.src, b.csize, dst + b.off, 0, b.len) == 0;
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
    // the rest in order, each with the preceding output as history
    for (size_t k = 0; k < blocks.size(); ++k) {
        if (done[k]) continue;
        const Block &b = blocks[k];
        const uint64_t hist = std::min<uint64_t>(b.off, 64 * 1024);
        if (lz4_decompress_block(file + b.src, b.csize, dst + b.off - hist, hist, b.len) != 0)
            return set_error(SVO_ERR_FORMAT, "%s: corrupt LZ4 block at payload offset %llu", path,
                             (unsigned long long)b.off);
    }
    *words_out = wguard.release();
    *n_out = n;
    return SVO_OK;
}

int svo_oct_write(const char *path, const uint32_t *words, uint64_t n_words, const float center[3]) {
    if (!path || !words || !center || n_words == 0) return set_error(SVO_ERR_INVALID, "bad argument");
    const uint64_t bytes = n_words * 4;
    const uint64_t nblocks = (bytes + kOctBlock - 1) / kOctBlock;
    // Blocks are independent, so they compress in parallel.
    std::vector<std::vector<uint8_t>> comp(nblocks);
    std::vector<size_t> csize(nblocks, 0);
    auto work = [&](uint64_t b) {
        uint64_t off = b * kOctBlock;
        size_t len = (size_t)std::min<uint64_t>(bytes - off, kOctBlock);
        comp[b].resize(lz4_compress_bound(len));
        csize[b] = lz4_compress_block(reinterpret_cast<const uint8_t *>(words) + off, len, comp[b].data(),
                                      comp[b].size());
    };
    unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)nblocks));
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t)
        pool.emplace_back([&, t] {
            for (uint64_t b = t; b < nblocks; b += nt) work(b);
        });
    for (auto &th : pool) th.join();
    FILE *fp = fopen(path, "wb");
    if (!fp) return set_error(SVO_ERR_IO, "cannot create %s", path);
    std::unique_ptr<FILE, int (*)(FILE *)> guard(fp, fclose);
    bool ok = fwrite(center, sizeof(float), 3, fp) == 3 && fwrite(&n_words, sizeof(uint64_t), 1, fp) == 1;
    for (uint64_t b = 0; ok && b < nblocks; ++b) {
        uint64_t cs = csize[b];
        ok = fwrite(&cs, sizeof(uint64_t), 1, fp) == 1 && fwrite(comp[b].data(), 1, cs, fp) == cs;
    }
    if (!ok) return set_error(SVO_ERR_IO, "write to %s failed", path);
    return SVO_OK;
}

int svo_octree_load(const char *path, svo_octree **out) {
    if (!path || !out) return set_error(SVO_ERR_INVALID, "null argument");
    uint32_t *words = nullptr;
    uint64_t n = 0;
    float center[3];
    int rc = svo_oct_read(path, &words, &n, center);
    if (rc) return rc;
    std::unique_ptr<uint32_t, void (*)(void *)> wguard(words, free);
    return upload_words(words, n, center, out);
}

int svo_octree_save(const svo_octree *oct, const char *path) {
    if (!oct || !path) return set_error(SVO_ERR_INVALID, "null argument");
    std::vector<uint32_t> words(oct->n_words);
    SVO_CUDA_TRY(cudaMemcpy(words.data(), oct->d_words, oct->n_words * 4, cudaMemcpyDeviceToHost));
    return svo_oct_write(path, words.data(), oct->n_words, oct->center);
}

int svo_octree_from_words(const uint32_t *words, uint64_t n_words, const float center[3], svo_octree **out) {
    if (!words || !center || !out) return set_error(SVO_ERR_INVALID, "null argument");
    return upload_words(words, n_words, center, out);
}

int svo_octree_destroy(svo_octree *oct) {
    if (!oct) return SVO_OK;
    if (oct->stage_pending) {  // asynchronous host traces still reading and writing the staging arena
        std::lock_guard<std::mutex> lock(oct->staging_mtx);
        host_drain(oct);
    }
    if (oct->d_words) cudaFree(oct->d_words);
    if (oct->d_tab) cudaFree(oct->d_tab);
    if (oct->d_queue) cudaFree(oct->d_queue);  // the control block (d_status lies inside it)
    if (oct->stage_dev) cudaFree(oct->stage_dev);
    if (oct->copy_in) cudaStreamDestroy(oct->copy_in);
    if (oct->copy_out) cudaStreamDestroy(oct->copy_out);
    for (int k = 0; k < svo_octree::kStageBuffers; ++k) {
        if (oct->stage_trace[k]) cudaStreamDestroy(oct->stage_trace[k]);
        if (oct->stage_in[k]) cudaEventDestroy(oct->stage_in[k]);
        if (oct->stage_traced[k]) cudaEventDestroy(oct->stage_traced[k]);
        if (oct->stage_out[k]) cudaEventDestroy(oct->stage_out[k]);
    }
    delete oct;
    return SVO_OK;
}

int svo_octree_num_words(const svo_octree *oct, uint64_t *n) {
    if (!oct || !n) return set_error(SVO_ERR_INVALID, "null argument");
    *n = oct->n_words;
    return SVO_OK;
}

int svo_octree_set_index_width(svo_octree *oct, int bits) {
    if (!oct) return set_error(SVO_ERR_INVALID, "null argument");
    if (bits != 32 && bits != 64) return set_error(SVO_ERR_INVALID, "index width %d is neither 32 nor 64", bits);
    if (bits == 32 && wide_octree(oct))
        return set_error(SVO_ERR_LIMIT, "an octree of %llu words needs 64-bit word indices",
                         (unsigned long long)oct->n_words);
    oct->index_bits = bits;
    return SVO_OK;
}

int svo_octree_set_table(svo_octree *oct, int enable) {
    if (!oct) return set_error(SVO_ERR_INVALID, "null argument");
    oct->use_table = enable != 0;
    return SVO_OK;
}

int svo_octree_table_size(svo_octree *oct, uint64_t *entries) {
    if (!oct || !entries) return set_error(SVO_ERR_INVALID, "null argument");
    const bool was = oct->use_table;
    oct->use_table = true;
    const uint4 *t = octree_table(oct, nullptr);
    oct->use_table = was;
    *entries = t ? oct->n_tab : 0;
    return SVO_OK;
}

int svo_octree_copy_words(const svo_octree *oct, uint32_t *dst, uint64_t n) {
    if (!oct || !dst) return set_error(SVO_ERR_INVALID, "null argument");
    if (n != oct->n_words) return set_error(SVO_ERR_INVALID, "destination holds %llu words, octree has %llu",
                                            (unsigned long long)n, (unsigned long long)oct->n_words);
    SVO_CUDA_TRY(cudaMemcpy(dst, oct->d_words, n * 4, cudaMemcpyDeviceToHost));
    return SVO_OK;
}

int svo_octree_device_words(const svo_octree *oct, const uint32_t **d_words) {
    if (!oct || !d_words) return set_error(SVO_ERR_INVALID, "null argument");
    *d_words = oct->d_words;
    return SVO_OK;
}

int svo_octree_center(const svo_octree *oct, float center[3]) {
    if (!oct || !center) return set_error(SVO_ERR_INVALID, "null argument");
    std::memcpy(center, oct->center, sizeof(oct->center));
    return SVO_OK;
}

int svo_octree_device_status(svo_octree *oct, uint32_t *flags) {
    if (!oct || !flags) return set_error(SVO_ERR_INVALID, "null argument");
    SVO_CUDA_TRY(cudaMemcpy(flags, oct->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    SVO_CUDA_TRY(cudaMemset(oct->d_status, 0, sizeof(uint32_t)));
    return SVO_OK;
}

int svo_octree_validate(const svo_octree *oct, uint64_t *n_desc, uint64_t *n_leaves) {
    if (!oct) return set_error(SVO_ERR_INVALID, "null argument");
    const uint64_t n = oct->n_words;
    std::vector<uint32_t> w(n);
    SVO_CUDA_TRY(cudaMemcpy(w.data(), oct->d_words, n * 4, cudaMemcpyDeviceToHost));
    // Iterative walk: (descriptor index, depth).  Child blocks always follow
    // their parent (offset >= 1), so the walk terminates.
    std::vector<std::pair<uint64_t, int>> stack;
    stack.push_back({0, 0});
    uint64_t nd = 0, nl = 0;
    while (!stack.empty()) {
        uint64_t p = stack.back().first;
        int depth = stack.back().second;
        stack.pop_back();
        if (p >= n) return set_error(SVO_ERR_FORMAT, "descriptor index %llu out of range", (unsigned long long)p);
        if (depth > 22) return set_error(SVO_ERR_FORMAT, "octree deeper than 23 levels at %llu", (unsigned long long)p);
        ++nd;
        uint32_t d = w[p];
        uint32_t valid = (d >> 8) & 0xFF, nonleaf = d & 0xFF;
        if (nonleaf & ~valid) return set_error(SVO_ERR_FORMAT, "descriptor %llu: non-leaf bit outside valid mask",
                                               (unsigned long long)p);
        uint64_t off = d >> 18;
        if (d & 0x20000u) {
            if (p + 1 >= n) return set_error(SVO_ERR_FORMAT, "far word of %llu out of range", (unsigned long long)p);
            off = (off << 32) | w[p + 1];
        }
        if (valid == 0) continue;
        if (off == 0) return set_error(SVO_ERR_FORMAT, "descriptor %llu: zero child offset", (unsigned long long)p);
        uint64_t base = p + off;
        uint64_t stride = (d & 0x10000u) ? 2 : 1;
        // Slots in descending octant order; leaves index by valid bits,
        // internal children by non-leaf bits (VoxelOctree.cpp:282, :290-293).
        for (int i = 0; i < 8; ++i) {
            uint32_t bit = 128u >> i;
            if (!(valid & bit)) continue;
            uint32_t higher = (uint32_t)__builtin_popcount(valid & (bit - 1));
            if (nonleaf & bit) {
                uint32_t sib = (uint32_t)__builtin_popcount(nonleaf & (bit - 1));
                stack.push_back({base + sib * stride, depth + 1});
            } else {
                if (base + higher >= n) return set_error(SVO_ERR_FORMAT, "leaf of %llu out of range",
                                                         (unsigned long long)p);
                ++nl;
            }
        }
    }
    if (n_desc) *n_desc = nd;
    if (n_leaves) *n_leaves = nl;
    return SVO_OK;
}

int svo_octree_build_dense(const uint32_t *grid, int w, int h, int d, uint64_t mem, int grid_on_device,
                           svo_stream stream, svo_octree **out) {
    if (!grid || !out || w <= 0 || h <= 0 || d <= 0) return set_error(SVO_ERR_INVALID, "bad grid arguments");
    int side = std::max(round_to_pow2(w), std::max(round_to_pow2(h), round_to_pow2(d)));
    if (side < 2) return set_error(SVO_ERR_INVALID, "virtual side %d below 2 (the reference recurses forever)", side);
    if (side > 65536) return set_error(SVO_ERR_LIMIT, "virtual side %d above 65536", side);
    int lb = cache_block_log2(w, h, d, mem, 4);
    if (lb < 1) return set_error(SVO_ERR_MEMORY, "memory budget %llu admits no cache block", (unsigned long long)mem);
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t *dg = grid;
    uint32_t *owned = nullptr;
    const uint64_t cells = (uint64_t)w * h * d;
    if (!grid_on_device) {
        SVO_CUDA_TRY(cudaMalloc((void **)&owned, cells * 4));
        cudaError_t e = cudaMemcpyAsync(owned, grid, cells * 4, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            cudaFree(owned);
            return cuda_fail(e, "upload grid");
        }
        dg = owned;
    }
    uint32_t *dw = nullptr;
    uint64_t nw = 0;
    int rc = build_dense_device(dg, w, h, d, log2_exact((uint64_t)side), lb, st, &dw, &nw);
    if (owned) cudaFree(owned);
    if (rc) return rc;
    float center[3] = {(float)w * 0.5f / (float)side, (float)h * 0.5f / (float)side, (float)d * 0.5f / (float)side};
    return make_handle(dw, nw, center, out);
}

// The .voxel build: the whole grid on the device when it fits in half the
// free device memory, else streamed in z slabs (voxel_stream.cu).  Both give
// the same words.  slab_bytes > 0 forces the streamed form with slabs of
// about that many bytes.
static int build_voxel_file_impl(const char *path, uint64_t mem, uint64_t slab_bytes, svo_stream stream,
                                 svo_octree **out) {
    if (!path || !out) return set_error(SVO_ERR_INVALID, "null argument");
    FILE *fp = fopen(path, "rb");
    if (!fp) return set_error(SVO_ERR_IO, "cannot open %s", path);
    std::unique_ptr<FILE, int (*)(FILE *)> guard(fp, fclose);
    int32_t dims[3];
    if (fread(dims, 4, 3, fp) != 3) return set_error(SVO_ERR_FORMAT, "%s: truncated header", path);
    int w = dims[0], h = dims[1], d = dims[2];
    if (w <= 0 || h <= 0 || d <= 0) return set_error(SVO_ERR_FORMAT, "%s: bad dimensions", path);
    const uint64_t slab = (uint64_t)w * h;
    const int side = std::max(round_to_pow2(w), std::max(round_to_pow2(h), round_to_pow2(d)));
    if (side > 65536) return set_error(SVO_ERR_LIMIT, "virtual side %d above 65536", side);
    bool streamed = slab_bytes > 0 && side >= 16;
    if (!streamed && side >= 16) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && slab * d * 4 > free_b / 2) {
            streamed = true;
            slab_bytes = std::min<uint64_t>(free_b / 8, 8ull << 30);
        }
    }
    if (streamed) {
        int lb = cache_block_log2(w, h, d, mem, 4);
        if (lb < 1) return set_error(SVO_ERR_MEMORY, "memory budget %llu admits no cache block", (unsigned long long)mem);
        uint32_t *dw = nullptr;
        uint64_t nw = 0;
        float center[3];
        int rc = build_voxel_file_streamed(fp, w, h, d, mem, slab_bytes, (cudaStream_t)stream, &dw, &nw, center);
        if (rc) return rc;
        return make_handle(dw, nw, center, out);
    }
    uint32_t *dg = nullptr;
    SVO_CUDA_TRY(cudaMalloc((void **)&dg, slab * d * 4));
    std::unique_ptr<uint32_t, cudaError_t (*)(void *)> dguard(dg, cudaFree);
    // Stream z slabs through a pinned buffer of about 64 MiB.
    uint64_t zs = std::max<uint64_t>(1, (64ull << 20) / (slab * 4));
    uint32_t *pin = nullptr;
    SVO_CUDA_TRY(cudaMallocHost((void **)&pin, zs * slab * 4));
    std::unique_ptr<uint32_t, cudaError_t (*)(void *)> pguard(pin, cudaFreeHost);
    for (uint64_t z = 0; z < (uint64_t)d; z += zs) {
        uint64_t nz = std::min<uint64_t>(zs, (uint64_t)d - z);
        size_t want = (size_t)(nz * slab);
        size_t got = fread(pin, 4, want, fp);
        if (got != want) return set_error(SVO_ERR_FORMAT, "%s: truncated voxel data", path);
        SVO_CUDA_TRY(cudaMemcpy(dg + z * slab, pin, want * 4, cudaMemcpyHostToDevice));
    }
    return svo_octree_build_dense(dg, w, h, d, mem, 1, stream, out);
}

int svo_octree_build_voxel_file(const char *path, uint64_t mem, svo_stream stream, svo_octree **out) {
    return build_voxel_file_impl(path, mem, 0, stream, out);
}

int svo_octree_build_voxel_file_streamed(const char *path, uint64_t mem, uint64_t slab_bytes, svo_stream stream,
                                         svo_octree **out) {
    if (slab_bytes == 0) return set_error(SVO_ERR_INVALID, "slab_bytes must be > 0");
    return build_voxel_file_impl(path, mem, slab_bytes, stream, out);
}

int svo_trace(const svo_octree *oct, const float *rays, uint64_t n, float ray_scale, const float light[3],
              const svo_trace_out *out, svo_stream stream) {
    if (!oct || (!rays && n) || !out) return set_error(SVO_ERR_INVALID, "null argument");
    if (n > 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "more than 2^32-1 rays");
    return launch_trace(oct, rays, n, ray_scale, light, *out, (cudaStream_t)stream);
}

int svo_trace_image(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height, float ray_scale,
                    const float light[3], const svo_trace_out *out, svo_stream stream) {
    if (!oct || (!rays && width && height) || !out) return set_error(SVO_ERR_INVALID, "null argument");
    if ((uint64_t)width * height > 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "more than 2^32-1 pixels");
    return launch_trace_image(oct, rays, width, height, ray_scale, light, *out, (cudaStream_t)stream);
}

int svo_trace_count_loads(const svo_octree *oct, const float *rays, uint64_t n, float ray_scale, uint32_t *loads,
                          svo_stream stream) {
    if (!oct || (!rays && n) || (!loads && n)) return set_error(SVO_ERR_INVALID, "null argument");
    return launch_count_loads(oct, rays, n, ray_scale, loads, (cudaStream_t)stream);
}

// svo_trace_host and svo_trace_host_async: the chunk plan and the per-chunk
// launch; `wait` drains the pipeline before returning.
static int trace_host(svo_octree *oct, const float *rays, uint64_t n, float ray_scale, const float light[3],
                      const svo_trace_out *out, bool wait) {
    if (!oct || (!rays && n) || !out) return set_error(SVO_ERR_INVALID, "null argument");
    if (n > 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "more than 2^32-1 rays");
    std::lock_guard<std::mutex> lock(oct->staging_mtx);
    if (n) {
        // warp-aligned chunks
        const std::vector<uint64_t> plan = plan_chunks(n, kStageRays, 32);
        const float lt[3] = {light ? light[0] : 0.0f, light ? light[1] : 0.0f, light ? light[2] : 0.0f};
        int rc = host_enqueue(oct, rays, plan, *out,
                              [&](const float *d_rays, uint64_t m, const svo_trace_out &o, cudaStream_t st, int) {
                                  return launch_trace(oct, d_rays, m, ray_scale, lt, o, st);
                              });
        if (rc) return rc;
    }
    return wait ? host_drain(oct) : SVO_OK;
}

static int trace_image_host(svo_octree *oct, const float *rays, uint32_t width, uint32_t height, float ray_scale,
                            const float light[3], const svo_trace_out *out, bool wait) {
    if (!oct || (!rays && width && height) || !out) return set_error(SVO_ERR_INVALID, "null argument");
    if ((uint64_t)width * height > 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "more than 2^32-1 pixels");
    std::lock_guard<std::mutex> lock(oct->staging_mtx);
    if (width && height) {
        // Chunks of whole rows, a multiple of the 4-row tile height (all but
        // the last), about kStageRays rays at full size; each chunk is traced
        // as an image of its own.
        const uint64_t rows = std::max<uint64_t>(4, (kStageRays / width) & ~uint64_t(3));
        std::vector<uint64_t> plan = plan_chunks(height, rows, 4);
        for (auto &c : plan) c *= width;
        const float lt[3] = {light ? light[0] : 0.0f, light ? light[1] : 0.0f, light ? light[2] : 0.0f};
        int rc = host_enqueue(oct, rays, plan, *out,
                              [&](const float *d_rays, uint64_t m, const svo_trace_out &o, cudaStream_t st,
                                  int buffer) {
                                  return launch_trace_image(oct, d_rays, width, (uint32_t)(m / width), ray_scale,
                                                            lt, o, st, 1 + buffer);
                              });
        if (rc) return rc;
    }
    return wait ? host_drain(oct) : SVO_OK;
}

int svo_trace_host(svo_octree *oct, const float *rays, uint64_t n, float ray_scale, const float light[3],
                   const svo_trace_out *out) {
    return trace_host(oct, rays, n, ray_scale, light, out, true);
}

int svo_trace_host_async(svo_octree *oct, const float *rays, uint64_t n, float ray_scale, const float light[3],
                         const svo_trace_out *out) {
    return trace_host(oct, rays, n, ray_scale, light, out, false);
}

int svo_trace_image_host(svo_octree *oct, const float *rays, uint32_t width, uint32_t height, float ray_scale,
                         const float light[3], const svo_trace_out *out) {
    return trace_image_host(oct, rays, width, height, ray_scale, light, out, true);
}

int svo_trace_image_host_async(svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                               float ray_scale, const float light[3], const svo_trace_out *out) {
    return trace_image_host(oct, rays, width, height, ray_scale, light, out, false);
}

int svo_octree_synchronize(svo_octree *oct) {
    if (!oct) return set_error(SVO_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lock(oct->staging_mtx);
    return host_drain(oct);
}

}  // extern "C"
