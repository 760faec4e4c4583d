// octree_table.cu — builds an octree handle's descriptor table, the structure
// the table traversal (ray_step_tab) walks instead of decoding relative and
// far offsets with bounds checks at every PUSH.
//
// Breadth first from the root, one level at a time:
//   1. k_table_nodes: per node of the level, table_node's checks
//      (octree_table.cuh), its entry {descriptor, -, child block, stride} and
//      its internal-child count;
//   2. an exclusive scan of the counts gives each node's first child in the
//      next level;
//   3. k_table_children: the entry's first-child ordinal, and the next
//      level's node words (block start + j * stride for its j-th internal
//      child).
// A failed check anywhere, a level past 22 or more entries than words (a
// node reachable twice) leaves the handle without a table.  The table costs
// 16 bytes per node, about 2 bytes per octree word on the benchmark scenes.
#include <memory>
#include <vector>

#include "octree_table.cuh"
#include "scan.cuh"
#include "svo_internal.h"

namespace svo {
namespace {

__global__ void k_table_nodes(const uint32_t *__restrict__ words, uint32_t n_words, const uint32_t *__restrict__ level,
                              uint32_t n, int L, uint4 *__restrict__ entries, uint32_t *__restrict__ n_int,
                              uint32_t *__restrict__ err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t d = level[i];
    uint32_t cb, stride, k;
    if (!table_node(words, n_words, d, L, cb, stride, k)) {
        atomicOr(err, 1u);
        k = 0;
    }
    entries[i] = make_uint4(words[d], 0u, cb, stride);
    n_int[i] = k;
}

__global__ void k_table_children(const uint32_t *__restrict__ n_int, const uint32_t *__restrict__ first, uint32_t n,
                                 uint32_t next_base, uint4 *__restrict__ entries, uint32_t *__restrict__ next) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint4 e = entries[i];
    const uint32_t k = n_int[i], o = first[i], stride = e.w;
    for (uint32_t j = 0; j < k; ++j) next[o + j] = e.z + j * stride;
    e.y = next_base + o;
    e.w = 0;
    entries[i] = e;
}

struct Scratch {
    void *p = nullptr;
    cudaStream_t st = nullptr;
    Scratch() = default;
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;
    cudaError_t alloc(size_t bytes, cudaStream_t s) {
        st = s;
        return scratch_alloc(&p, bytes ? bytes : 4, s);
    }
    ~Scratch() {
        if (p) cudaFreeAsync(p, st);
    }
};

inline unsigned grid_for(uint64_t n) { return (unsigned)((n + 255) / 256); }

// Builds the table on `st` and waits for it.  Returns SVO_OK with *tab set
// (cudaMalloc'd, n_tab entries) or with *tab = nullptr when the octree does
// not qualify; an error code only for CUDA failures.
int build_table(const uint32_t *d_words, uint64_t n_words, cudaStream_t st, uint4 **tab, uint64_t *n_tab) {
    *tab = nullptr;
    *n_tab = 0;
    if (n_words == 0 || n_words > kMaxNarrowWords) return SVO_OK;
    const uint32_t W = (uint32_t)n_words;
    std::unique_ptr<Scratch[]> lv_entries(new Scratch[kTableMaxParentLevel + 2]);
    std::vector<uint32_t> lv_n;
    Scratch err, cur, total;
    SVO_CUDA_TRY(err.alloc(sizeof(uint32_t), st));
    SVO_CUDA_TRY(total.alloc(sizeof(uint32_t), st));
    SVO_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(uint32_t), st));
    SVO_CUDA_TRY(cur.alloc(sizeof(uint32_t), st));
    SVO_CUDA_TRY(cudaMemsetAsync(cur.p, 0, sizeof(uint32_t), st));  // level 0: the root at word 0
    uint32_t n = 1;
    uint64_t base = 0;
    bool ok = true;
    for (int L = 0; n > 0; ++L) {
        if (L > kTableMaxParentLevel + 1 || base + n > n_words) {
            ok = false;
            break;
        }
        Scratch &ent = lv_entries[L];
        SVO_CUDA_TRY(ent.alloc((size_t)n * sizeof(uint4), st));
        Scratch c, f, sc;
        SVO_CUDA_TRY(c.alloc((size_t)n * sizeof(uint32_t), st));
        SVO_CUDA_TRY(f.alloc((size_t)n * sizeof(uint32_t), st));
        SVO_CUDA_TRY(sc.alloc(scan_scratch_elems(n) * sizeof(uint32_t), st));
        k_table_nodes<<<grid_for(n), 256, 0, st>>>(d_words, W, (const uint32_t *)cur.p, n, L, (uint4 *)ent.p,
                                                   (uint32_t *)c.p, (uint32_t *)err.p);
        SVO_CUDA_TRY(cudaGetLastError());
        SVO_CUDA_TRY((exclusive_scan<uint32_t, uint32_t>((const uint32_t *)c.p, (uint32_t *)f.p, n,
                                                         (uint32_t *)total.p, (uint32_t *)sc.p, st)));
        uint32_t next_n = 0;
        SVO_CUDA_TRY(cudaMemcpyAsync(&next_n, total.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        SVO_CUDA_TRY(cudaStreamSynchronize(st));
        Scratch nxt;
        SVO_CUDA_TRY(nxt.alloc((size_t)next_n * sizeof(uint32_t), st));
        const uint64_t next_base = base + n;
        if (next_base + next_n > n_words) {
            lv_n.push_back(n);
            ok = false;
            break;
        }
        k_table_children<<<grid_for(n), 256, 0, st>>>((const uint32_t *)c.p, (const uint32_t *)f.p, n,
                                                      (uint32_t)next_base, (uint4 *)ent.p, (uint32_t *)nxt.p);
        SVO_CUDA_TRY(cudaGetLastError());
        lv_n.push_back(n);
        base = next_base;
        n = next_n;
        std::swap(cur.p, nxt.p);  // nxt now owns the finished level's node list
    }
    uint32_t err_h = 0;
    SVO_CUDA_TRY(cudaMemcpyAsync(&err_h, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    if (!ok || err_h) return SVO_OK;
    uint4 *t = nullptr;
    SVO_CUDA_TRY(cudaMalloc((void **)&t, (size_t)base * sizeof(uint4)));
    uint64_t at = 0;
    for (size_t L = 0; L < lv_n.size(); ++L) {
        cudaError_t e = cudaMemcpyAsync(t + at, lv_entries[L].p, (size_t)lv_n[L] * sizeof(uint4),
                                        cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) {
            cudaFree(t);
            return cuda_fail(e, "descriptor table copy");
        }
        at += lv_n[L];
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(t);
        return cuda_fail(e, "descriptor table");
    }
    *tab = t;
    *n_tab = base;
    return SVO_OK;
}

}  // namespace

const uint4 *octree_table(const svo_octree *oct, cudaStream_t caller) {
    if (!oct->use_table) return nullptr;
    if (oct->tab_state == 1) return oct->d_tab;
    if (oct->tab_state != 0) return nullptr;
    // Never build while the caller's stream is being captured: the checked
    // traversal runs instead, and a later uncaptured call builds the table.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(caller, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return nullptr;
    std::lock_guard<std::mutex> lock(oct->tab_mtx);
    if (oct->tab_state == 0) {
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
        uint4 *t = nullptr;
        uint64_t nt = 0;
        int rc = build_table(oct->d_words, oct->n_words, st, &t, &nt);
        cudaStreamDestroy(st);
        if (rc != SVO_OK) {
            // A CUDA failure (device memory, most likely): keep the word
            // traversal for this handle rather than retry on every call.
            clear_error();
            cudaGetLastError();  // drop a non-sticky allocation error so later calls do not report it
            oct->tab_state = -1;
            return nullptr;
        }
        oct->d_tab = t;
        oct->n_tab = nt;
        oct->tab_state = t ? 1 : -1;
    }
    return oct->tab_state == 1 ? oct->d_tab : nullptr;
}

}  // namespace svo
