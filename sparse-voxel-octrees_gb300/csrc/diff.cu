// diff.cu — differentiable leaf shading over the octree (no counterpart in
// the reference; the shading model is the viewer's shade(), Main.cpp:81-90,
// with per-leaf parameters in place of the packed leaf word).
//
// Parameters are FP32 arrays indexed by the leaf's word index (the `leaf`
// output of svo_trace): rgb[3*i..] and normal[3*i..].  For a ray with
// direction d, hitting leaf i, under light l:
//   n     = p / |p|                 (p = normal parameters; n = 0 when p = 0)
//   a     = |l.n|
//   r     = d - 2 (n.d) n           (Vec3::reflect, math/Vec3.hpp:63-71)
//   s     = max(l.r, 0)
//   rgb_k = c_k * 0.9 * a + 0.2 * s^2          (c = rgb parameters)
// Rays that hit no leaf produce 0 and no gradient.  Traversal is the discrete
// ESVO raymarch, unchanged; only the shading is differentiated:
//   dL/dc_k = g_k 0.9 a
//   dL/dn   = (0.9 sgn(l.n) sum_k g_k c_k) l - 0.8 G s [s > 0] ((n.d) l + (n.l) d),  G = sum_k g_k
//   dL/dp   = (dL/dn - n (n.dL/dn)) / |p|
// with g = dL/drgb.  Gradients are summed over rays with atomics; lanes of a
// warp that hit the same leaf are first reduced in registers (match_any +
// a rank-ordered shuffle tree), so one lane per distinct leaf issues the six
// atomicAdds.  Summation order across warps is not fixed, so gradients can
// differ in the last bits between runs.
#include "svo_device.cuh"
#include "svo_internal.h"

namespace svo {
namespace {

struct DiffArgs {
    const uint32_t *oct;
    const uint4 *tab;  // descriptor table (kernels instantiated with kTab)
    uint32_t n_words;
    const float *rays;
    uint32_t width, height, n_views;  // image = width x (height * n_views), view v = rows [v*height, (v+1)*height)
    uint32_t tiles_x;
    uint64_t total;
    const float *lights;  // 3 per view (device)
    const float *p_rgb, *p_n;
    uint32_t stride;  // floats from one leaf's parameters (and gradients) to the next
    uint32_t *hit_leaf;
    float *rgb;
    const float *d_rgb;
    float *g_rgb, *g_n;
    unsigned long long *queue;
    uint32_t *status;
    // fused L2 loss (svo_diff_backward_l2): dL/drgb = loss_scale (rgb - target)
    const float *target;
    float loss_scale;
    double *loss_sum;  // optional: += sum over rays and channels of (rgb - target)^2
    // optional record of the leaves that received a gradient
    uint32_t *touched;     // one bit per octree word
    uint32_t *leaf_list;   // leaves in order of first touch
    uint32_t *leaf_count;  // entries in leaf_list
    uint32_t leaf_cap;
};

__device__ __forceinline__ bool tile_pixel(const DiffArgs &a, uint64_t slot, uint32_t &idx, uint32_t &view) {
    if (slot >= a.total) return false;
    const uint32_t tile = (uint32_t)(slot >> 5), r = (uint32_t)(slot & 31);  // tile < 2^27: 32-bit division
    const uint32_t ty = tile / a.tiles_x, tx = tile - ty * a.tiles_x;
    uint32_t px = tx * 8u + (r & 7u);
    uint32_t py = ty * 4u + (r >> 3);
    if (px >= a.width || py >= a.height * a.n_views) return false;
    idx = py * a.width + px;
    view = py / a.height;
    return true;
}

struct Shading {
    float nx, ny, nz, inv_len, ln, a, nd, s;
};

__device__ __forceinline__ Shading shade_terms(const float *p_n, uint32_t stride, uint32_t leaf, float dx, float dy,
                                               float dz, float lx, float ly, float lz) {
    Shading sh;
    const float *pn = p_n + (uint64_t)stride * leaf;
    float px = pn[0], py = pn[1], pz = pn[2];
    float len2 = px * px + py * py + pz * pz;
    sh.inv_len = len2 > 0.0f ? 1.0f / sqrtf(len2) : 0.0f;
    sh.nx = px * sh.inv_len;
    sh.ny = py * sh.inv_len;
    sh.nz = pz * sh.inv_len;
    sh.ln = lx * sh.nx + ly * sh.ny + lz * sh.nz;
    sh.a = fabsf(sh.ln);
    sh.nd = sh.nx * dx + sh.ny * dy + sh.nz * dz;
    float proj = sh.nd * 2.0f;
    float rx = dx - sh.nx * proj, ry = dy - sh.ny * proj, rz = dz - sh.nz * proj;
    sh.s = fmaxf(lx * rx + ly * ry + lz * rz, 0.0f);
    return sh;
}

// Slots a warp takes from the queue at once (multiples of 32): a forward
// warp traces one 8x4 tile at a time; the adjoint, without traversal, is
// short per slot, so it takes several tiles per queue access.
constexpr int kFwdChunk = 64;
constexpr int kBwdChunk = 128;

template <bool kTab, bool kRecord>
__global__ void k_diff_forward(DiffArgs a) {
    const int lane = threadIdx.x & 31;
    RayStackFor<kTab> stk;
    unsigned long long base = 0, end = 0;
    while (true) {
        if (base >= end) {
            if (lane == 0) base = atomicAdd(a.queue, (unsigned long long)kFwdChunk);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= a.total) break;
            end = min(base + (unsigned long long)kFwdChunk, (unsigned long long)a.total);
        }
        const unsigned long long slot = base + lane;
        base += 32;
        uint32_t idx, view;
        if (!tile_pixel(a, slot, idx, view)) continue;
        const float2 *r2 = reinterpret_cast<const float2 *>(a.rays) + 3 * (uint64_t)idx;
        float2 p0 = __ldg(r2), p1 = __ldg(r2 + 1), p2 = __ldg(r2 + 2);
        RayState st;
        ray_init_any<kTab>(st, a.oct, a.tab, p0.x, p0.y, p1.x, p1.y, p2.x, p2.y);
        RayResult res;
        while (!ray_step_any<kTab, false>(st, stk, a.oct, a.tab, a.n_words, 0.0f, res)) {
        }
        if (res.status == kFault) atomicOr(a.status, 1u);
        bool hit = res.status == kLeafHit;
        if (kRecord) a.hit_leaf[idx] = hit ? res.leaf : 0xFFFFFFFFu;
        float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
        if (hit) {
            float lx = a.lights[3 * view], ly = a.lights[3 * view + 1], lz = a.lights[3 * view + 2];
            Shading sh = shade_terms(a.p_n, a.stride, res.leaf, p1.y, p2.x, p2.y, lx, ly, lz);
            float spec = sh.s * sh.s * 0.2f;
            const float *c = a.p_rgb + (uint64_t)a.stride * res.leaf;
            c0 = c[0] * 0.9f * sh.a + spec;
            c1 = c[1] * 0.9f * sh.a + spec;
            c2 = c[2] * 0.9f * sh.a + spec;
        }
        a.rgb[3 * (uint64_t)idx] = c0;
        a.rgb[3 * (uint64_t)idx + 1] = c1;
        a.rgb[3 * (uint64_t)idx + 2] = c2;
    }
}

// Sum of v over the lanes in `peers` (the lanes holding the same key), left
// in the group's lowest lane.  Lane ranks within the group form a binary
// tree: at distance k a lane whose rank is a multiple of 2k adds the value of
// the group member k ranks above it.  All 32 lanes execute every shuffle.
__device__ __forceinline__ float group_sum(unsigned peers, unsigned rank, unsigned size, float v) {
    for (unsigned k = 1; k < 32; k <<= 1) {
        unsigned src_rank = rank + k;
        bool take = (rank % (2 * k)) == 0 && src_rank < size;
        int src = take ? (int)__fns(peers, 0, (int)src_rank + 1) : (int)(threadIdx.x & 31);
        float o = __shfl_sync(0xffffffffu, v, src);
        if (take) v += o;
    }
    return v;
}

// Records `leaf` in the touched set the first time any warp adds a gradient
// to it (called by the one lane that adds the leaf's gradient).
__device__ __forceinline__ void mark_touched(const DiffArgs &a, uint32_t leaf) {
    const uint32_t w = leaf >> 5, bit = 1u << (leaf & 31u);
    if (__ldcg(a.touched + w) & bit) return;  // already recorded (the common case after the first pass)
    if (atomicOr(a.touched + w, bit) & bit) return;
    const uint32_t pos = atomicAdd(a.leaf_count, 1u);
    if (pos < a.leaf_cap) a.leaf_list[pos] = leaf;
}

// kRetrace: recompute the hit leaf by traversal instead of reading hit_leaf.
// kFused: dL/drgb = loss_scale (rgb - target) from the forward pass's rgb
// instead of a d_rgb array, and the loss summed on the way.
template <bool kTab, bool kRetrace, bool kFused>
__global__ void k_diff_backward(DiffArgs a) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    RayStackFor<kTab> stk;
    float loss = 0.0f;  // this lane's share of sum (rgb - target)^2
    unsigned long long base = 0, end = 0;
    while (true) {
        if (base >= end) {
            if (lane == 0) base = atomicAdd(a.queue, (unsigned long long)kBwdChunk);
            base = __shfl_sync(FULL, base, 0);
            if (base >= a.total) break;
            end = min(base + (unsigned long long)kBwdChunk, (unsigned long long)a.total);
        }
        const unsigned long long slot = base + lane;
        base += 32;
        uint32_t idx = 0, view = 0;
        bool live = tile_pixel(a, slot, idx, view);
        uint32_t leaf = 0xFFFFFFFFu;
        float dx = 0.f, dy = 0.f, dz = 0.f;
        if (live) {
            const float2 *r2 = reinterpret_cast<const float2 *>(a.rays) + 3 * (uint64_t)idx;
            float2 p1 = __ldg(r2 + 1), p2 = __ldg(r2 + 2);
            dx = p1.y;
            dy = p2.x;
            dz = p2.y;
            if (kRetrace) {
                float2 p0 = __ldg(r2);
                RayState st;
                ray_init_any<kTab>(st, a.oct, a.tab, p0.x, p0.y, p1.x, dx, dy, dz);
                RayResult res;
                while (!ray_step_any<kTab, false>(st, stk, a.oct, a.tab, a.n_words, 0.0f, res)) {
                }
                if (res.status == kFault) atomicOr(a.status, 1u);
                if (res.status == kLeafHit) leaf = res.leaf;
            } else {
                leaf = a.hit_leaf[idx];
            }
        }
        float gc0 = 0.f, gc1 = 0.f, gc2 = 0.f, gp0 = 0.f, gp1 = 0.f, gp2 = 0.f;
        bool contrib = leaf != 0xFFFFFFFFu;
        float g0 = 0.f, g1 = 0.f, g2 = 0.f;
        if (kFused && live) {
            // every ray adds to the loss; a miss (rgb 0) contributes no gradient
            const float *c3 = a.rgb + 3 * (uint64_t)idx, *t3 = a.target + 3 * (uint64_t)idx;
            const float e0 = c3[0] - t3[0], e1 = c3[1] - t3[1], e2 = c3[2] - t3[2];
            loss += e0 * e0 + e1 * e1 + e2 * e2;
            g0 = a.loss_scale * e0;
            g1 = a.loss_scale * e1;
            g2 = a.loss_scale * e2;
        }
        if (contrib) {
            float lx = a.lights[3 * view], ly = a.lights[3 * view + 1], lz = a.lights[3 * view + 2];
            Shading sh = shade_terms(a.p_n, a.stride, leaf, dx, dy, dz, lx, ly, lz);
            const float *c = a.p_rgb + (uint64_t)a.stride * leaf;
            if (!kFused) {
                g0 = a.d_rgb[3 * (uint64_t)idx];
                g1 = a.d_rgb[3 * (uint64_t)idx + 1];
                g2 = a.d_rgb[3 * (uint64_t)idx + 2];
            }
            gc0 = g0 * 0.9f * sh.a;
            gc1 = g1 * 0.9f * sh.a;
            gc2 = g2 * 0.9f * sh.a;
            float sgn = sh.ln > 0.0f ? 1.0f : (sh.ln < 0.0f ? -1.0f : 0.0f);
            float wl = 0.9f * sgn * (g0 * c[0] + g1 * c[1] + g2 * c[2]);
            float ws = sh.s > 0.0f ? -0.8f * (g0 + g1 + g2) * sh.s : 0.0f;
            // dL/dn = wl l + ws ((n.d) l + (n.l) d)
            float gnx = wl * lx + ws * (sh.nd * lx + sh.ln * dx);
            float gny = wl * ly + ws * (sh.nd * ly + sh.ln * dy);
            float gnz = wl * lz + ws * (sh.nd * lz + sh.ln * dz);
            float ndg = sh.nx * gnx + sh.ny * gny + sh.nz * gnz;
            gp0 = (gnx - sh.nx * ndg) * sh.inv_len;
            gp1 = (gny - sh.ny * ndg) * sh.inv_len;
            gp2 = (gnz - sh.nz * ndg) * sh.inv_len;
        }
        // warp aggregation by leaf: one set of atomics per distinct leaf
        unsigned peers = __match_any_sync(FULL, leaf);
        unsigned rank = __popc(peers & lt), size = __popc(peers);
        gc0 = group_sum(peers, rank, size, gc0);
        gc1 = group_sum(peers, rank, size, gc1);
        gc2 = group_sum(peers, rank, size, gc2);
        gp0 = group_sum(peers, rank, size, gp0);
        gp1 = group_sum(peers, rank, size, gp1);
        gp2 = group_sum(peers, rank, size, gp2);
        if (contrib && rank == 0) {
            float *gr = a.g_rgb + (uint64_t)a.stride * leaf;
            float *gn = a.g_n + (uint64_t)a.stride * leaf;
            atomicAdd(gr, gc0);
            atomicAdd(gr + 1, gc1);
            atomicAdd(gr + 2, gc2);
            atomicAdd(gn, gp0);
            atomicAdd(gn + 1, gp1);
            atomicAdd(gn + 2, gp2);
            if (a.touched) mark_touched(a, leaf);
        }
    }
    if (kFused && a.loss_sum) {
        // one atomic per warp, at its end (a per-pass atomic on one address
        // would serialise the warps)
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(FULL, loss, o);
        if (lane == 0) atomicAdd(a.loss_sum, (double)loss);
    }
}

int prepare(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height, uint32_t n_views,
            const float *lights, const float *p_rgb, const float *p_n, uint32_t stride, DiffArgs &a) {
    if (!oct || !rays || !lights || !p_rgb || !p_n || width == 0 || height == 0 || n_views == 0)
        return set_error(SVO_ERR_INVALID, "bad arguments");
    if (stride < 3) return set_error(SVO_ERR_INVALID, "parameter stride %u below 3", stride);
    if ((uint64_t)width * height * n_views > 0xFFFFFFFFull) return set_error(SVO_ERR_LIMIT, "more than 2^32-1 rays");
    if (wide_octree(oct)) return set_error(SVO_ERR_LIMIT, "leaf shading takes octrees of up to 2^32-1 words");
    std::memset(&a, 0, sizeof(a));
    a.oct = oct->d_words;
    a.n_words = (uint32_t)oct->n_words;
    a.rays = rays;
    a.width = width;
    a.height = height;
    a.n_views = n_views;
    a.tiles_x = (width + 7) / 8;
    a.total = (uint64_t)a.tiles_x * ((height * n_views + 3) / 4) * 32;
    a.lights = lights;
    a.p_rgb = p_rgb;
    a.p_n = p_n;
    a.stride = stride;
    a.queue = oct->d_queue;
    a.status = oct->d_status;
    return SVO_OK;
}

template <typename K>
int launch_persistent(K kern, const DiffArgs &a, cudaStream_t st) {
    int dev = 0, sms = 0, resident = 0;
    SVO_CUDA_TRY(cudaGetDevice(&dev));
    SVO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, 256, 0));
    SVO_CUDA_TRY(cudaMemsetAsync(a.queue, 0, sizeof(unsigned long long), st));
    kern<<<(unsigned)(sms * (resident > 0 ? resident : 1)), 256, 0, st>>>(a);
    SVO_CUDA_TRY(cudaGetLastError());
    return SVO_OK;
}

}  // namespace
}  // namespace svo

using namespace svo;

extern "C" {

int svo_diff_forward_stride(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                            uint32_t n_views, const float *lights, const float *leaf_rgb, const float *leaf_normal,
                            uint32_t param_stride, uint32_t *hit_leaf, float *rgb, svo_stream stream) {
    DiffArgs a;
    int rc = prepare(oct, rays, width, height, n_views, lights, leaf_rgb, leaf_normal, param_stride, a);
    if (rc) return rc;
    if (!rgb) return set_error(SVO_ERR_INVALID, "rgb output required");
    a.hit_leaf = hit_leaf;
    a.rgb = rgb;
    cudaStream_t st = (cudaStream_t)stream;
    a.tab = octree_table(oct, st);
    if (a.tab)
        return hit_leaf ? launch_persistent(k_diff_forward<true, true>, a, st)
                        : launch_persistent(k_diff_forward<true, false>, a, st);
    return hit_leaf ? launch_persistent(k_diff_forward<false, true>, a, st)
                    : launch_persistent(k_diff_forward<false, false>, a, st);
}

int svo_diff_backward_stride(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                             uint32_t n_views, const float *lights, const float *leaf_rgb, const float *leaf_normal,
                             uint32_t param_stride, const uint32_t *hit_leaf, const float *d_rgb, float *grad_rgb,
                             float *grad_normal, svo_stream stream) {
    DiffArgs a;
    int rc = prepare(oct, rays, width, height, n_views, lights, leaf_rgb, leaf_normal, param_stride, a);
    if (rc) return rc;
    if (!d_rgb || !grad_rgb || !grad_normal) return set_error(SVO_ERR_INVALID, "gradient buffers required");
    a.hit_leaf = const_cast<uint32_t *>(hit_leaf);
    a.d_rgb = d_rgb;
    a.g_rgb = grad_rgb;
    a.g_n = grad_normal;
    cudaStream_t st = (cudaStream_t)stream;
    a.tab = hit_leaf ? nullptr : octree_table(oct, st);  // the table only serves the retrace
    if (a.tab) return launch_persistent(k_diff_backward<true, true, false>, a, st);
    return hit_leaf ? launch_persistent(k_diff_backward<false, false, false>, a, st)
                    : launch_persistent(k_diff_backward<false, true, false>, a, st);
}

int svo_diff_backward_l2_stride(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                                uint32_t n_views, const float *lights, const float *leaf_rgb,
                                const float *leaf_normal, uint32_t param_stride, const uint32_t *hit_leaf,
                                const float *rgb, const float *target, float loss_scale, float *grad_rgb,
                                float *grad_normal, double *loss_sum, uint32_t *touched, uint32_t *leaf_list,
                                uint32_t *leaf_count, uint64_t leaf_capacity, svo_stream stream) {
    DiffArgs a;
    int rc = prepare(oct, rays, width, height, n_views, lights, leaf_rgb, leaf_normal, param_stride, a);
    if (rc) return rc;
    if (!rgb || !target || !grad_rgb || !grad_normal)
        return set_error(SVO_ERR_INVALID, "rgb, target and gradient buffers required");
    if ((touched != nullptr) != (leaf_list != nullptr) || (touched != nullptr) != (leaf_count != nullptr))
        return set_error(SVO_ERR_INVALID, "touched, leaf_list and leaf_count go together");
    if (touched && leaf_capacity < oct->n_words)
        return set_error(SVO_ERR_INVALID, "leaf_list holds %llu entries; it needs one per octree word (%llu)",
                         (unsigned long long)leaf_capacity, (unsigned long long)oct->n_words);
    a.hit_leaf = const_cast<uint32_t *>(hit_leaf);
    a.rgb = const_cast<float *>(rgb);
    a.target = target;
    a.loss_scale = loss_scale;
    a.loss_sum = loss_sum;
    a.g_rgb = grad_rgb;
    a.g_n = grad_normal;
    a.touched = touched;
    a.leaf_list = leaf_list;
    a.leaf_count = leaf_count;
    a.leaf_cap = touched ? (uint32_t)oct->n_words : 0u;
    cudaStream_t st = (cudaStream_t)stream;
    a.tab = hit_leaf ? nullptr : octree_table(oct, st);
    if (a.tab) return launch_persistent(k_diff_backward<true, true, true>, a, st);
    return hit_leaf ? launch_persistent(k_diff_backward<false, false, true>, a, st)
                    : launch_persistent(k_diff_backward<false, true, true>, a, st);
}

// The separate-array forms: 3 floats per leaf in each array.
int svo_diff_forward(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height, uint32_t n_views,
                     const float *lights, const float *leaf_rgb, const float *leaf_normal, uint32_t *hit_leaf,
                     float *rgb, svo_stream stream) {
    return svo_diff_forward_stride(oct, rays, width, height, n_views, lights, leaf_rgb, leaf_normal, 3, hit_leaf,
                                   rgb, stream);
}

int svo_diff_backward(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height, uint32_t n_views,
                      const float *lights, const float *leaf_rgb, const float *leaf_normal, const uint32_t *hit_leaf,
                      const float *d_rgb, float *grad_rgb, float *grad_normal, svo_stream stream) {
    return svo_diff_backward_stride(oct, rays, width, height, n_views, lights, leaf_rgb, leaf_normal, 3, hit_leaf,
                                    d_rgb, grad_rgb, grad_normal, stream);
}

int svo_diff_backward_l2(const svo_octree *oct, const float *rays, uint32_t width, uint32_t height,
                         uint32_t n_views, const float *lights, const float *leaf_rgb, const float *leaf_normal,
                         const uint32_t *hit_leaf, const float *rgb, const float *target, float loss_scale,
                         float *grad_rgb, float *grad_normal, double *loss_sum, uint32_t *touched,
                         uint32_t *leaf_list, uint32_t *leaf_count, uint64_t leaf_capacity, svo_stream stream) {
    return svo_diff_backward_l2_stride(oct, rays, width, height, n_views, lights, leaf_rgb, leaf_normal, 3, hit_leaf,
                                       rgb, target, loss_scale, grad_rgb, grad_normal, loss_sum, touched, leaf_list,
                                       leaf_count, leaf_capacity, stream);
}

}  // extern "C"
