// mem_pool.cpp — the library's stream-ordered scratch pool.
//
// Builds allocate and free their working arrays on the build's stream.  The
// device's default pool hands freed memory back to the driver at every
// synchronisation, so each build would map its scratch again (hundreds of
// MB for a 1024^3 mesh build).  The library therefore keeps one pool per
// device whose release threshold is unbounded: freed scratch stays mapped
// for the next build until svo_trim_memory() returns it.
#include <mutex>

#include "svo_internal.h"

namespace svo {

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_pool_mtx;
cudaMemPool_t g_pools[kMaxDevices] = {};
}  // namespace

cudaError_t pool_for_current_device(cudaMemPool_t *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_pool_mtx);
    if (!g_pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        e = cudaMemPoolCreate(&pool, &props);
        if (e != cudaSuccess) return e;
        uint64_t keep = ~0ull;
        e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(pool);
            return e;
        }
        g_pools[dev] = pool;
    }
    *out = g_pools[dev];
    return cudaSuccess;
}

cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t st) {
    cudaMemPool_t pool;
    cudaError_t e = pool_for_current_device(&pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

}  // namespace svo

extern "C" int svo_trim_memory(void) {
    svo::clear_error();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return svo::cuda_fail(e, "cudaGetDevice");
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lk(svo::g_pool_mtx);
        if (dev >= 0 && dev < svo::kMaxDevices) pool = svo::g_pools[dev];
    }
    if (!pool) return SVO_OK;
    e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemPoolTrimTo(pool, 0);
    if (e != cudaSuccess) return svo::cuda_fail(e, "trimming the scratch pool");
    return SVO_OK;
}
