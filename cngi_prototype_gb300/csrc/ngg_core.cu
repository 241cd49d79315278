// Error state, scratch allocation and library-level entry points.
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>

#include "ngg_internal.cuh"

namespace ngg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? NGG_ERR_NOMEM : NGG_ERR_CUDA;
}

static std::mutex g_pool_mu;
static bool g_pool_ready[64] = {false};

int scratch_alloc(void **p, size_t bytes, cudaStream_t s) {
    *p = nullptr;
    if (bytes == 0) bytes = 256;
    int dev = 0;
    NGG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64) {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        if (!g_pool_ready[dev]) {
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
                uint64_t thr = UINT64_MAX;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
            }
            g_pool_ready[dev] = true;
        }
    }
    cudaError_t e = cudaMallocAsync(p, bytes, s);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, "cudaMallocAsync(scratch)");
    }
    return NGG_OK;
}

void scratch_free(void *p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
}

int num_sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

void release_fft_plans();  // fft.cu

}  // namespace ngg

extern "C" int ngg_version(void) { return 100; }

extern "C" const char *ngg_last_error(void) { return ngg::g_last_error.c_str(); }

extern "C" void ngg_release_cache(void) {
    ngg::release_fft_plans();
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
    }
}
