// Inverse FFT of gridded planes, centre crop and gridding correction.
//
// Reference behaviour (make_image.py:116-130, make_psf.py:117-131,
// _remove_padding.py:20-31):
//     img = fftshift(ifft2(ifftshift(grid))) ; crop centre (n_l, n_m) window
//     img = img.real * Nu*Nv / sum_weight(0->1) / correction
// Because the gridder already wrote each plane in ifftshift order
// (NGG_LAYOUT_FFT), the shifts reduce to index arithmetic: an unnormalised
// inverse C2C transform (cuFFT, in place) followed by one epilogue kernel that
// reads only the cropped window, applies the fftshift mapping
// out[(l - n_l/2) mod Nu, (m - n_m/2) mod Nv], and divides by sum_weight and
// the correction image. numpy's ifft2 times Nu*Nv equals cuFFT's unnormalised
// CUFFT_INVERSE, so no scaling is applied.
#include <cufft.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "ngg_internal.cuh"

namespace ngg {

namespace {
struct PlanKey {
    int dev;
    int64_t nu, nv;
    int batch;
    bool z;   // double precision (Z2Z)
    bool operator<(const PlanKey &o) const {
        return std::tie(dev, nu, nv, batch, z) < std::tie(o.dev, o.nu, o.nv, o.batch, o.z);
    }
};
std::mutex g_plan_mu;
std::map<PlanKey, cufftHandle> g_plans;

int get_plan(int64_t nu, int64_t nv, int batch, cufftHandle *out, bool z = false) {
    int dev = 0;
    cudaGetDevice(&dev);
    PlanKey k{dev, nu, nv, batch, z};
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plans.find(k);
    if (it != g_plans.end()) {
        *out = it->second;
        return NGG_OK;
    }
    cufftHandle h;
    if (cufftCreate(&h) != CUFFT_SUCCESS) return fail(NGG_ERR_CUDA, "cufftCreate");
    long long n[2] = {(long long)nu, (long long)nv};
    size_t ws = 0;
    cufftResult r = cufftMakePlanMany64(h, 2, n, nullptr, 1, nu * nv, nullptr, 1, nu * nv, z ? CUFFT_Z2Z : CUFFT_C2C, batch,
                                        &ws);
    if (r != CUFFT_SUCCESS) {
        cufftDestroy(h);
        return fail(r == CUFFT_ALLOC_FAILED ? NGG_ERR_NOMEM : NGG_ERR_CUDA, "cufftMakePlanMany64 failed");
    }
    g_plans[k] = h;
    *out = h;
    return NGG_OK;
}

// Per-plane 1/sum_weight (0 -> 1) of a batch, staged in shared memory: the
// epilogues multiply by reciprocals. GB300 runs FP64 at a small fraction of
// FP32, and two FP64 divisions per pixel and plane made these kernels
// FP64-bound; the complex64 planes (FP32 transform) are scaled in FP32 (the
// result is within 3 FP32 ulps of the FP64 quotient of the same FP32 value,
// below the transform's own error), the complex128 planes in FP64 with
// reciprocals (within 2 ulps of the FP64 quotient).
constexpr int MAX_BATCH = 64;
__device__ __forceinline__ void stage_inv_sw(const double *sum_weight, int plane0, int nplanes, double *isw,
                                             float *iswf) {
    for (int q = threadIdx.x; q < nplanes; q += blockDim.x) {
        double sw = sum_weight[plane0 + q];
        if (sw == 0.0) sw = 1.0;
        isw[q] = 1.0 / sw;
        iswf[q] = (float)isw[q];
    }
    __syncthreads();
}

// one thread per output pixel (l, m) of one plane batch
template <typename C2>
__global__ void k_crop_correct(const C2 *__restrict__ planes, int nplanes, int plane0, int64_t nu, int64_t nv,
                               int64_t nl, int64_t nm, int64_t n_planes_total, const double *__restrict__ sum_weight,
                               const double *__restrict__ correction, double *__restrict__ image) {
    __shared__ double isw[MAX_BATCH];
    __shared__ float iswf[MAX_BATCH];
    stage_inv_sw(sum_weight, plane0, nplanes, isw, iswf);
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nl * nm) return;
    const int64_t l = id / nm, m = id % nm;
    int64_t k1 = l - nl / 2, k2 = m - nm / 2;
    if (k1 < 0) k1 += nu;
    if (k2 < 0) k2 += nv;
    const C2 *__restrict__ src = planes + k1 * nv + k2;
    double *__restrict__ dst = image + id * n_planes_total + plane0;
    const int64_t plane = nu * nv;
    if constexpr (sizeof(C2) == 8) {
        const float ic = 1.0f / (float)correction[id];
#pragma unroll 4
        for (int q = 0; q < nplanes; ++q) dst[q] = (double)(src[(int64_t)q * plane].x * (iswf[q] * ic));
    } else {
        const double ic = 1.0 / correction[id];
#pragma unroll 4
        for (int q = 0; q < nplanes; ++q) dst[q] = src[(int64_t)q * plane].x * (isw[q] * ic);
    }
}
// complex64 planes -> complex128 (exact)
__global__ void k_widen(const float2 *src, double2 *dst, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = src[i];
        dst[i] = make_double2((double)v.x, (double)v.y);
    }
}
// adjoint of k_crop_correct: one thread per padded-plane cell (k1, k2) of a
// plane batch; cells inside the image window get the scaled image value,
// the others zero (the whole plane is written: no separate clearing pass)
__global__ void k_embed(const void *__restrict__ image, int is_f64, int nplanes, int plane0, int64_t nu, int64_t nv,
                        int64_t nl, int64_t nm, int64_t n_planes_total, const double *__restrict__ sum_weight,
                        const double *__restrict__ correction, float2 *__restrict__ planes) {
    __shared__ double isw[MAX_BATCH];
    __shared__ float iswf[MAX_BATCH];
    stage_inv_sw(sum_weight, plane0, nplanes, isw, iswf);
    const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= nu * nv) return;
    const int64_t k1 = cell / nv, k2 = cell - (cell / nv) * nv;
    // inverse of k = (x - n/2) mod N for x in [0, n)
    int64_t l = k1 + nl / 2, m = k2 + nm / 2;
    if (l >= nu) l -= nu;
    if (m >= nv) m -= nv;
    float2 *__restrict__ dst = planes + cell;
    const int64_t plane = nu * nv;
    if (l >= nl || m >= nm) {
        for (int q = 0; q < nplanes; ++q) dst[(int64_t)q * plane] = make_float2(0.f, 0.f);
        return;
    }
    const int64_t id = l * nm + m;
    const float ic = 1.0f / (float)correction[id];
    const int64_t ii = id * n_planes_total + plane0;
    if (is_f64) {
        const double *__restrict__ x = (const double *)image + ii;
#pragma unroll 4
        for (int q = 0; q < nplanes; ++q) dst[(int64_t)q * plane] = make_float2((float)x[q] * (iswf[q] * ic), 0.f);
    } else {
        const float *__restrict__ x = (const float *)image + ii;
#pragma unroll 4
        for (int q = 0; q < nplanes; ++q) dst[(int64_t)q * plane] = make_float2(x[q] * (iswf[q] * ic), 0.f);
    }
}
}  // namespace

void release_fft_plans() {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    for (auto &kv : g_plans) cufftDestroy(kv.second);
    g_plans.clear();
}

}  // namespace ngg

using namespace ngg;

extern "C" int ngg_fft_correct(void *grid, int64_t n_img, int64_t P, int64_t nu, int64_t nv, int64_t nl, int64_t nm,
                               const double *sum_weight, const double *correction, double *image, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (n_img < 0 || P < 1 || nu < 1 || nv < 1 || nl < 1 || nm < 1 || nl > nu || nm > nv)
        return fail(NGG_ERR_INVALID, "dims (need 1 <= n_l <= n_u, 1 <= n_m <= n_v)");
    if (!grid || !sum_weight || !correction || !image) return fail(NGG_ERR_INVALID, "NULL pointer");
    const int64_t n_planes = n_img * P;
    if (n_planes == 0) return NGG_OK;
    // batch size: bound the per-call working set to ~4 GB of planes
    const int64_t plane_bytes = nu * nv * 8;
    int64_t batch = (4ll << 30) / plane_bytes;
    if (batch < 1) batch = 1;
    if (batch > n_planes) batch = n_planes;
    if (batch > MAX_BATCH) batch = MAX_BATCH;   // the epilogues stage one value per plane of a batch
    float2 *g = (float2 *)grid;
    for (int64_t p0 = 0; p0 < n_planes; p0 += batch) {
        const int nb = (int)((n_planes - p0) < batch ? (n_planes - p0) : batch);
        cufftHandle h;
        int rc = get_plan(nu, nv, nb, &h);
        if (rc != NGG_OK) return rc;
        if (cufftSetStream(h, s) != CUFFT_SUCCESS) return fail(NGG_ERR_CUDA, "cufftSetStream");
        float2 *base = g + p0 * nu * nv;
        if (cufftExecC2C(h, (cufftComplex *)base, (cufftComplex *)base, CUFFT_INVERSE) != CUFFT_SUCCESS)
            return fail(NGG_ERR_CUDA, "cufftExecC2C");
        const int64_t npx = nl * nm;
        k_crop_correct<<<(unsigned)((npx + 255) / 256), 256, 0, s>>>(base, nb, (int)p0, nu, nv, nl, nm, n_planes,
                                                                     sum_weight, correction, image);
        NGG_CHECK_LAUNCH("k_crop_correct");
    }
    return NGG_OK;
}

extern "C" int ngg_fft_correct_f64(const void *grid, int64_t n_img, int64_t P, int64_t nu, int64_t nv, int64_t nl,
                                   int64_t nm, const double *sum_weight, const double *correction, double *image,
                                   void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (n_img < 0 || P < 1 || nu < 1 || nv < 1 || nl < 1 || nm < 1 || nl > nu || nm > nv)
        return fail(NGG_ERR_INVALID, "dims (need 1 <= n_l <= n_u, 1 <= n_m <= n_v)");
    if (!grid || !sum_weight || !correction || !image) return fail(NGG_ERR_INVALID, "NULL pointer");
    const int64_t n_planes = n_img * P;
    if (n_planes == 0) return NGG_OK;
    // complex128 working planes in library scratch, ~2 GB per batch
    const int64_t plane_bytes = nu * nv * 16;
    int64_t batch = (2ll << 30) / plane_bytes;
    if (batch < 1) batch = 1;
    if (batch > n_planes) batch = n_planes;
    if (batch > MAX_BATCH) batch = MAX_BATCH;   // the epilogues stage one value per plane of a batch
    ScratchList sl(s);
    double2 *work = nullptr;
    int rc = sl.get((void **)&work, (size_t)(batch * plane_bytes));
    if (rc != NGG_OK) return rc;
    const float2 *g = (const float2 *)grid;
    for (int64_t p0 = 0; p0 < n_planes; p0 += batch) {
        const int nb = (int)((n_planes - p0) < batch ? (n_planes - p0) : batch);
        const int64_t n = (int64_t)nb * nu * nv;
        k_widen<<<(unsigned)std::min<int64_t>((n + 255) / 256, 65535), 256, 0, s>>>(g + p0 * nu * nv, work, n);
        NGG_CHECK_LAUNCH("k_widen");
        cufftHandle h;
        rc = get_plan(nu, nv, nb, &h, true);
        if (rc != NGG_OK) return rc;
        if (cufftSetStream(h, s) != CUFFT_SUCCESS) return fail(NGG_ERR_CUDA, "cufftSetStream");
        if (cufftExecZ2Z(h, (cufftDoubleComplex *)work, (cufftDoubleComplex *)work, CUFFT_INVERSE) != CUFFT_SUCCESS)
            return fail(NGG_ERR_CUDA, "cufftExecZ2Z");
        const int64_t npx = nl * nm;
        k_crop_correct<<<(unsigned)((npx + 255) / 256), 256, 0, s>>>(work, nb, (int)p0, nu, nv, nl, nm, n_planes,
                                                                     sum_weight, correction, image);
        NGG_CHECK_LAUNCH("k_crop_correct");
    }
    return NGG_OK;
}

extern "C" int ngg_fft_correct_adjoint(const void *image, int is_f64, int64_t n_img, int64_t P, int64_t nu, int64_t nv,
                                       int64_t nl, int64_t nm, const double *sum_weight, const double *correction,
                                       void *grid, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (n_img < 0 || P < 1 || nu < 1 || nv < 1 || nl < 1 || nm < 1 || nl > nu || nm > nv)
        return fail(NGG_ERR_INVALID, "dims (need 1 <= n_l <= n_u, 1 <= n_m <= n_v)");
    if (!grid || !sum_weight || !correction || !image) return fail(NGG_ERR_INVALID, "NULL pointer");
    const int64_t n_planes = n_img * P;
    if (n_planes == 0) return NGG_OK;
    const int64_t plane_bytes = nu * nv * 8;
    int64_t batch = (4ll << 30) / plane_bytes;
    if (batch < 1) batch = 1;
    if (batch > n_planes) batch = n_planes;
    if (batch > MAX_BATCH) batch = MAX_BATCH;   // the epilogues stage one value per plane of a batch
    float2 *g = (float2 *)grid;
    for (int64_t p0 = 0; p0 < n_planes; p0 += batch) {
        const int nb = (int)((n_planes - p0) < batch ? (n_planes - p0) : batch);
        float2 *base = g + p0 * nu * nv;
        const int64_t ncell = nu * nv;
        k_embed<<<(unsigned)((ncell + 255) / 256), 256, 0, s>>>(image, is_f64, nb, (int)p0, nu, nv, nl, nm, n_planes,
                                                                sum_weight, correction, base);
        NGG_CHECK_LAUNCH("k_embed");
        cufftHandle h;
        int rc = get_plan(nu, nv, nb, &h);
        if (rc != NGG_OK) return rc;
        if (cufftSetStream(h, s) != CUFFT_SUCCESS) return fail(NGG_ERR_CUDA, "cufftSetStream");
        if (cufftExecC2C(h, (cufftComplex *)base, (cufftComplex *)base, CUFFT_FORWARD) != CUFFT_SUCCESS)
            return fail(NGG_ERR_CUDA, "cufftExecC2C");
    }
    return NGG_OK;
}
