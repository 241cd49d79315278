// Hogbom CLEAN minor cycle (ngcasa/deconvolution/deconvolve_point_clean.py:
// _clean_jit :174-236 and _abs_image_peaks :303-320).
//
// Per image plane: peak = the pixel of largest |residual| (strictly larger
// than 0 and than every earlier pixel in (l, m) scan order: the first one
// wins ties; NaN is never a peak); stop at a NaN or zero peak; threshold is
// relative to the first peak; while |peak| > threshold*|peak0| and fewer than
// n_iter subtractions: model[peak] += gain*peak and, over the window where the
// PSF (centre = shape // 2) overlaps the image, residual -= s*psf[shifted],
// then find the next peak. s = gain*peak (Hogbom, scale_by_peak != 0) or the
// reference's literal s = gain (its code omits the peak, :216).
//
// GB300: one CTA of 1024 threads per plane; each iteration is one pass over
// the plane in FP64 (the reference's arithmetic, one rounding per operation:
// the results match it bit for bit) that subtracts inside the window and
// tracks each thread's (|r|, first index) maximum, then a block reduction.
// Warp w owns rows x = w (mod 32), lanes the columns (coalesced rows); the
// plane stays in L2 (512^2 FP64 = 2 MB). GB300 runs FP64 at a small fraction
// of FP32, so the peak search compares |value| as the unsigned integer bit
// pattern of the sign-cleared double (for non-negative doubles the same
// order as the values; NaN patterns map to 0, so a NaN is never a peak) and
// only the window subtraction uses the FP64 pipe.
#include "ngg_internal.cuh"

namespace ngg {
namespace {

struct Peak {
    unsigned long long a;   // bits of |value| (see mag_key), 0 when none
    long long i;            // linear index x*ny + y, -1 when none
};

// |v| as an order-preserving integer key; NaN -> 0 (never above a peak)
__device__ __forceinline__ unsigned long long mag_key(double v) {
    const unsigned long long k = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return k > 0x7ff0000000000000ull ? 0ull : k;
}

__device__ __forceinline__ Peak better(Peak p, Peak q) {
    if (q.i < 0) return p;
    if (p.i < 0) return q;
    if (q.a > p.a || (q.a == p.a && q.i < p.i)) return q;
    return p;
}

__device__ __forceinline__ Peak block_peak(Peak p, Peak *s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        Peak q;
        q.a = __shfl_xor_sync(0xffffffffu, p.a, o);
        q.i = __shfl_xor_sync(0xffffffffu, p.i, o);
        p = better(p, q);
    }
    if (lane == 0) s_red[warp] = p;
    __syncthreads();
    if (warp == 0) {
        p = lane < (int)(blockDim.x >> 5) ? s_red[lane] : Peak{0ull, -1};
        for (int o = 16; o > 0; o >>= 1) {
            Peak q;
            q.a = __shfl_xor_sync(0xffffffffu, p.a, o);
            q.i = __shfl_xor_sync(0xffffffffu, p.i, o);
            p = better(p, q);
        }
        if (lane == 0) s_red[32] = p;
    }
    __syncthreads();
    const Peak r = s_red[32];
    __syncthreads();   // s_red is rewritten by the next reduction
    return r;
}

__global__ void __launch_bounds__(1024) k_hogbom(double *residual, const double *psf, double *model, int64_t nx,
                                                 int64_t ny, int64_t px, int64_t py, double gain, double threshold,
                                                 int n_iter, int scale_by_peak, int32_t *iterations) {
    __shared__ Peak s_red[33];
    const int64_t plane = blockIdx.x;
    double *r = residual + plane * nx * ny;
    double *mdl = model + plane * nx * ny;
    const double *ps = psf + plane * px * py;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int64_t pcx = px / 2, pcy = py / 2;

    // first peak
    Peak p{0ull, -1};
    for (int64_t x = warp; x < nx; x += nw)
        for (int64_t y = lane; y < ny; y += 32) {
            const unsigned long long a = mag_key(r[x * ny + y]);
            if (a > p.a) p = Peak{a, x * ny + y};   // scan order within the thread: first wins
        }
    p = block_peak(p, s_red);
    int it = 0;
    if (p.i < 0) it = n_iter;   // nothing above zero: the reference's peak is 0 (or NaN) and it stops
    const double thr = threshold * __longlong_as_double((long long)p.a);
    while (it < n_iter && __longlong_as_double((long long)p.a) > thr) {
        const int64_t x0 = p.i / ny, y0 = p.i - (p.i / ny) * ny;
        const double peak = r[p.i];   // signed value (all threads read it before anyone writes)
        __syncthreads();
        if (threadIdx.x == 0) mdl[p.i] = __dadd_rn(mdl[p.i], __dmul_rn(gain, peak));
        const double s = scale_by_peak ? __dmul_rn(gain, peak) : gain;
        const int64_t sx = max(x0 - pcx, (int64_t)0), ex = min(x0 + (px - pcx), nx);
        const int64_t sy = max(y0 - pcy, (int64_t)0), ey = min(y0 + (py - pcy), ny);
        Peak q{0ull, -1};
        for (int64_t x = warp; x < nx; x += nw) {
            const bool rowin = x >= sx && x < ex;
            for (int64_t y = lane; y < ny; y += 32) {
                double v = r[x * ny + y];
                if (rowin && y >= sy && y < ey) {
                    v = __dsub_rn(v, __dmul_rn(s, ps[(pcx + x - x0) * py + (pcy + y - y0)]));
                    r[x * ny + y] = v;
                }
                const unsigned long long a = mag_key(v);
                if (a > q.a) q = Peak{a, x * ny + y};
            }
        }
        p = block_peak(q, s_red);
        ++it;
        if (p.i < 0) break;   // the new peak is 0 or NaN: the reference sets i = niter
    }
    if (threadIdx.x == 0 && iterations) iterations[plane] = it > n_iter ? n_iter : it;
}

}  // namespace
}  // namespace ngg

using namespace ngg;

extern "C" int ngg_hogbom_clean(double *residual, const double *psf, double *model, int64_t n_planes, int64_t nx,
                                int64_t ny, int64_t px, int64_t py, double gain, double threshold, int n_iter,
                                int scale_by_peak, int32_t *iterations, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (n_planes < 0 || nx < 0 || ny < 0 || px < 1 || py < 1 || n_iter < 0) return fail(NGG_ERR_INVALID, "dims");
    if (n_planes == 0 || nx * ny == 0) return NGG_OK;
    if (!residual || !psf || !model) return fail(NGG_ERR_INVALID, "NULL pointer");
    if (n_planes > 0x7fffffff) return fail(NGG_ERR_UNSUPPORTED, "too many planes");
    k_hogbom<<<(unsigned)n_planes, 1024, 0, s>>>(residual, psf, model, nx, ny, px, py, gain, threshold, n_iter,
                                                 scale_by_peak, iterations);
    NGG_CHECK_LAUNCH("k_hogbom");
    return NGG_OK;
}
