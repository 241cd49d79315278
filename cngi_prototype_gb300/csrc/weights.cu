// Imaging weights: weight-density grid, Briggs factors and nearest-cell lookup.
//
// Reference behaviour:
//  * density grid: _standard_grid_jit with do_psf and do_imaging_weight,
//    support 1, oversampling 0 on the unpadded grid
//    (make_imaging_weight.py:153-161; _standard_grid.py:327-333, 349-369);
//  * calculate_briggs_parms (make_imaging_weight.py:198-213);
//  * _standard_imaging_weight_degrid_jit (_standard_grid.py:466-518).
//
// The density grid is built track by track: one thread follows one
// (baseline, channel) track through time, keeps the weight of the current
// cell (and of the mirrored cell) in a register while the track stays on it,
// and adds it to the plane with one atomic when the track moves on. Lanes of a
// warp take consecutive channels of the same baseline, so weight loads are
// coalesced.
#include "ngg_internal.cuh"

namespace ngg {
namespace {

struct ChanScale {
    double su, sv;
    float suh, sul, svh, svl;
};

__global__ void k_chan_scale(const double *freq, int C, double dl0, double dl1, int64_t nu, int64_t nv,
                             ChanScale *out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    double su, sv;
    uv_scale_dev(freq[c], dl0, dl1, nu, nv, su, sv);
    Split a = split_double(su), b = split_double(sv);
    out[c] = ChanScale{su, sv, a.hi, a.lo, b.hi, b.lo};
}

// uvw rows split into FP32 pairs once per row, baseline-major: uvs[b*T + t]
__global__ void k_split(const double *uvw, int64_t T, int64_t B, float4 *uvs) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= T * B) return;
    const int64_t t = id / B, b = id % B;
    Split a = split_double(uvw[id * 3 + 0]), c = split_double(uvw[id * 3 + 1]);
    uvs[b * T + t] = make_float4(a.hi, a.lo, c.hi, c.lo);
}

// exact nearest cell (support 1) of both coordinates; false if uvw is NaN
__device__ __forceinline__ bool nearest_cell(const double *uvw, const float4 &us, int64_t row, const ChanScale &cs,
                                             int cu_c, int cv_c, bool neg, int &cu, int &cv) {
    if (isnan(us.x) || isnan(us.z)) return false;
    int o;
    if (!cell_pair(us.x, us.y, cs.suh, cs.sul, neg, cu_c, 0, cu, o)) {
        long long i64, o64;
        cell_fp64(uvw[row * 3 + 0], cs.su, neg, cu_c, 0, i64, o64);
        cu = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
    }
    if (!cell_pair(us.z, us.w, cs.svh, cs.svl, neg, cv_c, 0, cv, o)) {
        long long i64, o64;
        cell_fp64(uvw[row * 3 + 1], cs.sv, neg, cv_c, 0, i64, o64);
        cv = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
    }
    return true;
}

__global__ void k_density(const double *uvw, const float4 *uvs, const float *weight, const ChanScale *cs_all, int64_t T, int64_t B,
                          int64_t C, int64_t P, int64_t nu, int64_t nv, int continuum, float *density,
                          double *dsw) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= B * C) return;
    const int64_t b = id / C, c = id % C;
    const ChanScale cs = cs_all[c];
    const int64_t cimg = continuum ? 0 : c;
    float *plane = density + cimg * nu * nv;
    const int cu_c = (int)(nu / 2), cv_c = (int)(nv / 2);
    int64_t cur = -1, curc = -1;
    float acc = 0.f, accc = 0.f;
    float sws = 0.f, swc = 0.f;  // Kahan
    for (int64_t t = 0; t < T; ++t) {
        const int64_t row = t * B + b;
        const int64_t base = (row * C + c) * P;
        float w = P >= 2 ? (weight[base] + weight[base + 1]) * 0.5f : weight[base];
        if (isnan(w) || w == 0.f) continue;
        const float4 us = uvs[b * T + t];
        int cu, cv;
        if (!nearest_cell(uvw, us, row, cs, cu_c, cv_c, false, cu, cv)) continue;
        if (cu < 0 || cu >= nu || cv < 0 || cv >= nv) continue;
        int cuc, cvc;
        nearest_cell(uvw, us, row, cs, cu_c, cv_c, true, cuc, cvc);
        const int64_t cell = (int64_t)cu * nv + cv;
        if (cell != cur) {
            if (cur >= 0) atomicAdd(plane + cur, acc);
            cur = cell;
            acc = 0.f;
        }
        acc += w;
        if (cuc >= 0 && cuc < nu && cvc >= 0 && cvc < nv) {
            const int64_t cc = (int64_t)cuc * nv + cvc;
            if (cc != curc) {
                if (curc >= 0) atomicAdd(plane + curc, accc);
                curc = cc;
                accc = 0.f;
            }
            accc += w;
        }
        // sum_weight receives weight*norm twice (norm = 1)
        for (int k = 0; k < 2; ++k) {
            float y = w - swc;
            float tt = sws + y;
            swc = (tt - sws) - y;
            sws = tt;
        }
    }
    if (cur >= 0) atomicAdd(plane + cur, acc);
    if (curc >= 0) atomicAdd(plane + curc, accc);
    const double v = (double)sws - (double)swc;
    if (v != 0.0) atomicAdd(dsw + cimg, v);
}

__global__ void k_briggs(int weighting, double numer, double robust, double noise, int64_t nuv,
                         const float *density, const double *dsw, double *factors, int64_t n_img) {
    const int64_t c = blockIdx.x;
    __shared__ double red[32];
    double s = 0.0;
    if (weighting == NGG_WEIGHTING_BRIGGS) {
        // sum of W^2 in FP32 pairs (GB300's FP64 rate made the FP64 loop the
        // bound): x*x = p + e exactly (FMA), accumulated by two-sum into
        // (hi, lo): ~48-bit sums at FP32 issue rate, then FP64 across threads
        const float *pl = density + c * nuv;
        float hi = 0.f, lo = 0.f;
        for (int64_t i = threadIdx.x; i < nuv; i += blockDim.x) {
            const float x = pl[i];
            const float p = x * x;
            const float e = fmaf(x, x, -p);
            const float t = hi + p;
            const float bp = t - hi;
            lo += ((hi - (t - bp)) + (p - bp)) + e;
            hi = t;
        }
        s = (double)hi + (double)lo;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
        double f0, f1;
        if (weighting == NGG_WEIGHTING_BRIGGS) {
            f0 = numer / (tot / dsw[c]);
            f1 = 1.0;
        } else if (weighting == NGG_WEIGHTING_BRIGGS_ABS) {
            f0 = robust * robust;
            f1 = 2.0 * noise * noise;
        } else {  // uniform (natural is handled by the caller: weights pass through)
            f0 = 1.0;
            f1 = 0.0;
        }
        factors[c] = f0;
        factors[n_img + c] = f1;
    }
}

__global__ void k_lookup(const double *uvw, const float4 *uvs, const float *weight, const ChanScale *cs_all, int64_t T, int64_t B,
                         int64_t C, int64_t P, int64_t nu, int64_t nv, int continuum, const float *density,
                         const double *factors, int64_t n_img, float *out) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= T * B * C) return;
    const int64_t row = id / C, c = id % C;
    const int64_t base = id * P;
    const ChanScale cs = cs_all[c];
    const int64_t cimg = continuum ? 0 : c;
    int cu, cv;
    const float4 us = uvs[(row % B) * T + row / B];
    bool ok = nearest_cell(uvw, us, row, cs, (int)(nu / 2), (int)(nv / 2), false, cu, cv);
    ok = ok && cu >= 0 && cu < nu && cv >= 0 && cv < nv;
    if (!ok) {
        for (int64_t p = 0; p < P; ++p) out[base + p] = 0.f;
        return;
    }
    const float W = density[(cimg * nu + cu) * nv + cv];
    const float f0 = (float)factors[cimg], f1 = (float)factors[n_img + cimg];
    const bool Wok = !isnan(W) && W != 0.f;
    const float avg = P == 2 ? (weight[base] + weight[base + 1]) * 0.5f : 0.f;
    for (int64_t p = 0; p < P; ++p) {
        const float wp = weight[base + p];
        float iw = P == 2 ? avg : wp;
        if (!isnan(wp) && wp != 0.f && Wok) iw = iw / (f0 * W + f1);
        out[base + p] = iw;
    }
}

int scales(const double *freq, int64_t C, const double dl[2], int64_t nu, int64_t nv, ChanScale **out,
           cudaStream_t s) {
    int rc = scratch_alloc((void **)out, sizeof(ChanScale) * (C > 0 ? C : 1), s);
    if (rc != NGG_OK) return rc;
    if (C > 0) {
        k_chan_scale<<<(unsigned)((C + 127) / 128), 128, 0, s>>>(freq, (int)C, dl[0], dl[1], nu, nv, *out);
        NGG_CHECK_LAUNCH("k_chan_scale");
    }
    return NGG_OK;
}

}  // namespace
}  // namespace ngg

using namespace ngg;

extern "C" int ngg_grid_density(int chan_mode, int64_t T, int64_t B, int64_t C, int64_t P, int64_t nu, int64_t nv,
                                const double delta_lm[2], const double *uvw, const float *weight,
                                const double *freq, float *density, double *dsw, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (chan_mode != NGG_CHAN_CUBE && chan_mode != NGG_CHAN_CONTINUUM) return fail(NGG_ERR_INVALID, "chan_mode");
    if (T < 0 || B < 0 || C < 0 || P < 1 || nu < 1 || nv < 1 || nu > 65535 || nv > 65535)
        return fail(NGG_ERR_INVALID, "dims");
    if (!density || !dsw || !delta_lm) return fail(NGG_ERR_INVALID, "NULL output");
    const int64_t n_img = chan_mode == NGG_CHAN_CONTINUUM ? 1 : C;
    if (n_img == 0) return NGG_OK;
    NGG_CUDA(cudaMemsetAsync(density, 0, sizeof(float) * n_img * nu * nv, s));
    NGG_CUDA(cudaMemsetAsync(dsw, 0, sizeof(double) * n_img, s));
    if (T * B * C == 0) return NGG_OK;
    if (!uvw || !weight || !freq) return fail(NGG_ERR_INVALID, "NULL input");
    ChanScale *cs = nullptr;
    int rc = scales(freq, C, delta_lm, nu, nv, &cs, s);
    if (rc != NGG_OK) return rc;
    float4 *uvs = nullptr;
    if ((rc = scratch_alloc((void **)&uvs, sizeof(float4) * T * B, s)) != NGG_OK) { scratch_free(cs, s); return rc; }
    k_split<<<(unsigned)((T * B + 255) / 256), 256, 0, s>>>(uvw, T, B, uvs);
    const int64_t n = B * C;
    k_density<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(uvw, uvs, weight, cs, T, B, C, P, nu, nv,
                                                          chan_mode == NGG_CHAN_CONTINUUM, density, dsw);
    cudaError_t e = cudaGetLastError();
    scratch_free(uvs, s);
    scratch_free(cs, s);
    if (e != cudaSuccess) return cuda_fail(e, "k_density");
    return NGG_OK;
}

extern "C" int ngg_briggs_factors(int weighting, double robust, double noise, int64_t n_img, int64_t nu, int64_t nv,
                                  const float *density, const double *dsw, double *factors, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (weighting != NGG_WEIGHTING_UNIFORM && weighting != NGG_WEIGHTING_BRIGGS && weighting != NGG_WEIGHTING_BRIGGS_ABS)
        return fail(NGG_ERR_INVALID, "weighting must be uniform, briggs or briggs_abs");
    if (n_img < 0 || nu < 1 || nv < 1) return fail(NGG_ERR_INVALID, "dims");
    if (n_img == 0) return NGG_OK;
    if (!factors || (weighting == NGG_WEIGHTING_BRIGGS && (!density || !dsw))) return fail(NGG_ERR_INVALID, "NULL");
    // np.square(5.0*10.0**(-robust)), evaluated on the host as Python does
    const double x = 5.0 * pow(10.0, -robust);
    const double numer = x * x;
    k_briggs<<<(unsigned)n_img, 1024, 0, s>>>(weighting, numer, robust, noise, nu * nv, density, dsw, factors, n_img);
    NGG_CHECK_LAUNCH("k_briggs");
    return NGG_OK;
}

extern "C" int ngg_weight_lookup(int chan_mode, int64_t T, int64_t B, int64_t C, int64_t P, int64_t nu, int64_t nv,
                                 const double delta_lm[2], const double *uvw, const float *weight, const double *freq,
                                 const float *density, const double *factors, float *out, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (chan_mode != NGG_CHAN_CUBE && chan_mode != NGG_CHAN_CONTINUUM) return fail(NGG_ERR_INVALID, "chan_mode");
    if (T < 0 || B < 0 || C < 0 || P < 1 || nu < 1 || nv < 1 || nu > 65535 || nv > 65535)
        return fail(NGG_ERR_INVALID, "dims");
    if (T * B * C == 0) return NGG_OK;
    if (!uvw || !weight || !freq || !density || !factors || !out || !delta_lm) return fail(NGG_ERR_INVALID, "NULL");
    ChanScale *cs = nullptr;
    int rc = scales(freq, C, delta_lm, nu, nv, &cs, s);
    if (rc != NGG_OK) return rc;
    float4 *uvs = nullptr;
    if ((rc = scratch_alloc((void **)&uvs, sizeof(float4) * T * B, s)) != NGG_OK) { scratch_free(cs, s); return rc; }
    k_split<<<(unsigned)((T * B + 255) / 256), 256, 0, s>>>(uvw, T, B, uvs);
    const int64_t n = T * B * C;
    const int64_t n_img = chan_mode == NGG_CHAN_CONTINUUM ? 1 : C;
    k_lookup<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(uvw, uvs, weight, cs, T, B, C, P, nu, nv,
                                                         chan_mode == NGG_CHAN_CONTINUUM, density, factors, n_img, out);
    cudaError_t e = cudaGetLastError();
    scratch_free(uvs, s);
    scratch_free(cs, s);
    if (e != cudaSuccess) return cuda_fail(e, "k_lookup");
    return NGG_OK;
}
