// Direction rotation: uvw rotation and visibility phase rotation to a new
// phase centre (ngcasa/imaging/direction_rotate.py).
//
// Reference behaviour:
//   apply_rotation_matrix (:189-211): uvw_rot[t,b,:] = uvw[t,b,:] @ M[f(t)]
//     (row vector times the field's 3x3 matrix; f(t) the one field of time row t)
//   apply_phasor (:215-248): pd[t,b] = uvw_rot[t,b,0:k] . R[f(t),0:k]
//     (k = 2 with common tangent reprojection, else 3);
//     vis_rot = vis * exp(2 pi i pd f / c), in FP64; with single_precision the
//     product is rounded to complex64.
// GB300: one thread per (time, baseline) row for the rotation (FP64, 48 B per
// row), one thread per (time, baseline, channel) for the phasor. GB300 runs
// FP64 at a small fraction of FP32, so for the complex64 output the phase
// pd*f/c is formed from (hi, lo) FP32 pairs of pd (per row) and f/c (per
// channel): an error-free FP32 product of the high parts plus the cross
// terms, reduced to a fraction of a turn r = rh + rl by rint of the high
// product and an exact two-sum (error < 2e-9 turns while |pd*f/c| < 2^22
// turns; larger phases, and NaN, take the FP64 reduction), then
// sincospif(2 rh) corrected by the first-order term of 2 pi rl: error ~1e-7,
// inside the complex64 rounding the reference applies. Two pols move as one
// 16-byte access. The complex128 output reduces and evaluates in FP64.
#include "ngg_internal.cuh"

namespace ngg {
namespace {

__global__ void k_rotate_uvw(const double *uvw, const int32_t *row_field, int64_t T, int64_t B,
                             const double *mats, const double *phase, int n_field, int k, double *uvw_rot,
                             double *pd) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T * B) return;
    const int64_t t = i / B;
    const int f = row_field[t];
    if (f < 0 || f >= n_field) return;   // checked on the host
    const double *m = mats + 9 * f;
    const double x = uvw[3 * i], y = uvw[3 * i + 1], z = uvw[3 * i + 2];
    double r[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) r[j] = __dadd_rn(__dadd_rn(__dmul_rn(x, m[j]), __dmul_rn(y, m[3 + j])), __dmul_rn(z, m[6 + j]));
    uvw_rot[3 * i] = r[0];
    uvw_rot[3 * i + 1] = r[1];
    uvw_rot[3 * i + 2] = r[2];
    const double *ph = phase + 3 * f;
    double d = __dadd_rn(__dmul_rn(r[0], ph[0]), __dmul_rn(r[1], ph[1]));
    if (k == 3) d = __dadd_rn(d, __dmul_rn(r[2], ph[2]));
    pd[i] = d;
}

// (hi, lo) FP32 pair of each FP64 value
__global__ void k_split_pairs(const double *x, int64_t n, float2 *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Split a = split_double(x[i]);
    out[i] = make_float2(a.hi, a.lo);
}

// phasor (cos, sin) of the phase pd[row] * f_over_c[c] (see the header)
__device__ __forceinline__ void phasor_f32(const double *__restrict__ pd, float2 a, const double *__restrict__ f_over_c,
                                           float2 f, int64_t row, int64_t c, float &pc, float &ps) {
    const float p1 = __fmul_rn(a.x, f.x);
    float rh, rl;
    if (fabsf(p1) < 4194304.0f) {
        const float e1 = fmaf(a.x, f.x, -p1);                // a.x*f.x = p1 + e1 exactly
        const float cr = fmaf(a.x, f.y, fmaf(a.y, f.x, e1));  // cross terms (a.y*f.y < 2^-48 |p|)
        const float fr = __fsub_rn(p1, rintf(p1));           // exact
        two_sum(fr, cr, rh, rl);
    } else {   // large phase or NaN: the FP64 reduction
        const double cyc = pd[row] * f_over_c[c];
        const double r = cyc - rint(cyc);
        rh = (float)r;
        rl = (float)(r - (double)rh);
    }
    float s, co;
    sincospif(2.0f * rh, &s, &co);
    const float dl = 6.28318531f * rl;   // |dl| < 2e-7: first order suffices
    ps = fmaf(co, dl, s);
    pc = fmaf(-s, dl, co);
}

// complex64 output. VEC2 (two pols, 16-byte aligned arrays): a block covers
// PER * blockDim.x consecutive (row, chan) elements, each thread PER of
// them a block width apart, all loads issued before any use (one 16-byte
// load per thread cannot keep enough bytes in flight to saturate HBM).
constexpr int PER = 4;
template <bool VEC2, bool IDX32>
__global__ void k_phasor_f32(const float2 *__restrict__ vis, const double *__restrict__ pd,
                             const float2 *__restrict__ pdp, int64_t TB, int64_t C, int64_t P,
                             const double *__restrict__ f_over_c, const float2 *__restrict__ focp,
                             float2 *__restrict__ out) {
    const int64_t n = TB * C;
    if constexpr (VEC2) {
        const int64_t i0 = (int64_t)blockIdx.x * blockDim.x * PER + threadIdx.x;
        // every load of the thread's PER elements is issued before any store
        float4 v[PER];
        float2 a[PER], f[PER];
        int64_t row[PER], c[PER];
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int64_t i = i0 + (int64_t)k * blockDim.x;
            if (i < n) {
                if (IDX32) {   // n < 2^31: 32-bit division (the 64-bit one is a long instruction sequence)
                    const unsigned r32 = (unsigned)i / (unsigned)C;
                    row[k] = r32;
                    c[k] = (int64_t)((unsigned)i - r32 * (unsigned)C);
                } else {
                    row[k] = i / C;
                    c[k] = i - row[k] * C;
                }
                v[k] = reinterpret_cast<const float4 *>(vis)[i];
                a[k] = pdp[row[k]];
                f[k] = focp[c[k]];
            }
        }
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int64_t i = i0 + (int64_t)k * blockDim.x;
            if (i >= n) break;
            float pc, ps;
            phasor_f32(pd, a[k], f_over_c, f[k], row[k], c[k], pc, ps);
            reinterpret_cast<float4 *>(out)[i] =
                make_float4(fmaf(v[k].x, pc, -v[k].y * ps), fmaf(v[k].x, ps, v[k].y * pc),
                            fmaf(v[k].z, pc, -v[k].w * ps), fmaf(v[k].z, ps, v[k].w * pc));
        }
    } else {
        const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n) return;
        const int64_t row = i / C, c = i - row * C;
        float pc, ps;
        phasor_f32(pd, pdp[row], f_over_c, focp[c], row, c, pc, ps);
        const float2 *v = vis + i * P;
        float2 *o = out + i * P;
        for (int p = 0; p < P; ++p) {
            const float2 x = v[p];
            o[p] = make_float2(fmaf(x.x, pc, -x.y * ps), fmaf(x.x, ps, x.y * pc));
        }
    }
}

// complex128 output: reduction and phasor in FP64
__global__ void k_phasor_f64(const float2 *vis, const double *pd, int64_t TB, int64_t C, int64_t P,
                             const double *f_over_c, double2 *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= TB * C) return;
    const int64_t row = i / C, c = i - row * C;
    const double cyc = pd[row] * f_over_c[c];
    const double r = cyc - rint(cyc);   // [-1/2, 1/2] of a turn
    double s, co;
    sincospi(2.0 * r, &s, &co);
    const float2 *v = vis + i * P;
    double2 *o = out + i * P;
    for (int p = 0; p < P; ++p) {
        const double ax = v[p].x, ay = v[p].y;
        o[p] = make_double2(ax * co - ay * s, ax * s + ay * co);
    }
}

}  // namespace
}  // namespace ngg

using namespace ngg;

extern "C" int ngg_rotate_uvw(const double *uvw, const int32_t *row_field, int64_t n_time, int64_t n_baseline,
                              const double *rotmat, const double *phase_rotation, int n_field,
                              int common_tangent_reprojection, double *uvw_rot, double *phase_dir, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (n_time < 0 || n_baseline < 0 || n_field < 0) return fail(NGG_ERR_INVALID, "negative dims");
    const int64_t n = n_time * n_baseline;
    if (n == 0) return NGG_OK;
    if (!uvw || !row_field || !rotmat || !phase_rotation || !uvw_rot || !phase_dir || n_field < 1)
        return fail(NGG_ERR_INVALID, "NULL pointer or no field");
    k_rotate_uvw<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(uvw, row_field, n_time, n_baseline, rotmat,
                                                             phase_rotation, n_field,
                                                             common_tangent_reprojection ? 2 : 3, uvw_rot, phase_dir);
    NGG_CHECK_LAUNCH("k_rotate_uvw");
    return NGG_OK;
}

extern "C" int ngg_phase_rotate(const void *vis, const double *phase_dir, int64_t n_time, int64_t n_baseline,
                                int64_t n_chan, int64_t n_pol, const double *freq_over_c, int single_precision,
                                void *vis_rot, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (n_time < 0 || n_baseline < 0 || n_chan < 0 || n_pol < 1) return fail(NGG_ERR_INVALID, "dims");
    const int64_t n = n_time * n_baseline * n_chan;
    if (n == 0) return NGG_OK;
    if (!vis || !phase_dir || !freq_over_c || !vis_rot) return fail(NGG_ERR_INVALID, "NULL pointer");
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (single_precision) {
        const int64_t TB = n_time * n_baseline;
        float2 *pairs = nullptr;
        int rc = scratch_alloc((void **)&pairs, sizeof(float2) * (size_t)(TB + n_chan), s);
        if (rc != NGG_OK) return rc;
        k_split_pairs<<<(unsigned)((TB + 255) / 256), 256, 0, s>>>(phase_dir, TB, pairs);
        k_split_pairs<<<(unsigned)((n_chan + 255) / 256), 256, 0, s>>>(freq_over_c, n_chan, pairs + TB);
        const bool vec2 = n_pol == 2 && ((uintptr_t)vis % 16 == 0) && ((uintptr_t)vis_rot % 16 == 0);
        const unsigned vblocks = (unsigned)((n + 256 * PER - 1) / (256 * PER));
        if (vec2 && n < ((int64_t)1 << 31))
            k_phasor_f32<true, true><<<vblocks, 256, 0, s>>>((const float2 *)vis, phase_dir, pairs, TB, n_chan, n_pol,
                                                             freq_over_c, pairs + TB, (float2 *)vis_rot);
        else if (vec2)
            k_phasor_f32<true, false><<<vblocks, 256, 0, s>>>((const float2 *)vis, phase_dir, pairs, TB, n_chan,
                                                              n_pol, freq_over_c, pairs + TB, (float2 *)vis_rot);
        else
            k_phasor_f32<false, false><<<blocks, 256, 0, s>>>((const float2 *)vis, phase_dir, pairs, TB, n_chan, n_pol,
                                                       freq_over_c, pairs + TB, (float2 *)vis_rot);
        cudaError_t e = cudaGetLastError();
        scratch_free(pairs, s);
        if (e != cudaSuccess) return cuda_fail(e, "k_phasor_f32");
        return NGG_OK;
    }
    k_phasor_f64<<<blocks, 256, 0, s>>>((const float2 *)vis, phase_dir, n_time * n_baseline, n_chan, n_pol,
                                        freq_over_c, (double2 *)vis_rot);
    NGG_CHECK_LAUNCH("k_phasor_f64");
    return NGG_OK;
}
