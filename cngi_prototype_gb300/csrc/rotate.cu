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
// FP64 at a small fraction of FP32, so the phase is reduced in FP64 to a
// fraction of a turn r = pd*f/c - rint(pd*f/c) and, for the complex64 output,
// the phasor is evaluated in FP32 from r split into hi + lo parts
// (sincospif(2 hi), corrected by the first-order term of 2 pi lo): error
// ~1e-7, inside the complex64 rounding the reference applies. The complex128
// output evaluates sincospi in FP64.
#include "ngg_internal.cuh"

namespace ngg {
namespace {

constexpr double C_LIGHT = 299792458.0;

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

template <bool SINGLE>
__global__ void k_phasor(const float2 *vis, const double *pd, int64_t TB, int64_t C, int64_t P,
                         const double *f_over_c, void *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= TB * C) return;
    const int64_t row = i / C, c = i - row * C;
    const double cyc = pd[row] * f_over_c[c];
    const double r = cyc - rint(cyc);   // [-1/2, 1/2] of a turn
    const float2 *v = vis + i * P;
    if constexpr (SINGLE) {
        const float rh = (float)r;
        const float rl = (float)(r - (double)rh);
        float s, co;
        sincospif(2.0f * rh, &s, &co);
        const float dl = 6.28318531f * rl;   // |dl| < 2e-7: first order suffices
        const float ps = fmaf(co, dl, s), pc = fmaf(-s, dl, co);
        float2 *o = reinterpret_cast<float2 *>(out) + i * P;
        for (int p = 0; p < P; ++p) {
            const float2 a = v[p];
            o[p] = make_float2(fmaf(a.x, pc, -a.y * ps), fmaf(a.x, ps, a.y * pc));
        }
    } else {
        double s, co;
        sincospi(2.0 * r, &s, &co);
        double2 *o = reinterpret_cast<double2 *>(out) + i * P;
        for (int p = 0; p < P; ++p) {
            const double ax = v[p].x, ay = v[p].y;
            o[p] = make_double2(ax * co - ay * s, ax * s + ay * co);
        }
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
    if (single_precision)
        k_phasor<true><<<blocks, 256, 0, s>>>((const float2 *)vis, phase_dir, n_time * n_baseline, n_chan, n_pol,
                                              freq_over_c, vis_rot);
    else
        k_phasor<false><<<blocks, 256, 0, s>>>((const float2 *)vis, phase_dir, n_time * n_baseline, n_chan, n_pol,
                                               freq_over_c, vis_rot);
    NGG_CHECK_LAUNCH("k_phasor");
    return NGG_OK;
}
