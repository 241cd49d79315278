// Internal helpers shared by the libngg translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "ngg.h"

namespace ngg {

constexpr double kCLight = 299792458.0;

// ---- error reporting (thread-local last message) -------------------------
void set_error(const std::string &msg);
void clear_error();
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define NGG_CUDA(call)                                           \
    do {                                                         \
        cudaError_t _e = (call);                                 \
        if (_e != cudaSuccess) return ::ngg::cuda_fail(_e, #call); \
    } while (0)
#define NGG_CHECK_LAUNCH(name)                                    \
    do {                                                          \
        cudaError_t _e = cudaGetLastError();                      \
        if (_e != cudaSuccess) return ::ngg::cuda_fail(_e, name); \
    } while (0)

// Stream-ordered scratch allocation from the device's default memory pool.
// The pool keeps freed blocks (release threshold = max), so steady-state calls
// do not reach the driver allocator.
int scratch_alloc(void **p, size_t bytes, cudaStream_t s);
void scratch_free(void *p, cudaStream_t s);

int num_sms();

// Scratch blocks released (stream-ordered) when the list goes out of scope.
struct ScratchList {
    void *p[32];
    int n = 0;
    cudaStream_t s;
    explicit ScratchList(cudaStream_t st) : s(st) {}
    int get(void **out, size_t bytes) {
        if (n == 32) return fail(NGG_ERR_INVALID, "too many scratch blocks");
        int rc = scratch_alloc(out, bytes, s);
        if (rc == NGG_OK) p[n++] = *out;
        return rc;
    }
    ~ScratchList() {
        for (int i = 0; i < n; ++i) scratch_free(p[i], s);
    }
    ScratchList(const ScratchList &) = delete;
    ScratchList &operator=(const ScratchList &) = delete;
};

// ---- exact reproduction of the reference's FP64 index arithmetic ---------
//
// The reference computes, in FP64 with one rounding per operation
// (_standard_grid.py:273-276, 299-324):
//     s      = -(f * dl * N) / c                    (per channel)
//     u      = uvw_u * s
//     u_pos  = u + C                                (C = N // 2)
//     idx    = int(u_pos + 0.5)                     (truncation toward zero)
//     off    = floor((idx - u_pos) * os + 0.5)
// GB300 executes FP64 at ~1.6 instructions/clock/SM, far too slow to do this
// per visibility. Instead the chain is evaluated in FP32 pairs (error-free
// products and sums, relative error ~1e-14), and a result is accepted only
// when the pair estimate is farther than a certified margin from the
// rounding boundary; then the FP64 chain rounds to the same integer. Near a
// boundary (probability ~1e-7) the FP64 chain itself is evaluated.

struct Split { float hi, lo; };

__host__ __device__ inline Split split_double(double x) {
    Split s;
    s.hi = (float)x;
    s.lo = (float)(x - (double)s.hi);
    return s;
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// floor of (h + l) for |h| < 2^22 with |l| << 1. Returns false when the value
// is within `margin` of an integer (then the caller falls back to FP64).
__device__ __forceinline__ bool floor_pair(float h, float l, float margin, int &f, float &fr_h, float &fr_l) {
    float fl = floorf(h);
    float a = __fsub_rn(h, fl);            // exact fractional part of h
    float d_lo = __fadd_rn(a, l);          // distance above fl (accurate near 0)
    float d_hi = __fsub_rn(__fsub_rn(1.0f, a), l);  // distance below fl+1 (accurate near 0)
    int fi = (int)fl;
    if (d_lo < 0.0f) { fi -= 1; a = __fadd_rn(a, 1.0f); }
    else if (d_hi < 0.0f) { fi += 1; a = __fsub_rn(a, 1.0f); }
    f = fi;
    fr_h = a;
    fr_l = l;
    return fabsf(d_lo) > margin && fabsf(d_hi) > margin;
}

// Nearest cell and oversampling offset of one coordinate.
//   p = x * s as an unevaluated pair (ph + pl); neg flips the sign (the
//   mirrored position -u + C of the weight-density mode).
// Returns false if the pair estimate cannot certify the FP64 result.
__device__ __forceinline__ bool cell_pair(float xh, float xl, float sh, float sl, bool neg,
                                          int center, int os, int &idx, int &off) {
    float ph = __fmul_rn(xh, sh);
    float pe = fmaf(xh, sh, -ph);
    float pl = fmaf(xh, sl, fmaf(xl, sh, pe));
    if (neg) { ph = -ph; pl = -pl; }
    if (!(fabsf(ph) < 65536.0f)) return false;   // margin analysis holds below 2^16; also catches NaN
    float th, te;
    two_sum(ph, (float)center + 0.5f, th, te);      // t = u_pos + 0.5
    float tl = __fadd_rn(te, pl);
    int fl;
    float fr_h, fr_l;
    if (!floor_pair(th, tl, 1e-8f, fl, fr_h, fr_l)) return false;
    // int() truncates toward zero: for t < 0 (non-integer) that is floor + 1
    idx = fl >= 0 ? fl : fl + 1;
    if (os == 0) { off = 0; return true; }   // floor(x*0 + 0.5) = 0
    // off_real = idx - u_pos = (idx - fl + 0.5) - (fr_h + fr_l)
    float oh = __fsub_rn((float)(idx - fl) + 0.5f, fr_h);   // exact for |t| >= 1
    if (!(fabsf(th) >= 1.0f)) return false;
    float ol = -fr_l;
    float osf = (float)os;
    float qh = __fmul_rn(oh, osf);
    float qe = fmaf(oh, osf, -qh);
    float ql = fmaf(ol, osf, qe);
    float rh, re;
    two_sum(qh, 0.5f, rh, re);
    float rl = __fadd_rn(re, ql);
    int of;
    float a, b;
    if (!floor_pair(rh, rl, 1e-8f * osf + 1e-7f, of, a, b)) return false;
    off = of;
    return true;
}

// The same chain with one certified floor instead of two (gridding, where
// os >= 1). With G = (u_pos + 0.5) * os the cell is floor(G / os) (=
// trunc(u_pos + 0.5) for u_pos >= 0) and the offset is
//     floor((idx - u_pos) * os + 0.5) = idx * os + floor((os + 1) / 2 - G),
// and both change value only where 2G crosses an integer. 2G = P + K with
// P = x * (2 os s) and the integer K = (2 C + 1) os, so one pair estimate of
// P, certified to lie farther from every integer than the margins of
// cell_pair (scaled to 2G: 1e-8 cells is 2e-8 os, 1e-8 os + 1e-7 offset
// units is twice that) plus its own error bound (3e-14 |P|), gives both
// results: with H = K + floor(P),
//     idx = floor(floor(H / 2) / os),  off = idx * os + floor((os - H) / 2).
// floor(P) = r - (d < 0) with r = rint(ph) and d = (ph - r) + pl, the
// signed distance of P from r (ph - r is exact). (s2h, s2l) = 2 os s as a
// pair (scale_pair); the division by os is a multiplication by
// osm = ceil(2^40 / os), exact for H < 2^25 and os < 2^16. margin0 =
// 2e-8 os + 2e-7. Returns false unless |ph| < 2^24, 1 <= H < 2^24 and the
// estimate is certified (the caller then uses cell_pair).
__device__ __forceinline__ bool cell_half(float xh, float xl, float s2h, float s2l, int K, int os,
                                          unsigned long long osm, float margin0, int &idx, int &off) {
    const float ph = __fmul_rn(xh, s2h);
    const float pe = fmaf(xh, s2h, -ph);
    const float pl = fmaf(xh, s2l, fmaf(xl, s2h, pe));
    if (!(fabsf(ph) < 16777216.0f)) return false;   // also NaN
    const float r = rintf(ph);
    const float d = __fadd_rn(__fsub_rn(ph, r), pl);
    if (!(fabsf(d) > fmaf(3e-14f, fabsf(ph), margin0))) return false;
    const int h = K + (int)r - (d < 0.0f ? 1 : 0);
    if (h < 1 || h >= (1 << 24)) return false;
    const int q = (int)(((unsigned long long)(unsigned)(h >> 1) * osm) >> 40);
    idx = q;
    off = q * os + ((os - h) >> 1);
    return true;
}

// cell_half's host-side constants: ceil(2^40 / os), so that floor(g / os) =
// (g * os_magic(os)) >> 40 for g < 2^24 and 1 <= os < 2^16; and its margin
inline unsigned long long os_magic(int os) {
    return os >= 1 ? ((1ull << 40) + (unsigned long long)os - 1) / (unsigned long long)os : 0ull;
}
inline float half_margin(int os) { return 2e-8f * (float)os + 2e-7f; }

// (h, l) ~ (sh + sl) * f for a small integer f (error ~2^-47 relative)
__device__ __forceinline__ void scale_pair(float sh, float sl, float f, float &h, float &l) {
    h = __fmul_rn(sh, f);
    l = fmaf(sl, f, fmaf(sh, f, -h));
}

// The FP64 chain, operation for operation (used near rounding boundaries).
static __device__ __noinline__ void cell_fp64(double x, double s, bool neg, int center, int os, long long &idx,
                                       long long &off) {
    double u = __dmul_rn(x, s);
    if (neg) u = -u;
    double u_pos = __dadd_rn(u, (double)center);
    double t = __dadd_rn(u_pos, 0.5);
    long long i = __double2ll_rz(t);
    idx = i;
    double o = __dsub_rn((double)i, u_pos);
    double r = __dadd_rn(__dmul_rn(o, (double)os), 0.5);
    off = (long long)floor(r);
}

// Host-side uv scale with the reference's operation order.
inline void uv_scale_host(double f, const double dl[2], int64_t nu, int64_t nv, double &su, double &sv) {
    volatile double a = f * dl[0];
    volatile double b = a * (double)nu;
    su = (-b) / kCLight;
    volatile double c2 = f * dl[1];
    volatile double d = c2 * (double)nv;
    sv = (-d) / kCLight;
}

__device__ __forceinline__ void uv_scale_dev(double f, double dl0, double dl1, int64_t nu, int64_t nv,
                                             double &su, double &sv) {
    su = __ddiv_rn(-__dmul_rn(__dmul_rn(f, dl0), (double)nu), kCLight);
    sv = __ddiv_rn(-__dmul_rn(__dmul_rn(f, dl1), (double)nv), kCLight);
}

}  // namespace ngg
