// Mosaic (aperture-projection) gridding with a gridding-convolution-function
// table, the mosaic weight grid, and GCF generation.
//
// Reference behaviour:
//  * _aperture_grid_jit (ngcasa/imaging/_imaging_utils/_aperture_grid.py:376-513):
//    per row, the field's table conv_kernel * phase_gradient[field]; per
//    visibility the (support x support) taps
//    table[cfb, cfc, cfp, os*iu + off_u + R/2, os*iv + off_v + R/2] times the
//    weighted datum added to the grid; sum_weight += w*Re(norm^2) (image) or
//    w*Re(norm) (PSF); rows skipped if any cell within max(support) of the
//    centre is off the grid.
//  * _aperture_weight_grid_jit (:180-291): the weight table placed at the
//    grid centre for every visibility.
//  * make_gridding_convolution_function.py:181-246 + _make_pb_symmetric.py:
//    Airy voltage patterns per antenna pair, FFT, real part.
//
// GB300 design of ngg_grid_gcf: one warp per (channel, baseline, 32-step
// chunk, pol), channel-major so the atomics of consecutive warps stay in one
// L2-resident channel grid. A lane owns one column residue class (Romein)
// and keeps the support's rows of its current column in registers (natural
// order, shifted when the track moves a row), flushing a cell with an atomic
// add when it leaves. The table is reorganised by oversampling-offset class
// (each lane reads one contiguous run of taps per visibility) and the phase
// gradient, exp(i(x px + y py)), is applied separably from per-field x and y
// tables; the per-(field, CF, offset) tap sums used for sum_weight are
// precomputed in FP64.
#include <cufft.h>

#include <vector>

#include "ngg_internal.cuh"
#include "gcf_grid.cuh"
#include "mlp.cuh"

namespace ngg {
namespace {




__global__ void k_gchan(const double *freq, int C, double dl0, double dl1, int64_t nu, int64_t nv, GChan *out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    double su, sv;
    uv_scale_dev(freq[c], dl0, dl1, nu, nv, su, sv);
    Split a = split_double(su), b = split_double(sv);
    out[c] = GChan{su, sv, a.hi, a.lo, b.hi, b.lo};
}

__global__ void k_gsplit(const double *uvw, int64_t n, float4 *uvs) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    Split a = split_double(uvw[id * 3 + 0]), c = split_double(uvw[id * 3 + 1]);
    uvs[id] = make_float4(a.hi, a.lo, c.hi, c.lo);
}

__device__ __forceinline__ bool in_support(int i, int s) { return i >= -(s / 2) && i < s - s / 2; }

// ckt[cf][ou][ov][r][col]: tap row r in [0, 2S) holds dv + S/2 = r mod S (each
// row stored twice, so a rotated run of S rows is contiguous), col = du + S/2
// in [0, 32) (one per lane); zero outside the CF's support and for col >= S
__global__ void k_reorg(const double *ck, int64_t ncf, int64_t R0, int64_t R1, int os0, int os1, const int32_t *support,
                        int S, float *ckt) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = ncf * (os0 + 1) * (os1 + 1) * 2 * S * SP;
    if (id >= n) return;
    int64_t r = id;
    const int col = (int)(r % SP); r /= SP;
    const int row = (int)(r % (2 * S)); r /= 2 * S;
    const int ov_i = (int)(r % (os1 + 1)); r /= (os1 + 1);
    const int ou_i = (int)(r % (os0 + 1)); r /= (os0 + 1);
    const int64_t cf = r;
    const int sc = S / 2;
    const int iu = col - sc, iv = row % S - sc;
    const int ou = ou_i - os0 / 2, ov = ov_i - os1 / 2;
    float val = 0.f;
    if (col < S && in_support(iu, support[cf * 2 + 0]) && in_support(iv, support[cf * 2 + 1])) {
        const int64_t x = (int64_t)os0 * iu + ou + R0 / 2, y = (int64_t)os1 * iv + ov + R1 / 2;
        if (x >= 0 && x < R0 && y >= 0 && y < R1) val = (float)ck[(cf * R0 + x) * R1 + y];
    }
    ckt[id] = val;
}

// Phase gradient factored by grid position: the tap at table offset
// x' = os0*(u - cu) + ou has phase x' px = os0 u px + ou px - os0 cu px, so a
// visibility carries Hx[ou] conj(Gx[cu]) (and the same in v) and a grid cell
// u is rotated by Gx[u] when it is flushed. Gx[f][u] = e^{i os0 u px_f},
// Hx[f][oi] = e^{i (oi - os0/2) px_f}; arguments in FP64.
__global__ void k_cell_phase(const double *slope, int nf, int64_t nu, int64_t nv, int os0, int os1, float2 *gx,
                             float2 *gy, float2 *hx, float2 *hy) {
    const int64_t per = nu + nv + (os0 + 1) + (os1 + 1);
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (int64_t)nf * per) return;
    const int64_t f = id / per;
    int64_t x = id % per;
    const double px = slope[f * 2 + 0], py = slope[f * 2 + 1];
    double s, c;
    if (x < nu) {
        sincos((double)os0 * (double)x * px, &s, &c);
        gx[f * nu + x] = make_float2((float)c, (float)s);
        return;
    }
    x -= nu;
    if (x < nv) {
        sincos((double)os1 * (double)x * py, &s, &c);
        gy[f * nv + x] = make_float2((float)c, (float)s);
        return;
    }
    x -= nv;
    if (x < os0 + 1) {
        sincos((double)(x - os0 / 2) * px, &s, &c);
        hx[f * (os0 + 1) + x] = make_float2((float)c, (float)s);
        return;
    }
    x -= os0 + 1;
    sincos((double)(x - os1 / 2) * py, &s, &c);
    hy[f * (os1 + 1) + x] = make_float2((float)c, (float)s);
}

// per-field FP64 phase tables for the tap sums: ex[f][x] = exp(i (x - R0/2) px_f),
// ey likewise
__global__ void k_phase_tabs(const double *slope, int nf, int64_t R0, int64_t R1, double2 *ex64, double2 *ey64) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (int64_t)nf * (R0 + R1)) return;
    const int64_t f = id / (R0 + R1), x = id % (R0 + R1);
    double s, c;
    if (x < R0) {
        sincos((double)(x - R0 / 2) * slope[f * 2 + 0], &s, &c);
        ex64[f * R0 + x] = make_double2(c, s);
    } else {
        sincos((double)(x - R0 - R1 / 2) * slope[f * 2 + 1], &s, &c);
        ey64[f * R1 + (x - R0)] = make_double2(c, s);
    }
}

// nrm[f][cf][ou][ov] = sum over the CF's support of table * phase (FP64; the
// phase exp(i(x px + y py)) = ex[x] ey[y]); centre_only: the zero offset only
// (the weight grid's taps)
__global__ void k_norms(const double *ck, const int32_t *support, const double2 *ex64, const double2 *ey64, int nf,
                        int64_t ncf, int64_t R0, int64_t R1, int os0, int os1, int centre_only, double2 *nrm) {
    const int64_t no = centre_only ? 1 : (int64_t)(os0 + 1) * (os1 + 1);
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nf * ncf * no) return;
    const int64_t f = id / (ncf * no), cf = (id / no) % ncf, o = id % no;
    const int ou = centre_only ? 0 : (int)(o / (os1 + 1)) - os0 / 2;
    const int ov = centre_only ? 0 : (int)(o % (os1 + 1)) - os1 / 2;
    const int su = support[cf * 2], sv = support[cf * 2 + 1];
    double re = 0.0, im = 0.0;
    for (int iv = -(sv / 2); iv < sv - sv / 2; ++iv) {
        const int64_t y = (int64_t)os1 * iv + ov + R1 / 2;
        if (y < 0 || y >= R1) continue;
        const double2 e = ey64[f * R1 + y];
        double rr = 0.0, ri = 0.0;   // sum over x of k * ex[x]
        for (int iu = -(su / 2); iu < su - su / 2; ++iu) {
            const int64_t x = (int64_t)os0 * iu + ou + R0 / 2;
            if (x < 0 || x >= R0) continue;
            const double k = ck[(cf * R0 + x) * R1 + y];
            const double2 q = ex64[f * R0 + x];
            rr += k * q.x;
            ri += k * q.y;
        }
        re += rr * e.x - ri * e.y;
        im += rr * e.y + ri * e.x;
    }
    nrm[id] = make_double2(re, im);
}



// ---- mosaic weight grid ----------------------------------------------------
// wsum[cimg][p][f][cfb][cfc] = sum of weights of the rows that pass the edge rule
__global__ void k_wsum(const GArgs a, int64_t nfb, double *wsum) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= a.T * a.B * a.C) return;
    const int64_t row = id / a.C, c = id % a.C;
    const int64_t b = row % a.B;
    const int fidx = a.field_index[row];
    if (fidx < 0 || fidx >= a.nf) return;
    const float4 us = a.uvs[row];
    if (isnan(us.x) || isnan(us.z)) return;
    const GChan cp = a.chan[c];
    const int cu_c = (int)(a.nu / 2), cv_c = (int)(a.nv / 2);
    int cu, cv, o;
    if (!cell_pair(us.x, us.y, cp.suh, cp.sul, false, cu_c, 0, cu, o)) {
        long long i64, o64;
        cell_fp64(a.uvw[row * 3 + 0], cp.su, false, cu_c, 0, i64, o64);
        cu = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
    }
    if (!cell_pair(us.z, us.w, cp.svh, cp.svl, false, cv_c, 0, cv, o)) {
        long long i64, o64;
        cell_fp64(a.uvw[row * 3 + 1], cp.sv, false, cv_c, 0, i64, o64);
        cv = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
    }
    if (!(cu + a.maxsup < a.nu && cv + a.maxsup < a.nv && cu - a.maxsup >= 0 && cv - a.maxsup >= 0)) return;
    const int64_t cimg = a.continuum ? 0 : c;
    const int cfb = a.cfb_map[b], cfc = a.cfc_map[c];
    if (cfb < 0 || cfb >= a.ncfb || cfc < 0 || cfc >= a.ncfc) return;
    for (int64_t p = 0; p < a.P; ++p) {
        const float w = a.weight[id * a.P + p];
        if (isnan(w) || w == 0.f) continue;
        atomicAdd(wsum + ((((cimg * a.P + p) * nfb + fidx) * a.ncfb + cfb) * a.ncfc + cfc),
                  (double)w);
    }
}

// weight-grid patch at the grid centre and its sum_weight
__global__ void k_wpatch(const GArgs a, const double *wk, const int32_t *support, int nf,
                         int64_t ncfb, const double *wsum, const double2 *nrm_w) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int S = a.S, sc = S / 2;
    const int64_t per = (int64_t)S * S;
    if (id >= (int64_t)a.n_img * a.P * per) return;
    const int64_t q = id / per;   // cimg * P + p
    const int p = (int)(q % a.P);
    const int iu = (int)((id % per) / S) - sc, iv = (int)(id % S) - sc;
    const int cfp = a.cfp_map[p];
    if (cfp < 0 || cfp >= a.ncfp) return;
    double re = 0.0, im = 0.0, sw = 0.0;
    for (int f = 0; f < nf; ++f)
        for (int64_t cfb = 0; cfb < ncfb; ++cfb)
            for (int64_t cfc = 0; cfc < a.ncfc; ++cfc) {
                const double w = wsum[(((q * nf + f) * ncfb + cfb) * a.ncfc + cfc)];
                if (w == 0.0) continue;
                const int64_t cf = (cfb * a.ncfc + cfc) * a.ncfp + cfp;
                if (iu == -sc && iv == -sc) sw += w * nrm_w[(int64_t)f * a.ncf + cf].x;
                if (!in_support(iu, support[cf * 2]) || !in_support(iv, support[cf * 2 + 1])) continue;
                const int64_t x = (int64_t)a.os0 * iu + a.R0 / 2, y = (int64_t)a.os1 * iv + a.R1 / 2;
                const double kk = wk[(cf * a.R0 + x) * a.R1 + y];
                const double2 ex = a.ex64[(int64_t)f * a.R0 + x], ey = a.ey64[(int64_t)f * a.R1 + y];
                const double c = ex.x * ey.x - ex.y * ey.y, s = ex.x * ey.y + ex.y * ey.x;
                re += w * kk * c;
                im += w * kk * s;
            }
    const int cu_c = (int)(a.nu / 2), cv_c = (int)(a.nv / 2);
    int u = cu_c + iu, v = cv_c + iv;
    if (u >= 0 && u < a.nu && v >= 0 && v < a.nv) {
        if (a.fftl) {
            u = u < cu_c ? u + ((int)a.nu - cu_c) : u - cu_c;
            v = v < cv_c ? v + ((int)a.nv - cv_c) : v - cv_c;
        }
        a.grid[(q * a.nu + u) * a.nv + v] = make_float2((float)re, (float)im);
    }
    if (iu == -sc && iv == -sc) a.sum_weight[q] = sw;
}

// ---- GCF generation ----------------------------------------------------------
__global__ void k_airy(int casa, const double *dish, const double *block, int64_t nt, const double *freq, int64_t nf,
                       int64_t n0, int64_t n1, double cell0, double cell1, int64_t c0, int64_t c1, double *pat) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nt * nf * n0 * n1) return;
    const int64_t j = id % n1, i = (id / n1) % n0, f = (id / (n0 * n1)) % nf, ty = id / (nf * n0 * n1);
    if (i == c0 && j == c1) {
        pat[id] = 1.0;
        return;
    }
    const double x = (double)(i - c0) * cell0, y = (double)(j - c1) * cell1;
    const double kw = (2.0 * M_PI * freq[f]) / kCLight;
    const double D = dish[ty], bl = block[ty];
    const double r = __dmul_rn(__dmul_rn(sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y))), kw), D / 2.0);
    double v;
    if (bl == 0.0) {
        v = 2.0 * j1(r) / r;
    } else if (casa) {
        const double A = (D / bl) * (D / bl), L = D / bl;
        v = (A * 2.0 * j1(r) / r - 2.0 * j1(r * L) / (r * L)) / (A - 1.0);
    } else {
        const double e = bl / D;
        v = (2.0 * j1(r) / r - 2.0 * e * j1(r * e) / r) / (1.0 - e * e);
    }
    pat[id] = v;
}

// primary beam of each dish type in the image layout (l, m, freq, type):
// the voltage pattern of k_airy raised to ipower, exactly 1 at the centre
__global__ void k_pb_layout(const double *pat, int64_t nt, int64_t nf, int64_t n0, int64_t n1, int ipower,
                            double *out) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nt * nf * n0 * n1) return;
    const int64_t ty = id % nt, f = (id / nt) % nf, j = (id / (nt * nf)) % n1, i = id / (nt * nf * n1);
    const double v = pat[((ty * nf + f) * n0 + i) * n1 + j];
    double r = v;
    for (int k = 1; k < ipower; ++k) r *= v;
    out[id] = r;
}

// pair product (ipower 1 or 2) into an ifftshift-ed complex buffer
__global__ void k_pair(const double *pat, const int32_t *pairs, int64_t np, int64_t nf, int64_t n0, int64_t n1,
                       int ipower, double2 *work) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np * nf * n0 * n1) return;
    const int64_t k2 = id % n1, k1 = (id / n1) % n0, f = (id / (n0 * n1)) % nf, q = id / (nf * n0 * n1);
    const int64_t i = (k1 + n0 / 2) % n0, j = (k2 + n1 / 2) % n1;   // ifftshift source
    const int64_t a0 = pairs[q * 2], a1 = pairs[q * 2 + 1];
    const double p0 = pat[((a0 * nf + f) * n0 + i) * n1 + j], p1 = pat[((a1 * nf + f) * n0 + i) * n1 + j];
    double v = ipower == 1 ? p0 * p1 : (p0 * p0) * (p1 * p1);
    work[id] = make_double2(v, 0.0);
}

__global__ void k_real_fftshift(const double2 *work, int64_t nq, int64_t n0, int64_t n1, double *out) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nq * n0 * n1) return;
    const int64_t j = id % n1, i = (id / n1) % n0, q = id / (n0 * n1);
    const int64_t si = (i - n0 / 2 + n0) % n0, sj = (j - n1 / 2 + n1) % n1;   // fftshift source
    out[id] = work[(q * n0 + si) * n1 + sj].x;
}

// ---- mosaic normalisation ------------------------------------------------------
// image (l, m, plane): image / (osc(l,m) * (ps_corr(l,m) * norm(l,m,plane))),
// osc = sinc(dl / (n_l os0)) sinc(dm / (n_m os1)); 0 where pb < pb_limit; float32 round trip.
// The sinc factors are separable: k_sinc tabulates them once per l and per m
// (FP64 sinpi and divisions are long sequences on GB300's FP64 pipe), so an
// element costs three products and one division, with the same values and
// operation order as the per-element formula.
__global__ void k_sinc(int64_t nl, int64_t nm, int os0, int os1, double *sl, double *sm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nl) {
        const double x = (double)(i - nl / 2) / (double)(nl * os0);
        sl[i] = x == 0.0 ? 1.0 : sinpi(x) / (M_PI * x);
    } else if (i < nl + nm) {
        const int64_t m = i - nl;
        const double x = (double)(m - nm / 2) / (double)(nm * os1);
        sm[m] = x == 0.0 ? 1.0 : sinpi(x) / (M_PI * x);
    }
}

__global__ void k_mnorm(double *image, int64_t nl, int64_t nm, int64_t np_, const double *ps, const double *nimg,
                        const double *pb, double pb_limit, const double *sinc_l, const double *sinc_m, int single) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nl * nm * np_) return;
    const int64_t lm = id / np_;
    const int64_t l = lm / nm, m = lm - (lm / nm) * nm;
    const double osc = sinc_l[l] * sinc_m[m];
    double d = ps ? ps[lm] : 1.0;
    if (nimg) d = d * nimg[id];
    double v = image[id] / (osc * d);
    if (pb && pb_limit > 0.0 && pb[id] < pb_limit) v = 0.0;
    if (single) v = (double)(float)v;
    image[id] = v;
}

// centre values -> their reciprocals (in place), then one product per element
__global__ void k_recip(double *v, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = 1.0 / v[i];
}

__global__ void k_centre_div(double *image, const double *inv, int64_t np_, int64_t n) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    image[id] = image[id] * inv[id % np_];
}

__global__ void k_sqrt_abs(const double *w, int64_t n, double *pb) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id < n) pb[id] = sqrt(fabs(w[id]));
}

// the same tap sums from the reorganised FP32 table ckt (learned path): FP32
// sums along a row, FP64 across rows (the table itself is a fit to ~1e-3)
__global__ void k_norms_tab(const float *ckt, const double2 *ex64, const double2 *ey64, int nf, int64_t ncf,
                            int64_t R0, int64_t R1, int os0, int os1, int S, double2 *nrm) {
    const int64_t no = (int64_t)(os0 + 1) * (os1 + 1);
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nf * ncf * no) return;
    const int64_t f = id / (ncf * no), cf = (id / no) % ncf, o = id % no;
    const int oui = (int)(o / (os1 + 1)), ovi = (int)(o % (os1 + 1));
    const int sc = S / 2;
    const float *blk = ckt + ((cf * (os0 + 1) + oui) * (os1 + 1) + ovi) * (2 * S) * SP;
    const double2 *exf = ex64 + f * R0 + (oui - os0 / 2 + R0 / 2 - (int64_t)os0 * sc);
    double re = 0.0, im = 0.0;
    for (int dv = 0; dv < S; ++dv) {
        const int64_t y = (int64_t)os1 * (dv - sc) + ovi - os1 / 2 + R1 / 2;
        const double2 e = ey64[f * R1 + y];
        float rr = 0.f, ri = 0.f;
        for (int du = 0; du < S; ++du) {
            const float k = blk[dv * SP + du];
            const double2 q = exf[(int64_t)os0 * du];
            rr = fmaf(k, (float)q.x, rr);
            ri = fmaf(k, (float)q.y, ri);
        }
        re += (double)rr * e.x - (double)ri * e.y;
        im += (double)rr * e.y + (double)ri * e.x;
    }
    nrm[id] = make_double2(re, im);
}

__global__ void k_iota(int32_t *p, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (int32_t)i;
}

int check_gcf(const NggGcfArgs *a, bool learned = false) {
    if (!a) return fail(NGG_ERR_INVALID, "args is NULL");
    if (a->chan_mode != NGG_CHAN_CUBE && a->chan_mode != NGG_CHAN_CONTINUUM) return fail(NGG_ERR_INVALID, "chan_mode");
    if (a->layout != NGG_LAYOUT_NATURAL && a->layout != NGG_LAYOUT_FFT) return fail(NGG_ERR_INVALID, "layout");
    if (a->n_time < 0 || a->n_baseline < 0 || a->n_chan < 0 || a->n_pol < 1 || a->n_u < 1 || a->n_v < 1 ||
        a->n_u > 65535 || a->n_v > 65535 || a->n_field < 1)
        return fail(NGG_ERR_INVALID, "dims");
    if (a->oversampling[0] < 1 || a->oversampling[1] < 1 || a->oversampling[0] > 1000 || a->oversampling[1] > 1000)
        return fail(NGG_ERR_UNSUPPORTED, "oversampling out of [1,1000]");
    if (a->n_cf_baseline < 1 || a->n_cf_chan < 1 || a->n_cf_pol < 1 || a->conv_size[0] < 1 || a->conv_size[1] < 1)
        return fail(NGG_ERR_INVALID, "GCF table dims");
    if (!a->grid || !a->sum_weight || !a->support || !a->phase_slope) return fail(NGG_ERR_INVALID, "NULL pointer");
    if (!learned && (!a->conv_kernel || !a->cf_baseline_map || !a->cf_chan_map || !a->cf_pol_map))
        return fail(NGG_ERR_INVALID, "NULL pointer");
    return NGG_OK;
}



// shared set-up of both gridders; returns the maximum support via *maxsup
struct Learned {
    const float *params;
    const NggMlpScale *scale;
};

// learned: the per-channel tables come from the network (conv_kernel and the
// CF maps are not read)
int gcf_setup(const NggGcfArgs *a, cudaStream_t s, ScratchList &sc, GArgs &g, int *S_out,
              const Learned *learned = nullptr) {
    const int64_t T = a->n_time, B = a->n_baseline, C = a->n_chan, P = a->n_pol;
    const int64_t ncf = a->n_cf_baseline * a->n_cf_chan * a->n_cf_pol;
    // supports (host copy: small)
    std::vector<int32_t> sup(ncf * 2);
    NGG_CUDA(cudaMemcpyAsync(sup.data(), a->support, sizeof(int32_t) * ncf * 2, cudaMemcpyDeviceToHost, s));
    NGG_CUDA(cudaStreamSynchronize(s));
    int maxsup = 0;
    for (auto x : sup) maxsup = x > maxsup ? x : maxsup;
    if (maxsup < 1 || maxsup > MAXS) return fail(NGG_ERR_UNSUPPORTED, "GCF support must be in [1, 31]");
    int S = maxsup | 1;   // odd number of column classes covering every CF
    if (S > MAXS) S = MAXS;
    *S_out = S;
    // every tap a lane can address, os*i + off + R/2 with |i| <= S/2 and
    // off in [-os/2, os - os/2], must lie in the table
    for (int d = 0; d < 2; ++d) {
        const int64_t os = a->oversampling[d], R = a->conv_size[d], h = S / 2;
        if (R / 2 - os * h - os / 2 < 0 || R / 2 + os * h + (os - os / 2) >= R)
            return fail(NGG_ERR_UNSUPPORTED, "GCF table smaller than (support + 1) * oversampling");
    }
    int rc;
    GChan *chan = nullptr;
    float4 *uvs = nullptr;
    float *ckt = nullptr;
    float2 *gx = nullptr, *gy = nullptr, *hx = nullptr, *hy = nullptr;
    double2 *ex64 = nullptr, *ey64 = nullptr;
    int32_t *maps = nullptr;
    double2 *nrm = nullptr;
    if ((rc = sc.get((void **)&chan, sizeof(GChan) * (C > 0 ? C : 1))) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&uvs, sizeof(float4) * (T * B > 0 ? T * B : 1))) != NGG_OK) return rc;
    const int64_t nck = ncf * (a->oversampling[0] + 1) * (a->oversampling[1] + 1) * 2 * S * SP;
    if ((rc = sc.get((void **)&ckt, sizeof(float) * nck)) != NGG_OK) return rc;
    const int64_t nf = a->n_field;
    if ((rc = sc.get((void **)&gx, sizeof(float2) * nf * a->n_u)) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&gy, sizeof(float2) * nf * a->n_v)) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&hx, sizeof(float2) * nf * (a->oversampling[0] + 1))) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&hy, sizeof(float2) * nf * (a->oversampling[1] + 1))) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&ex64, sizeof(double2) * a->n_field * a->conv_size[0])) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&ey64, sizeof(double2) * a->n_field * a->conv_size[1])) != NGG_OK) return rc;
    const int64_t nn = a->n_field * ncf * (a->oversampling[0] + 1) * (a->oversampling[1] + 1);
    if ((rc = sc.get((void **)&nrm, sizeof(double2) * nn)) != NGG_OK) return rc;
    if (C > 0) k_gchan<<<(unsigned)((C + 127) / 128), 128, 0, s>>>(a->freq, (int)C, a->delta_lm[0], a->delta_lm[1], a->n_u, a->n_v, chan);
    if (T * B > 0) k_gsplit<<<(unsigned)((T * B + 255) / 256), 256, 0, s>>>(a->uvw, T * B, uvs);
    if (learned) {
        if ((rc = sc.get((void **)&maps, sizeof(int32_t) * (B + C + P + 1))) != NGG_OK) return rc;
        NGG_CUDA(cudaMemsetAsync(maps, 0, sizeof(int32_t) * (B + C + P + 1), s));
        if (C > 0) k_iota<<<(unsigned)((C + 255) / 256), 256, 0, s>>>(maps + B, C);
        if ((rc = mlp_synth_table(learned->params, learned->scale, a->freq, C, a->oversampling[0], a->oversampling[1],
                                  S, a->support, ckt, s)) != NGG_OK)
            return rc;
    } else {
        k_reorg<<<(unsigned)((nck + 255) / 256), 256, 0, s>>>(a->conv_kernel, ncf, a->conv_size[0], a->conv_size[1],
                                                             a->oversampling[0], a->oversampling[1], a->support, S, ckt);
    }
    const int64_t ncp = nf * (a->n_u + a->n_v + a->oversampling[0] + 1 + a->oversampling[1] + 1);
    k_cell_phase<<<(unsigned)((ncp + 255) / 256), 256, 0, s>>>(a->phase_slope, a->n_field, a->n_u, a->n_v,
                                                              a->oversampling[0], a->oversampling[1], gx, gy, hx, hy);
    const int64_t npt = (int64_t)a->n_field * (a->conv_size[0] + a->conv_size[1]);
    k_phase_tabs<<<(unsigned)((npt + 255) / 256), 256, 0, s>>>(a->phase_slope, a->n_field, a->conv_size[0],
                                                              a->conv_size[1], ex64, ey64);
    if (learned)
        k_norms_tab<<<(unsigned)((nn + 127) / 128), 128, 0, s>>>(ckt, ex64, ey64, a->n_field, ncf, a->conv_size[0],
                                                                a->conv_size[1], a->oversampling[0],
                                                                a->oversampling[1], S, nrm);
    else
        k_norms<<<(unsigned)((nn + 127) / 128), 128, 0, s>>>(a->conv_kernel, a->support, ex64, ey64, a->n_field, ncf,
                                                            a->conv_size[0], a->conv_size[1], a->oversampling[0],
                                                            a->oversampling[1], 0, nrm);
    NGG_CHECK_LAUNCH("gcf set-up kernels");
    g.vis = (const float2 *)a->vis;
    g.weight = a->weight;
    g.uvw = a->uvw;
    g.uvs = uvs;
    g.chan = chan;
    g.field_index = a->field_index;
    g.cfb_map = learned ? maps : a->cf_baseline_map;
    g.cfc_map = learned ? maps + B : a->cf_chan_map;
    g.cfp_map = learned ? maps + B + C : a->cf_pol_map;
    g.ckt = ckt;
    g.gx = gx; g.gy = gy; g.hx = hx; g.hy = hy;
    g.ex64 = ex64;
    g.ey64 = ey64;
    g.nrm = nrm;
    g.grid = (float2 *)a->grid;
    g.sum_weight = a->sum_weight;
    g.T = T; g.B = B; g.C = C; g.P = P; g.nu = a->n_u; g.nv = a->n_v;
    g.ncfb = a->n_cf_baseline; g.ncfc = a->n_cf_chan; g.ncfp = a->n_cf_pol; g.ncf = ncf;
    g.nf = a->n_field;
    g.R0 = a->conv_size[0]; g.R1 = a->conv_size[1];
    g.os0 = a->oversampling[0]; g.os1 = a->oversampling[1];
    g.S = S;
    g.maxsup = maxsup;
    g.nk = (int)((T + GCH - 1) / GCH);
    g.n_img = a->chan_mode == NGG_CHAN_CONTINUUM ? 1 : (int)C;
    g.continuum = a->chan_mode == NGG_CHAN_CONTINUUM;
    g.fftl = a->layout == NGG_LAYOUT_FFT;
    return NGG_OK;
}

}  // namespace
}  // namespace ngg

using namespace ngg;

extern "C" int ngg_grid_gcf(const NggGcfArgs *a, void *stream) {
    clear_error();
    int rc = check_gcf(a);
    if (rc != NGG_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n_img = a->chan_mode == NGG_CHAN_CONTINUUM ? 1 : a->n_chan;
    if (n_img == 0) return NGG_OK;
    NGG_CUDA(cudaMemsetAsync(a->grid, 0, sizeof(float2) * n_img * a->n_pol * a->n_u * a->n_v, s));
    NGG_CUDA(cudaMemsetAsync(a->sum_weight, 0, sizeof(double) * n_img * a->n_pol, s));
    if (a->n_time * a->n_baseline * a->n_chan == 0) return NGG_OK;
    if (!a->uvw || !a->weight || !a->freq || !a->field_index || (a->mode == NGG_MODE_DATA && !a->vis))
        return fail(NGG_ERR_INVALID, "NULL input");
    ScratchList sc(s);
    GArgs g;
    int S = 0;
    if ((rc = gcf_setup(a, s, sc, g, &S)) != NGG_OK) return rc;
    const int64_t items = a->n_chan * a->n_baseline * g.nk * a->n_pol;
    const unsigned blocks = (unsigned)((items + 3) / 4);
    const bool data = a->mode == NGG_MODE_DATA;
    if (S <= 15) return launch_grid_gcf_lo(g, data, blocks, s);
    return S <= 23 ? launch_grid_gcf_mid(g, data, blocks, s) : launch_grid_gcf_hi(g, data, blocks, s);
}

extern "C" int ngg_grid_gcf_learned(const NggGcfArgs *a, const float *params, const NggMlpScale *scale, void *stream) {
    clear_error();
    int rc = check_gcf(a, true);
    if (rc != NGG_OK) return rc;
    if (!params || !scale) return fail(NGG_ERR_INVALID, "params / scale is NULL");
    if (a->n_cf_baseline != 1 || a->n_cf_pol != 1 || a->n_cf_chan != a->n_chan)
        return fail(NGG_ERR_INVALID, "learned GCF: one table per channel (n_cf_chan = n_chan, n_cf_baseline = n_cf_pol = 1)");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n_img = a->chan_mode == NGG_CHAN_CONTINUUM ? 1 : a->n_chan;
    if (n_img == 0) return NGG_OK;
    NGG_CUDA(cudaMemsetAsync(a->grid, 0, sizeof(float2) * n_img * a->n_pol * a->n_u * a->n_v, s));
    NGG_CUDA(cudaMemsetAsync(a->sum_weight, 0, sizeof(double) * n_img * a->n_pol, s));
    if (a->n_time * a->n_baseline * a->n_chan == 0) return NGG_OK;
    if (!a->uvw || !a->weight || !a->freq || !a->field_index || (a->mode == NGG_MODE_DATA && !a->vis))
        return fail(NGG_ERR_INVALID, "NULL input");
    ScratchList sc(s);
    GArgs g;
    int S = 0;
    Learned L{params, scale};
    if ((rc = gcf_setup(a, s, sc, g, &S, &L)) != NGG_OK) return rc;
    const int64_t items = a->n_chan * a->n_baseline * g.nk * a->n_pol;
    const unsigned blocks = (unsigned)((items + 3) / 4);
    const bool data = a->mode == NGG_MODE_DATA;
    if (S <= 15) return launch_grid_gcf_lo(g, data, blocks, s);
    return S <= 23 ? launch_grid_gcf_mid(g, data, blocks, s) : launch_grid_gcf_hi(g, data, blocks, s);
}

extern "C" int ngg_grid_gcf_weight(const NggGcfArgs *a, void *stream) {
    clear_error();
    int rc = check_gcf(a);
    if (rc != NGG_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n_img = a->chan_mode == NGG_CHAN_CONTINUUM ? 1 : a->n_chan;
    if (n_img == 0) return NGG_OK;
    NGG_CUDA(cudaMemsetAsync(a->grid, 0, sizeof(float2) * n_img * a->n_pol * a->n_u * a->n_v, s));
    NGG_CUDA(cudaMemsetAsync(a->sum_weight, 0, sizeof(double) * n_img * a->n_pol, s));
    if (a->n_time * a->n_baseline * a->n_chan == 0) return NGG_OK;
    if (!a->uvw || !a->weight || !a->freq || !a->field_index) return fail(NGG_ERR_INVALID, "NULL input");
    ScratchList sc(s);
    GArgs g;
    int S = 0;
    if ((rc = gcf_setup(a, s, sc, g, &S)) != NGG_OK) return rc;
    const int64_t ncfb = a->n_cf_baseline;
    const int64_t nws = n_img * a->n_pol * a->n_field * ncfb * a->n_cf_chan;
    double *wsum = nullptr;
    double2 *nrm_w = nullptr;
    if ((rc = sc.get((void **)&wsum, sizeof(double) * nws)) != NGG_OK) return rc;
    const int64_t nnw = (int64_t)a->n_field * g.ncf;
    if ((rc = sc.get((void **)&nrm_w, sizeof(double2) * nnw)) != NGG_OK) return rc;
    NGG_CUDA(cudaMemsetAsync(wsum, 0, sizeof(double) * nws, s));
    k_norms<<<(unsigned)((nnw + 127) / 128), 128, 0, s>>>(a->conv_kernel, a->support, g.ex64, g.ey64, a->n_field, g.ncf,
                                                         a->conv_size[0], a->conv_size[1], a->oversampling[0],
                                                         a->oversampling[1], 1, nrm_w);
    const int64_t n = a->n_time * a->n_baseline * a->n_chan;
    k_wsum<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, a->n_field, wsum);
    const int64_t np = n_img * a->n_pol * (int64_t)S * S;
    k_wpatch<<<(unsigned)((np + 127) / 128), 128, 0, s>>>(g, a->conv_kernel, a->support, a->n_field,
                                                         ncfb, wsum, nrm_w);
    NGG_CHECK_LAUNCH("ngg_grid_gcf_weight kernels");
    return NGG_OK;
}

extern "C" int ngg_primary_beam(int casa_model, int64_t nt, const double *dish, const double *block, int64_t nf,
                                const double *freq, int64_t n0, int64_t n1, const double cell[2], int64_t c0,
                                int64_t c1, int ipower, double *out, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (nt < 1 || nf < 0 || n0 < 1 || n1 < 1 || ipower < 1 || ipower > 8 || !cell || !dish || !block || !out ||
        (nf > 0 && !freq))
        return fail(NGG_ERR_INVALID, "ngg_primary_beam arguments");
    if (nf == 0) return NGG_OK;
    ScratchList sc(s);
    double *pat = nullptr;
    int rc;
    if ((rc = sc.get((void **)&pat, sizeof(double) * nt * nf * n0 * n1)) != NGG_OK) return rc;
    const int64_t n = nt * nf * n0 * n1;
    // out-of-grid centres leave no pixel at exactly 1 (k_airy only fixes an in-grid centre)
    k_airy<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(casa_model, dish, block, nt, freq, nf, n0, n1, cell[0], cell[1],
                                                        c0, c1, pat);
    NGG_CHECK_LAUNCH("k_airy");
    k_pb_layout<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(pat, nt, nf, n0, n1, ipower, out);
    NGG_CHECK_LAUNCH("k_pb_layout");
    return NGG_OK;
}

extern "C" int ngg_gcf_kernels(int casa_model, int64_t nt, const double *dish, const double *block, int64_t np,
                               const int32_t *pairs, int64_t nf, const double *freq, int64_t n0, int64_t n1,
                               const double cell[2], int64_t c0, int64_t c1, double *ck, double *wk, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (nt < 1 || np < 1 || nf < 1 || n0 < 2 || n1 < 2 || !cell || !dish || !block || !pairs || !freq || !ck || !wk)
        return fail(NGG_ERR_INVALID, "ngg_gcf_kernels arguments");
    {
        std::vector<int32_t> hp(np * 2);
        NGG_CUDA(cudaMemcpyAsync(hp.data(), pairs, sizeof(int32_t) * np * 2, cudaMemcpyDeviceToHost, s));
        NGG_CUDA(cudaStreamSynchronize(s));
        for (auto x : hp)
            if (x < 0 || x >= nt) return fail(NGG_ERR_INVALID, "antenna-type pair index out of range");
    }
    ScratchList sc(s);
    double *pat = nullptr;
    double2 *work = nullptr;
    int rc;
    if ((rc = sc.get((void **)&pat, sizeof(double) * nt * nf * n0 * n1)) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&work, sizeof(double2) * np * nf * n0 * n1)) != NGG_OK) return rc;
    const int64_t npat = nt * nf * n0 * n1;
    k_airy<<<(unsigned)((npat + 255) / 256), 256, 0, s>>>(casa_model, dish, block, nt, freq, nf, n0, n1, cell[0], cell[1],
                                                          c0, c1, pat);
    NGG_CHECK_LAUNCH("k_airy");
    cufftHandle h;
    long long n[2] = {(long long)n0, (long long)n1};
    size_t ws = 0;
    if (cufftCreate(&h) != CUFFT_SUCCESS) return fail(NGG_ERR_CUDA, "cufftCreate");
    if (cufftMakePlanMany64(h, 2, n, nullptr, 1, n0 * n1, nullptr, 1, n0 * n1, CUFFT_Z2Z, np * nf, &ws) != CUFFT_SUCCESS ||
        cufftSetStream(h, s) != CUFFT_SUCCESS) {
        cufftDestroy(h);
        return fail(NGG_ERR_CUDA, "cuFFT Z2Z plan");
    }
    const int64_t nw = np * nf * n0 * n1;
    for (int ip = 1; ip <= 2; ++ip) {
        k_pair<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(pat, pairs, np, nf, n0, n1, ip, work);
        if (cufftExecZ2Z(h, (cufftDoubleComplex *)work, (cufftDoubleComplex *)work, CUFFT_FORWARD) != CUFFT_SUCCESS) {
            cufftDestroy(h);
            return fail(NGG_ERR_CUDA, "cufftExecZ2Z");
        }
        k_real_fftshift<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(work, np * nf, n0, n1, ip == 1 ? ck : wk);
    }
    NGG_CHECK_LAUNCH("gcf kernels");
    // the plan's work area is released when the plan is destroyed; wait for the FFTs first
    cudaError_t e = cudaStreamSynchronize(s);
    cufftDestroy(h);
    if (e != cudaSuccess) return cuda_fail(e, "ngg_gcf_kernels");
    return NGG_OK;
}

extern "C" int ngg_mosaic_normalize(double *image, int64_t n_l, int64_t n_m, int64_t n_planes, const double *ps_corr,
                                    const double *norm_image, const double *pb, double pb_limit,
                                    const int oversampling[2], int single_precision, const int64_t *centre,
                                    void *stream) {
    clear_error();
    if (!image || !oversampling || n_l < 1 || n_m < 1 || n_planes < 0 || oversampling[0] < 1 || oversampling[1] < 1)
        return fail(NGG_ERR_INVALID, "ngg_mosaic_normalize arguments");
    if (centre && (centre[0] < 0 || centre[0] >= n_l || centre[1] < 0 || centre[1] >= n_m))
        return fail(NGG_ERR_INVALID, "centre outside the image");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n = n_l * n_m * n_planes;
    if (n == 0) return NGG_OK;
    ScratchList sc(s);
    double *sinc = nullptr;
    int rc;
    if ((rc = sc.get((void **)&sinc, sizeof(double) * (size_t)(n_l + n_m))) != NGG_OK) return rc;
    k_sinc<<<(unsigned)((n_l + n_m + 255) / 256), 256, 0, s>>>(n_l, n_m, oversampling[0], oversampling[1], sinc,
                                                                sinc + n_l);
    NGG_CHECK_LAUNCH("k_sinc");
    k_mnorm<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(image, n_l, n_m, n_planes, ps_corr, norm_image, pb, pb_limit,
                                                        sinc, sinc + n_l, single_precision);
    NGG_CHECK_LAUNCH("k_mnorm");
    if (centre) {
        // the centre pixels of every plane are copied out first (they are divided too)
        double *cval = nullptr;
        if ((rc = sc.get((void **)&cval, sizeof(double) * n_planes)) != NGG_OK) return rc;
        NGG_CUDA(cudaMemcpyAsync(cval, image + (centre[0] * n_m + centre[1]) * n_planes, sizeof(double) * n_planes,
                                 cudaMemcpyDeviceToDevice, s));
        k_recip<<<(unsigned)((n_planes + 255) / 256), 256, 0, s>>>(cval, n_planes);
        NGG_CHECK_LAUNCH("k_recip");
        k_centre_div<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(image, cval, n_planes, n);
        NGG_CHECK_LAUNCH("k_centre_div");
    }
    return NGG_OK;
}

extern "C" int ngg_sqrt_abs(const double *x, int64_t n, double *out, void *stream) {
    clear_error();
    if (n < 0 || (n > 0 && (!x || !out))) return fail(NGG_ERR_INVALID, "ngg_sqrt_abs arguments");
    if (n == 0) return NGG_OK;
    k_sqrt_abs<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, n, out);
    NGG_CHECK_LAUNCH("k_sqrt_abs");
    return NGG_OK;
}
