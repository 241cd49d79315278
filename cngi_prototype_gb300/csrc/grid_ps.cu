// Standard (prolate-spheroidal) convolutional gridder for sm_103a.
//
// Reference behaviour: _standard_grid_jit
// (ngcasa/imaging/_imaging_utils/_standard_grid.py:242-371) -- every
// visibility whose 7x7 footprint lies inside the grid adds
// conv_u*conv_v*weighted_datum to 49 cells and weight*sum(conv) to
// sum_weight.
//
// GB300 design (one call = the whole cube):
//  1. k_chan / k_uvw: per-channel uv scale (FP64, reference operation order)
//     split into FP32 pairs; per (baseline, time) uvw split into FP32 pairs in
//     baseline-major order; per 32-step track chunk a uv bounding box.
//  2. Binning: every chunk (chan, baseline, 32 time steps) is listed in each
//     64x64 uv-tile its footprint bounding box touches; keys
//     (bin = (image chan, tile), chunk) are radix-sorted so every bin holds
//     its chunks in (chan, baseline, time) order -- consecutive entries
//     continue the same track.
//  3. k_pack: one coalesced pass over the visibilities computes every step's
//     cell, oversampling offsets, weighted data and sum_weight term and
//     writes them track-major ([chan][baseline][time], 24 bytes a step), so
//     the tile pass reads each 32-step chunk as one contiguous run (reading
//     the (time, baseline, chan, pol) input directly from the tile pass
//     fetched ~9x the algorithmic bytes in scattered sectors).
//  4. k_tiles: a persistent kernel; each CTA takes work items (tile, image
//     channel) from a global counter, channel-fastest so CTAs working on
//     neighbouring channels share the visibility lines in L2. Empty tiles
//     are written as zeros; busy tiles are accumulated in shared memory and
//     written once, coalesced. The grid is therefore written exactly once
//     and never read back.
//  Inside a busy tile each warp takes a contiguous range of the tile's
//  chunks, one 32-step track chunk at a time: its lanes first turn the 32
//  packed steps into per-step tap products (tap_u x weighted data, tap_v),
//  then walk the steps with the 49 footprint cells owned in Romein's residue
//  classes (a lane holds one u class and two v classes in registers),
//  flushing a cell to shared memory (atomic add) only when the track moves
//  off it or, at the latest, at the end of the chunk. Taps come from the
//  oversampled table, loaded into shared memory by a TMA bulk copy. Cell and
//  oversampling indices are certified to equal the reference's FP64 results
//  (see cell_pair).
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "ngg_internal.cuh"

namespace ngg {
namespace {

constexpr int TU = 64;      // tile rows (u)
constexpr int TV = 64;      // tile columns (v, contiguous)
constexpr int CH = 32;      // time steps per chunk
constexpr int SUP = 7;
constexpr int SC = 3;
constexpr int MAX_TAB = 4096;
constexpr int MAX_OS = 1000;   // oversampling limit checked on the host
constexpr unsigned NO_CELL = 0xffffffffu;   // packed record of a step that adds nothing

struct ChanParms {
    double su, sv;
    float suh, sul, svh, svl;
};

struct TileArgs {
    const float2 *vis;        // (T,B,C,P)
    const float *weight;      // (T,B,C,P)
    const double *uvw;        // (T,B,3) (FP64 fallback only)
    const float4 *uvs;        // [B][T] (u_hi,u_lo,v_hi,v_lo)
    const ChanParms *chan;    // [C]
    const float *tab_g;       // table (float), padded to 16 bytes
    const uint2 *meta;        // packed steps [c][b][t]: (cell u<<16|v, offsets (ou+32768) | (ov+32768)<<16)
    const float4 *wvp;        // packed steps [c][b][t]: weighted data (re, im) per pol, or weights
    const unsigned long long *keys;
    const int64_t *bin_start; // [n_bins + 1]
    void *grid;
    double *sum_weight;
    int *work_counter;        // [0] tile queue, [1] zero queue
    int *err;                 // set to 1 when the table copy's bounded wait runs out
    const int *bbox;          // busy tile range (tu0, tu1, tv0, tv1) over all image channels
    const struct SubItem *subs;  // tile work items
    const int *n_subs;        // number of tile work items (device)
    int64_t T, B, C, P;
    int64_t nu, nv;
    int n_img, ntu, ntv, nk;
    int p0;            // first pol of this launch
    int os;
    int tab_len;       // floats in the table
    int tab_bytes;     // padded to 16
    int continuum;
    unsigned bnk;      // n_baseline * n_chunks_per_track (32-bit chunk decode)
};

__global__ void k_chan(const double *freq, int C, double dl0, double dl1, int64_t nu, int64_t nv,
                       ChanParms *out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    double su, sv;
    uv_scale_dev(freq[c], dl0, dl1, nu, nv, su, sv);
    ChanParms p;
    p.su = su;
    p.sv = sv;
    Split a = split_double(su), b = split_double(sv);
    p.suh = a.hi; p.sul = a.lo; p.svh = b.hi; p.svl = b.lo;
    out[c] = p;
}

// nsum[o + os/2] = sum_i tab[|os*i + o|], the 1-D tap sum at oversampling offset o
__global__ void k_nsum(const float *tab, int tab_len, int os, float *nsum) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > os) return;
    const int o = i - os / 2;
    float acc = 0.f;
    for (int d = -SC; d <= SC; ++d) {
        const int ix = abs(os * d + o);
        acc += ix < tab_len ? tab[ix] : 0.f;
    }
    nsum[i] = acc;
}

struct PackArgs {
    const float2 *vis;        // (T,B,C,P)
    const float *weight;      // (T,B,C,P)
    const double *uvw;        // (T,B,3) (FP64 fallback only)
    const float4 *uvs;        // [B][T]
    const ChanParms *chan;    // [C]
    const float *nsum;        // [os + 1]
    uint2 *meta;              // [C][B][nk*CH]
    float4 *wvp;              // [C][B][nk*CH]
    double *sw_part;          // [C][NP][B][nk] sum_weight partials
    int64_t T, B, C, P;
    int64_t c_stride, c_off;  // vis/weight are (T,B,c_stride,P); this call's channels start at c_off
    int64_t nu, nv;
    int nk, p0, os;
    // Imaging weights formed in this pass (ngg_grid_ps_weighted): the
    // weights above are then the natural weights, divided by f0*W + f1 at
    // the step's cell of the weight-density planes (NULL: used as given).
    const float *density;        // (n_img, dnu, dnv)
    const double *factors;       // (2, n_img)
    const ChanParms *dchan;      // [C] uv scale of the density grid
    const unsigned char *flag;   // (T,B,c_stride,P), nonzero = flagged visibility (DATA mode), or NULL
    int64_t dnu, dnv, n_img;
    int continuum;
    // cell_half's constants: K = (2 C + 1) os per axis, ceil(2^40 / os), the
    // margin; half_ok = 0 where K >= 2^24 (then cell_pair serves every step)
    int ku, kv;
    unsigned long long osm;
    float margin0;
    int half_ok;
    // both pols of a step load as one 16-byte visibility and one 8-byte
    // weight access (2 pols from pol 0, aligned buffers)
    int vec2;
};

// cell_pair, then the FP64 chain: the packing pass's rare path (a step near a
// rounding boundary), kept out of line so that its registers do not weigh on
// the common path. axis 0 = u, 1 = v; xyz points at the step's uvw row.
static __device__ __noinline__ void cell_slow(float xh, float xl, const ChanParms *cpp, int axis, const double *xyz,
                                              int center, int os, int &idx, int &off) {
    const ChanParms cp = *cpp;
    const float sh = axis ? cp.svh : cp.suh, sl = axis ? cp.svl : cp.sul;
    if (cell_pair(xh, xl, sh, sl, false, center, os, idx, off)) return;
    long long i64, o64;
    cell_fp64(xyz[axis], axis ? cp.sv : cp.su, false, center, os, i64, o64);
    idx = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
    off = (int)o64;
}

// The reference's nearest-cell weight lookup (_standard_imaging_weight_degrid_jit,
// _standard_grid.py:466-518), for one (time, baseline, channel): the step's
// cell in the unpadded density grid, W there, and the imaging weight of each
// pol from the natural weights (two pols are averaged first). false: the
// cell lies outside the density grid (the reference gives weight 0).
template <int NP>
__device__ __forceinline__ bool step_imaging_weights(const PackArgs &a, float4 us, int64_t t, int64_t b, int64_t c,
                                                     int64_t base, float (&w)[NP]) {
    const ChanParms dp = a.dchan[c];
    int du, dv, o;
    if (!cell_pair(us.x, us.y, dp.suh, dp.sul, false, (int)(a.dnu / 2), 0, du, o)) {
        long long i64, o64;
        cell_fp64(a.uvw[(t * a.B + b) * 3 + 0], dp.su, false, (int)(a.dnu / 2), 0, i64, o64);
        du = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
    }
    if (!cell_pair(us.z, us.w, dp.svh, dp.svl, false, (int)(a.dnv / 2), 0, dv, o)) {
        long long i64, o64;
        cell_fp64(a.uvw[(t * a.B + b) * 3 + 1], dp.sv, false, (int)(a.dnv / 2), 0, i64, o64);
        dv = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
    }
    if (du < 0 || du >= a.dnu || dv < 0 || dv >= a.dnv) return false;
    const int64_t cimg = a.continuum ? 0 : c;   // image channel of this call
    const float W = a.density[(cimg * a.dnu + du) * a.dnv + dv];
    const float f0 = (float)a.factors[cimg], f1 = (float)a.factors[a.n_img + cimg];
    const bool Wok = !isnan(W) && W != 0.f;
    const int64_t b0 = base - a.p0;   // pol 0 of this (time, baseline, channel)
    const float avg = a.P == 2 ? (a.weight[b0] + a.weight[b0 + 1]) * 0.5f : 0.f;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const float wp = a.weight[base + p];
        float iw = a.P == 2 ? avg : wp;
        if (!isnan(wp) && wp != 0.f && Wok) iw = iw / (f0 * W + f1);
        w[p] = iw;
    }
    return true;
}

// One pass over the visibilities (time, baseline, chan, pol): per step its
// cell and oversampling offsets (the FP64 index chain, certified FP32 pairs),
// its weighted data and its sum_weight term, written track-major
// ([chan][baseline][time]) so that the tile kernel reads each 32-step chunk
// as one contiguous run however many tiles the chunk touches. A block is 32
// channels x 32 steps of one (baseline, chunk): the reads are contiguous over
// channels, a shared-memory transpose makes the writes contiguous over time.
template <int NP, bool CPLX, bool FUSED>
__global__ void __launch_bounds__(256, 4) k_pack(const PackArgs a) {
    __shared__ uint2 s_meta[32][33];
    __shared__ float4 s_wv[32][33];
    __shared__ float s_sw[NP][32][9];       // per channel: the 8 row-threads' partial sums
    __shared__ float s_nsum[MAX_OS + 1];
    __shared__ float4 s_uvs[CH];             // the chunk's uvw pairs (every channel lane shares them)
    const int x = threadIdx.x;
    const int64_t b = blockIdx.x;
    const int k = blockIdx.y;
    const int64_t c0 = (int64_t)blockIdx.z * 32;
    const int cu_c = (int)(a.nu / 2), cv_c = (int)(a.nv / 2);
    for (int i = threadIdx.y * 32 + x; i <= a.os; i += 256) s_nsum[i] = a.nsum[i];
    float swc[NP];   // this thread's sum_weight terms over its 4 steps
#pragma unroll
    for (int p = 0; p < NP; ++p) swc[p] = 0.f;
    // All loads of the thread's 4 steps are issued before any index
    // arithmetic, so the pass waits for memory once rather than twice per
    // step (uvw and channel scale, then visibilities and weights).
    const int64_t c = c0 + x;
    const bool c_ok = c < a.C;
    ChanParms cp{};
    if (c_ok) cp = a.chan[c];
    // cell_half's scales for this channel (2 os s as pairs)
    float s2uh, s2ul, s2vh, s2vl;
    scale_pair(cp.suh, cp.sul, (float)(2 * a.os), s2uh, s2ul);
    scale_pair(cp.svh, cp.svl, (float)(2 * a.os), s2vh, s2vl);
    float wl[4][NP];
    float2 vl[4][NP];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t t = (int64_t)k * CH + threadIdx.y + 8 * i;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            wl[i][p] = 0.f;
            vl[i][p] = make_float2(0.f, 0.f);
        }
        if (c_ok && t < a.T) {
            const int64_t base = ((t * a.B + b) * a.c_stride + a.c_off + c) * a.P + a.p0;
            if (NP == 2 && a.vec2) {   // both pols of a (time, baseline, channel) in one 16- and one 8-byte load
                if (!FUSED) {
                    const float2 w2 = *reinterpret_cast<const float2 *>(a.weight + base);
                    wl[i][0] = w2.x;
                    wl[i][NP - 1] = w2.y;
                }
                if constexpr (CPLX) {
                    const float4 v4 = *reinterpret_cast<const float4 *>(a.vis + base);
                    vl[i][0] = make_float2(v4.x, v4.y);
                    vl[i][NP - 1] = make_float2(v4.z, v4.w);
                }
            } else {
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    if (!FUSED) wl[i][p] = a.weight[base + p];
                    if constexpr (CPLX) vl[i][p] = a.vis[base + p];
                }
            }
        }
    }
    // the uvw pairs through shared memory (issued after the visibility and
    // weight loads, so that all of them are in flight together)
    if (threadIdx.y == 0) {
        const int64_t t = (int64_t)k * CH + x;
        s_uvs[x] = t < a.T ? a.uvs[b * a.T + t] : make_float4(NAN, 0.f, NAN, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int y = threadIdx.y + 8 * i;
        const int64_t t = (int64_t)k * CH + y;
        uint2 meta = make_uint2(NO_CELL, 0u);
        float4 wv = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 us = s_uvs[y];
        if (c_ok && t < a.T && !isnan(us.x) && !isnan(us.z)) {
            int cu, ou, cv, ov;
            if (!(a.half_ok && cell_half(us.x, us.y, s2uh, s2ul, a.ku, a.os, a.osm, a.margin0, cu, ou)))
                cell_slow(us.x, us.y, a.chan + c, 0, a.uvw + (t * a.B + b) * 3, cu_c, a.os, cu, ou);
            if (!(a.half_ok && cell_half(us.z, us.w, s2vh, s2vl, a.kv, a.os, a.osm, a.margin0, cv, ov)))
                cell_slow(us.z, us.w, a.chan + c, 1, a.uvw + (t * a.B + b) * 3, cv_c, a.os, cv, ov);
            if (cu - SC >= 0 && cu + SC < a.nu && cv - SC >= 0 && cv + SC < a.nv) {
                const int64_t base = ((t * a.B + b) * a.c_stride + a.c_off + c) * a.P + a.p0;
                float w[NP];
                bool pv[NP];
                bool any = false;
                bool in_density = true;
                if constexpr (FUSED) {
                    if (a.density) in_density = step_imaging_weights<NP>(a, us, t, b, c, base, w);
                    else {
#pragma unroll
                        for (int p = 0; p < NP; ++p) w[p] = a.weight[base + p];
                    }
                } else {
#pragma unroll
                    for (int p = 0; p < NP; ++p) w[p] = wl[i][p];
                }
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    if (!in_density) w[p] = 0.f;
                    if constexpr (CPLX) {
                        const float2 vv = vl[i][p];
                        const float xr = vv.x * w[p], xi = vv.y * w[p];
                        pv[p] = !isnan(xr) && !isnan(xi) && (xr != 0.f || xi != 0.f);
                        if (FUSED && a.flag && a.flag[base + p]) pv[p] = false;   // flagged: the visibility is NaN
                        if (p == 0) { wv.x = pv[p] ? xr : 0.f; wv.y = pv[p] ? xi : 0.f; }
                        else { wv.z = pv[p] ? xr : 0.f; wv.w = pv[p] ? xi : 0.f; }
                    } else {
                        pv[p] = !isnan(w[p]) && w[p] != 0.f;
                        if (p == 0) wv.x = pv[p] ? w[p] : 0.f;
                        else wv.y = pv[p] ? w[p] : 0.f;
                    }
                    any = any || pv[p];
                }
                if (any) {
                    meta = make_uint2(((unsigned)cu << 16) | (unsigned)cv,
                                      (unsigned)(ou + 32768) | ((unsigned)(ov + 32768) << 16));
                    const float norm = s_nsum[ou + a.os / 2] * s_nsum[ov + a.os / 2];
#pragma unroll
                    for (int p = 0; p < NP; ++p)
                        if (pv[p]) swc[p] = __fadd_rn(swc[p], __fmul_rn(w[p], norm));
                }
            }
        }
        s_meta[x][y] = meta;
        s_wv[x][y] = wv;
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) s_sw[p][x][threadIdx.y] = swc[p];
    __syncthreads();
    // warp w writes channels c0 + w + 8i, lane x its step x
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int64_t c = c0 + y;
        if (c >= a.C) break;
        const int64_t ri = ((c * a.B + b) * a.nk + k) * CH + x;
        a.meta[ri] = s_meta[y][x];
        a.wvp[ri] = s_wv[y][x];
    }
    // the chunk's sum_weight partial per (channel, pol): its 8 row-threads' sums in a fixed order
    const int e = threadIdx.y * 32 + x;
    if (e < 32 * NP) {
        const int cl = e % 32, p = e / 32;
        const int64_t c = c0 + cl;
        if (c < a.C) {
            float v = 0.f;
#pragma unroll
            for (int r = 0; r < 8; ++r) v = __fadd_rn(v, s_sw[p][cl][r]);
            a.sw_part[((c * NP + p) * a.B + b) * a.nk + k] = (double)v;
        }
    }
}

// sum_weight[image chan, p0 + p] = sum of its partials (fixed order: deterministic)
__global__ void __launch_bounds__(256) k_sw_reduce(const double *sw_part, int64_t C, int np, int64_t per_chan,
                                                   int continuum, int64_t P, int p0, double *sum_weight) {
    __shared__ double red[256];
    const int64_t img = blockIdx.x / np;
    const int p = (int)(blockIdx.x % np);
    const int64_t c_lo = continuum ? 0 : img, c_hi = continuum ? C : img + 1;
    double acc = 0.0;
    for (int64_t c = c_lo; c < c_hi; ++c) {
        const double *q = sw_part + (c * np + p) * per_chan;
        for (int64_t i = threadIdx.x; i < per_chan; i += blockDim.x) acc += q[i];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) sum_weight[img * P + p0 + p] = red[0];
}

// one warp per (baseline, chunk): split uvw rows and reduce the chunk bbox
__global__ void k_uvw(const double *uvw, int64_t T, int64_t B, int nk, float4 *uvs, float4 *bbox) {
    int64_t w = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (w >= B * nk) return;
    int64_t b = w / nk;
    int k = (int)(w % nk);
    int64_t t = (int64_t)k * CH + lane;
    float umin = INFINITY, umax = -INFINITY, vmin = INFINITY, vmax = -INFINITY;
    if (t < T) {
        double u = uvw[(t * B + b) * 3 + 0];
        double v = uvw[(t * B + b) * 3 + 1];
        Split su = split_double(u), sv = split_double(v);
        uvs[b * T + t] = make_float4(su.hi, su.lo, sv.hi, sv.lo);
        if (!isnan(u) && !isnan(v)) {
            umin = umax = su.hi;
            vmin = vmax = sv.hi;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        umin = fminf(umin, __shfl_xor_sync(0xffffffffu, umin, o));
        umax = fmaxf(umax, __shfl_xor_sync(0xffffffffu, umax, o));
        vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
        vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    }
    if (lane == 0) bbox[w] = make_float4(umin, umax, vmin, vmax);
}

struct TileRange { int u0, u1, v0, v1; };  // inclusive tile index range, u0>u1 = empty

__device__ __forceinline__ TileRange chunk_tiles(float4 bb, const ChanParms &cp, int64_t nu, int64_t nv,
                                                 int ntu, int ntv) {
    TileRange r{1, 0, 1, 0};
    if (!(bb.x <= bb.y) || !(bb.z <= bb.w)) return r;
    float a = bb.x * cp.suh, b = bb.y * cp.suh;
    float lo_u = fminf(a, b) + (float)(nu / 2), hi_u = fmaxf(a, b) + (float)(nu / 2);
    a = bb.z * cp.svh;
    b = bb.w * cp.svh;
    float lo_v = fminf(a, b) + (float)(nv / 2), hi_v = fmaxf(a, b) + (float)(nv / 2);
    // nearest cell +- (half support + 2 cells of margin for float rounding)
    float cl_u = floorf(lo_u + 0.5f) - (SC + 2), ch_u = floorf(hi_u + 0.5f) + (SC + 2);
    float cl_v = floorf(lo_v + 0.5f) - (SC + 2), ch_v = floorf(hi_v + 0.5f) + (SC + 2);
    if (!(ch_u >= 0.f) || !(cl_u <= (float)(nu - 1)) || !(ch_v >= 0.f) || !(cl_v <= (float)(nv - 1))) return r;
    int iu0 = (int)fmaxf(cl_u, 0.f), iu1 = (int)fminf(ch_u, (float)(nu - 1));
    int iv0 = (int)fmaxf(cl_v, 0.f), iv1 = (int)fminf(ch_v, (float)(nv - 1));
    r.u0 = iu0 / TU; r.u1 = iu1 / TU; r.v0 = iv0 / TV; r.v1 = iv1 / TV;
    (void)ntu; (void)ntv;
    return r;
}

__global__ void k_count(const float4 *bbox, const ChanParms *chan, int64_t C, int64_t B, int nk,
                        int64_t nu, int64_t nv, int ntu, int ntv, unsigned *counts) {
    int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t n = C * B * nk;
    if (ch >= n) return;
    int64_t c = ch / (B * nk);
    int64_t bk = ch % (B * nk);
    TileRange r = chunk_tiles(bbox[bk], chan[c], nu, nv, ntu, ntv);
    unsigned cnt = 0;
    if (r.u0 <= r.u1 && r.v0 <= r.v1) cnt = (unsigned)((r.u1 - r.u0 + 1) * (r.v1 - r.v0 + 1));
    counts[ch] = cnt;
    if (ch == n - 1) counts[n] = 0;  // sentinel: the exclusive scan's last entry is the total
}

__global__ void k_emit(const float4 *bbox, const ChanParms *chan, int64_t C, int64_t B, int nk, int64_t nu,
                       int64_t nv, int ntu, int ntv, int continuum, const unsigned long long *offsets,
                       unsigned long long *keys) {
    int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t n = C * B * nk;
    if (ch >= n) return;
    int64_t c = ch / (B * nk);
    int64_t bk = ch % (B * nk);
    TileRange r = chunk_tiles(bbox[bk], chan[c], nu, nv, ntu, ntv);
    if (!(r.u0 <= r.u1 && r.v0 <= r.v1)) return;
    unsigned long long o = offsets[ch];
    // the key is (tile, chunk): the chunk index is channel-major, so keys in
    // tile order are in (tile, image channel) bin order as well
    for (int tu = r.u0; tu <= r.u1; ++tu)
        for (int tv = r.v0; tv <= r.v1; ++tv) {
            const unsigned long long tile = (unsigned long long)((int64_t)tu * ntv + tv);
            keys[o++] = (tile << 32) | (unsigned long long)ch;
        }
}

__global__ void k_bbox_init(int *bb) {
    bb[0] = 0x7fffffff; bb[1] = -1; bb[2] = 0x7fffffff; bb[3] = -1;
}

// range of tiles holding any chunk, over all image channels
__global__ void k_bbox(const int64_t *bin_start, int64_t n_bins, int n_img, int ntv, int *bb) {
    const int64_t bin = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (bin >= n_bins || bin_start[bin] == bin_start[bin + 1]) return;
    const int64_t tile = bin / n_img;
    const int tu = (int)(tile / ntv), tv = (int)(tile % ntv);
    atomicMin(&bb[0], tu); atomicMax(&bb[1], tu);
    atomicMin(&bb[2], tv); atomicMax(&bb[3], tv);
}

// bin = tile * n_img + image channel; its first key is (tile, the image
// channel's first chunk) (chunks_per_img = B * nk in cube mode, 0 in
// continuum mode, where every channel is image channel 0)
__global__ void k_bounds(const unsigned long long *keys, int64_t n, int64_t n_bins, int n_img,
                         int64_t chunks_per_img, int64_t *bin_start) {
    int64_t bin = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (bin > n_bins) return;
    const unsigned long long target = ((unsigned long long)(bin / n_img) << 32) |
                                      (unsigned long long)((bin % n_img) * chunks_per_img);
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (keys[mid] < target) lo = mid + 1; else hi = mid;
    }
    bin_start[bin] = lo;
}

// ---- the tile kernel -------------------------------------------------------

constexpr int MAXE = 2048;   // chunk entries per tile work item; heavier bins are split

struct SubItem {
    int box_item;   // index of (tile in busy box, image channel)
    int sub;        // part of the bin's entries
    int nsub;       // parts of this bin (> 1: flush with atomics into a zeroed tile)
    int pad;
};

__device__ __forceinline__ bool mbar_wait(unsigned addr, unsigned phase) {
    for (int it = 0; it < (1 << 22); ++it) {
        unsigned ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(addr), "r"(phase)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// box item -> (tile index, image channel, bin)
struct BoxMap {
    int bt0, bv0, nbu, nbv, n_img;
    int ntv;
    __device__ __forceinline__ void map(int64_t item, int &tiu, int &tiv, int &cimg, int64_t &bin) const {
        const int64_t tix = item / n_img;
        cimg = (int)(item % n_img);
        tiu = bt0 + (int)(tix / nbv);
        tiv = bv0 + (int)(tix % nbv);
        bin = ((int64_t)tiu * ntv + tiv) * n_img + cimg;   // tile-major bins
    }
};

__device__ __forceinline__ BoxMap box_map(const int *bbox, int n_img, int ntv) {
    BoxMap m;
    const bool have = bbox[0] <= bbox[1] && bbox[2] <= bbox[3];
    m.bt0 = bbox[0];
    m.bv0 = bbox[2];
    m.nbu = have ? bbox[1] - bbox[0] + 1 : 0;
    m.nbv = have ? bbox[3] - bbox[2] + 1 : 0;
    m.n_img = n_img;
    m.ntv = ntv;
    return m;
}

// number of work items of every box item (0 beyond the box)
__global__ void k_nsub(const int64_t *bin_start, const int *bbox, int n_img, int ntv, int64_t n_bound, int *nsub) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n_bound) return;
    const BoxMap m = box_map(bbox, n_img, ntv);
    const int64_t n_box = (int64_t)m.nbu * m.nbv * n_img;
    int k = 0;
    if (i < n_box) {
        int tiu, tiv, cimg;
        int64_t bin;
        m.map(i, tiu, tiv, cimg, bin);
        const int64_t n = bin_start[bin + 1] - bin_start[bin];
        k = n > MAXE ? (int)((n + MAXE - 1) / MAXE) : 1;
    }
    nsub[i] = k;
}

__global__ void k_fill_subs(const int *nsub, const int *off, int64_t n_bound, SubItem *subs, int *n_total) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_bound) return;
    const int k = nsub[i], o = off[i];
    for (int s = 0; s < k; ++s) subs[o + s] = SubItem{(int)i, s, k, 0};
    if (i == n_bound - 1) *n_total = o + k;
}

// zero the destination of bins split over several work items (they add
// their partial tiles with atomics); grid-stride over the busy box's items
// (a few of the ~10^6 bins are split: one block per bin was all launch cost)
template <bool CPLX, bool FFTL>
__global__ void k_zero_split(const int64_t *bin_start, const int *bbox, int n_img, int ntv,
                             int64_t n_bound, void *grid, int64_t P, int p0, int np, int64_t nu, int64_t nv) {
    const BoxMap m = box_map(bbox, n_img, ntv);
    const int64_t n_box = (int64_t)m.nbu * m.nbv * n_img;
    for (int64_t i = blockIdx.x; i < n_bound && i < n_box; i += gridDim.x) {
    int tiu, tiv, cimg;
    int64_t bin;
    m.map(i, tiu, tiv, cimg, bin);
    if (bin_start[bin + 1] - bin_start[bin] <= MAXE) continue;
    const int u0 = tiu * TU, v0 = tiv * TV;
    const int cu_c = (int)(nu / 2), cv_c = (int)(nv / 2);
    for (int e = threadIdx.x; e < np * TU * TV; e += blockDim.x) {
        const int p = e / (TU * TV), r = (e / TV) % TU, cl = e % TV;
        int u = u0 + r, v = v0 + cl;
        if (u >= nu || v >= nv) continue;
        if (FFTL) {
            u = u < cu_c ? u + (int)(nu - cu_c) : u - cu_c;
            v = v < cv_c ? v + (int)(nv - cv_c) : v - cv_c;
        }
        const int64_t off = (((int64_t)cimg * P + p0 + p) * nu + u) * nv + v;
        if (CPLX || FFTL) reinterpret_cast<float2 *>(grid)[off] = make_float2(0.f, 0.f);
        else reinterpret_cast<float *>(grid)[off] = 0.f;
    }
    }
}

constexpr int ZBUF = 2048;   // bytes of zeros in shared memory: the source of the zero-fill bulk stores

// Zero nbytes of the grid at gp (gp and nbytes multiples of elem): plain
// stores up to the first 16-byte boundary and after the last one, TMA bulk
// stores (asynchronous; committed by the caller) from the zero buffer at
// shared address zs for the aligned middle.
__device__ __forceinline__ void zero_fill(char *gp, int64_t nbytes, unsigned zs, int elem) {
    while (nbytes > 0 && ((uintptr_t)gp & 15)) {
        if (elem == 8) *reinterpret_cast<float2 *>(gp) = make_float2(0.f, 0.f);
        else *reinterpret_cast<float *>(gp) = 0.f;
        gp += elem;
        nbytes -= elem;
    }
    const int64_t mid = nbytes & ~(int64_t)15;
    for (char *q = gp + mid; q < gp + nbytes; q += elem) {
        if (elem == 8) *reinterpret_cast<float2 *>(q) = make_float2(0.f, 0.f);
        else *reinterpret_cast<float *>(q) = 0.f;
    }
    for (int64_t o = 0; o < mid; o += ZBUF) {
        const unsigned sz = (unsigned)(mid - o < ZBUF ? mid - o : ZBUF);
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gp + o), "r"(zs), "r"(sz)
                     : "memory");
    }
}

struct ZeroRows {
    void *grid;
    int64_t nu, nv, P;
    int p0, nrb;
    int64_t n_items;
    int R0, R1, V0, V1, cu_c, cv_c;   // busy box rows/columns (natural order), grid centre
    unsigned zs;                       // shared address of the zero buffer
    int *counter;
};

// Take the next block of ZR rows outside the busy box and zero it (the part
// of each row outside the box, in stored order); false when none is left.
template <int NP, int ELEM, bool FFTL>
__device__ __noinline__ bool zero_next(const ZeroRows &z) {
    constexpr int ZR = 8;
    const long long it = atomicAdd(z.counter, 1);
    if (it >= z.n_items) return false;
    const int64_t q = it / z.nrb;
    const int rb = (int)(it % z.nrb);
    const int cimg = (int)(q / NP), p = (int)(q % NP);
    const int64_t pbase = ((int64_t)cimg * z.P + z.p0 + p) * z.nu * z.nv;
    const int r_end = min(rb * ZR + ZR, (int)z.nu);
    for (int r = rb * ZR; r < r_end; ++r) {
        const int un = FFTL ? (r + z.cu_c >= z.nu ? r + z.cu_c - (int)z.nu : r + z.cu_c) : r;   // natural row
        char *row = reinterpret_cast<char *>(z.grid) + (pbase + (int64_t)r * z.nv) * ELEM;
        if (!(un >= z.R0 && un < z.R1 && z.V1 > z.V0)) {
            zero_fill(row, z.nv * ELEM, z.zs, ELEM);
            continue;
        }
        // stored columns of the natural busy range [V0, V1)
        int s0 = z.V0;
        const int L = z.V1 - z.V0;
        if (FFTL) { s0 = z.V0 - z.cv_c; if (s0 < 0) s0 += (int)z.nv; }
        if (s0 + L <= z.nv) {
            zero_fill(row, (int64_t)s0 * ELEM, z.zs, ELEM);
            zero_fill(row + (int64_t)(s0 + L) * ELEM, (z.nv - s0 - L) * ELEM, z.zs, ELEM);
        } else {
            const int e = s0 + L - (int)z.nv;
            zero_fill(row + (int64_t)e * ELEM, (int64_t)(s0 - e) * ELEM, z.zs, ELEM);
        }
    }
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group.read 4;" ::: "memory");   // bound this thread's stores in flight
    return true;
}

// ---- the tile kernel: one track per warp ------------------------------------
//
// A CTA owns one uv-tile (TU x TV cells, every pol of the launch) of one image
// channel at a time, accumulated in shared memory and written to the grid
// once. Its warps take contiguous ranges of the tile's chunk list; a warp
// handles one 32-step chunk at a time in two phases:
//  * producer: lane s takes step s of the chunk (its packed record, loaded
//    from global memory one chunk ahead) and writes to the warp's shared
//    record, in residue-class order, the 7 products tap_u * weighted data
//    (both pols) and the 7 v taps, plus the step's cell: class c holds the
//    tap whose cell has class c, tap k = (c - (cu - 3)) mod 7;
//  * consumer: the 49 footprint cells are owned in Romein's residue classes:
//    lane 4 kappa + g, kappa the u class (u mod 7) and g in 0..3, holds the
//    cells of u class kappa and v classes 2g and 2g+1 in registers (lanes
//    28-31 hold none). Thanks to the class order a lane
//    reads the same record slots at every step -- one 16-byte load of its u
//    product, one 8-byte load of its two v taps -- and adds them with four
//    paired FMAs.
//    The producer marks the steps where the track's cell changes (a ballot);
//    the consumer runs through the steps between two marks with nothing but
//    the two loads and the FMAs, and at a mark (a warp-uniform branch)
//    flushes to the shared tile (atomic adds) only the cells that leave the
//    footprint and restarts them; every second chunk all cells are flushed,
//    so that no FP32 register sum runs longer than 64 steps (long sums of
//    like-sized terms drift). The cells are absolute grid cells, so a chunk of another track
//    simply continues accumulating into whichever cells it shares.
// The taps come from the oversampled table staged in shared memory by a TMA
// bulk copy. The tile is stored as (re, im) planes per pol whose column
// index is XOR-swizzled by the row, so the flush atomics of the 7 u classes
// of one v cell fall into different banks.
constexpr int NWT = 24;                  // warps per CTA (one CTA per SM)
constexpr int RT = 12;                   // floats per step of v taps (8 used; a 48-byte row keeps the
                                         // 16-byte stores of a quarter-warp in different banks)
constexpr int WARP_REC_BYTES = CH * SUP * 16 + CH * RT * 4 + CH * 4;

// the tile kernel's compute warps (all but the zero-fill warp)
__device__ __forceinline__ void compute_sync() { asm volatile("bar.sync 1, %0;" ::"n"(NWT * 32) : "memory"); }

__device__ __forceinline__ int tile_addr(int lu, int lv) { return lu * TV + (lv ^ ((lu & 7) << 2)); }

__device__ __forceinline__ void red_shared(float *p, float v) {
    asm volatile("red.shared.add.f32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "f"(v) : "memory");
}

// the cell of class cls (0..7) in [lo, lo + 7), lo in [0, 65535]
__device__ __forceinline__ int residue_cell(int lo, int cls) {
    return lo + (int)((unsigned)(cls - lo + 7 * 9363) % 7u);
}

template <int NP, bool CPLX, bool FFTL>
__global__ void __launch_bounds__((NWT + 1) * 32, 1) k_tiles(const TileArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int NPL = CPLX ? 2 * NP : NP;   // float planes of the tile
    constexpr int NA = CPLX ? NP : 1;         // float2 accumulators per cell
    float *acc_s = reinterpret_cast<float *>(smem);
    float *tab = acc_s + NPL * TU * TV;
    unsigned char *recs = reinterpret_cast<unsigned char *>(tab + ((a.tab_bytes + 3) / 4));
    unsigned long long *mbar = reinterpret_cast<unsigned long long *>(recs + (size_t)NWT * WARP_REC_BYTES);
    int *s_item = reinterpret_cast<int *>(mbar + 1);   // [kind, item]
    float4 *zbuf = reinterpret_cast<float4 *>(
        (reinterpret_cast<uintptr_t>(s_item + 2) + 15) & ~static_cast<uintptr_t>(15));

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;

    // ---- stage the tap table with a TMA bulk copy -------------------------
    const unsigned mbar_addr = (unsigned)__cvta_generic_to_shared(mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_addr) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        const unsigned dst = (unsigned)__cvta_generic_to_shared(tab);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar_addr), "r"(a.tab_bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
            "l"(a.tab_g), "r"(a.tab_bytes), "r"(mbar_addr)
            : "memory");
    }
    if (!__syncthreads_and(mbar_wait(mbar_addr, 0))) {
        // The bounded wait ran out: report it and return once the copy has
        // landed (or a second bounded wait has also run out).
        if (tid == 0) {
            atomicExch(a.err, 1);
            mbar_wait(mbar_addr, 0);
        }
        __syncthreads();
        return;
    }
    for (int i = tid; i < NPL * TU * TV; i += blockDim.x) acc_s[i] = 0.f;
    for (int i = tid; i < ZBUF / 16; i += blockDim.x) zbuf[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // the bulk stores read zbuf
    __syncthreads();
    const unsigned zs = (unsigned)__cvta_generic_to_shared(zbuf);

    float4 *recA = reinterpret_cast<float4 *>(recs + (size_t)warp * WARP_REC_BYTES);   // [CH][SUP] by u class
    float *recT = reinterpret_cast<float *>(recA + CH * SUP);                           // [CH][RT] by v class
    unsigned *recC = reinterpret_cast<unsigned *>(recT + CH * RT);                      // [CH]

    const int cu_c = (int)(a.nu / 2), cv_c = (int)(a.nv / 2);
    const int64_t plane = a.nu * a.nv;
    const BoxMap bm = box_map(a.bbox, a.n_img, a.ntv);
    const int R0 = bm.nbu ? bm.bt0 * TU : 0, R1 = bm.nbu ? min((bm.bt0 + bm.nbu) * TU, (int)a.nu) : 0;
    const int V0 = bm.nbv ? bm.bv0 * TV : 0, V1 = bm.nbv ? min((bm.bv0 + bm.nbv) * TV, (int)a.nv) : 0;
    const int64_t n_tile_items = *a.n_subs;
    constexpr int ZR = 8;
    const int nrb = (int)((a.nu + ZR - 1) / ZR);
    const int64_t n_zero_items = (int64_t)a.n_img * NP * nrb;
    const int os = a.os;

    // this lane's residue classes (consumer): lane = 4 kappa + g. A half-warp
    // then reads at most 4 distinct u products (4 of the 7 16-byte slots of a
    // step), which a 16-byte shared load serves in one wavefront per half-warp
    // instead of two
    const bool act = lane < 28;
    const int kap = act ? lane >> 2 : 6, g = lane & 3;   // lanes 28-31 read valid slots (and never flush)
    const int rho0 = 2 * g, rho1 = 2 * g + 1;
    const bool has1 = act && g < 3;
    const int gr = g;

    // Warp NWT zeroes the rows outside the busy box: each of its lanes takes
    // blocks of rows from a counter and zeroes them with TMA bulk stores from
    // the shared zero buffer, independently of the tile work (the compute
    // warps synchronise on a named barrier of their own), so the grid's
    // zeros stream out while the other warps grid.
    const ZeroRows zr{a.grid, a.nu, a.nv, a.P, a.p0, nrb, n_zero_items, R0, R1, V0, V1, cu_c, cv_c, zs,
                      &a.work_counter[1]};
    if (warp == NWT) {
        while (zero_next<NP, (CPLX || FFTL) ? 8 : 4, FFTL>(zr)) {
        }
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");   // this lane's zero rows are written
        return;
    }
    constexpr int NCT = NWT * 32;   // compute threads
    for (;;) {
        if (tid == 0) {
            const long long it = atomicAdd(&a.work_counter[0], 1);
            s_item[0] = it < n_tile_items ? 0 : -1;
            s_item[1] = (int)it;
        }
        compute_sync();
        const int kind = s_item[0];
        const int64_t item = s_item[1];
        if (kind < 0) break;
        const SubItem si = a.subs[item];
        int tiu, tiv, cimg;
        int64_t bin;
        bm.map(si.box_item, tiu, tiv, cimg, bin);
        const int u0 = tiu * TU, v0 = tiv * TV;
        const int64_t b0 = a.bin_start[bin], b1 = a.bin_start[bin + 1];
        const int64_t e0 = b0 + ((b1 - b0) * si.sub) / si.nsub;
        const int64_t e1 = b0 + ((b1 - b0) * (si.sub + 1)) / si.nsub;
        const bool split = si.nsub > 1;

        if (e0 < e1) {
            // ---------------- busy tile: this warp's chunk range ----------------
            const int64_t n = e1 - e0;
            const int64_t rs = e0 + (n * warp) / NWT, re = e0 + (n * (warp + 1)) / NWT;
            // consumer state: the lane's cells and their accumulators
            int ucell = -(1 << 28), vcell0 = -(1 << 28), vcell1 = -(1 << 28);
            int lu = 0, lv0 = 0, lv1 = 0;
            bool ok0 = false, ok1 = false;
            float2 acc[2][NA];
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
                for (int q = 0; q < NA; ++q) acc[r][q] = make_float2(0.f, 0.f);

            auto flush = [&](int r) {
                const bool ok = r ? ok1 : ok0;
                if (!ok) return;
                const int ad = tile_addr(lu, r ? lv1 : lv0);
#pragma unroll
                for (int q = 0; q < NA; ++q) {
                    const float2 x = acc[r][q];
                    if constexpr (CPLX) {
                        if (x.x != 0.f) red_shared(acc_s + (2 * q) * TU * TV + ad, x.x);
                        if (x.y != 0.f) red_shared(acc_s + (2 * q + 1) * TU * TV + ad, x.y);
                    } else {
                        if (x.x != 0.f) red_shared(acc_s + ad, x.x);
                        if (NP > 1 && x.y != 0.f) red_shared(acc_s + TU * TV + ad, x.y);
                    }
                }
            };
            auto zero = [&](int r) {
#pragma unroll
                for (int q = 0; q < NA; ++q) acc[r][q] = make_float2(0.f, 0.f);
            };
            auto change = [&](unsigned cuv) {
                const int lo_u = (int)(cuv >> 16) - SC, lo_v = (int)(cuv & 0xffffu) - SC;
                const int nu_ = residue_cell(lo_u, kap);
                const int nv0 = residue_cell(lo_v, rho0), nv1 = residue_cell(lo_v, rho1);
                const bool cc = nu_ != ucell;
                if (cc || nv0 != vcell0) { flush(0); zero(0); }
                if (cc || nv1 != vcell1) { flush(1); zero(1); }
                ucell = nu_; vcell0 = nv0; vcell1 = nv1;
                lu = ucell - u0; lv0 = vcell0 - v0; lv1 = vcell1 - v0;
                const bool in_u = act && (unsigned)lu < (unsigned)TU;
                ok0 = in_u && (unsigned)lv0 < (unsigned)TV;
                ok1 = in_u && has1 && (unsigned)lv1 < (unsigned)TV;
            };

            // the chunk j's packed step of this lane (producer), loaded one
            // chunk ahead; the chunk keys two chunks ahead, so that a data
            // load never waits for the key load it depends on
            uint2 m_nx = make_uint2(NO_CELL, 0u);
            float4 d_nx = make_float4(0.f, 0.f, 0.f, 0.f);
            unsigned key_nx = 0;
            auto fetch = [&](unsigned chu) {
                const int64_t ri = (int64_t)chu * CH + lane;
                m_nx = __ldg(a.meta + ri);
                d_nx = __ldg(a.wvp + ri);
            };
            if (rs < re) fetch((unsigned)(__ldg(a.keys + rs) & 0xffffffffull));
            if (rs + 1 < re) key_nx = (unsigned)(__ldg(a.keys + rs + 1) & 0xffffffffull);
            const float4 *cA = recA + kap;                                      // this lane's slots
            const float2 *cT = reinterpret_cast<const float2 *>(recT) + gr;
            int jl = 0;
            unsigned carry = NO_CELL;   // the warp's current cell: the last cell of its previous chunks
            for (int64_t j = rs; j < re; ++j) {
                const uint2 m = m_nx;
                const float4 d = d_nx;
                if (j + 1 < re) {
                    fetch(key_nx);
                    if (j + 2 < re) key_nx = (unsigned)(__ldg(a.keys + j + 2) & 0xffffffffull);
                }
                // ---- producer: lane = step, records in residue-class order ----
                unsigned chg;   // bit s: step s may change the track's cell (uniform over the warp)
                {
                    float4 *ra = recA + lane * SUP;
                    float4 *rt = reinterpret_cast<float4 *>(recT + lane * RT);
                    if (m.x != NO_CELL) {
                        const int cu = (int)(m.x >> 16), cv = (int)(m.x & 0xffffu);
                        const int ou = (int)(m.y & 0xffffu) - 32768, ov = (int)(m.y >> 16) - 32768;
                        // the class of tap 0's cell
                        const int ku = (int)((unsigned)(cu - SC) % 7u), kv = (int)((unsigned)(cv - SC) % 7u);
                        float tv[SUP + 1];
#pragma unroll
                        for (int c = 0; c < SUP; ++c) {
                            // class c holds tap k = (c - k0) mod 7, whose table index is
                            // |os (k - 3) + o| (o lies in [-os/2, os/2]); the classes are
                            // written in order, so a quarter-warp's 16-byte stores fall into
                            // different banks
                            const int kku = c - ku + (c < ku ? SUP : 0);
                            const int kkv = c - kv + (c < kv ? SUP : 0);
                            const float tu = tab[abs(os * (kku - SC) + ou)];
                            tv[c] = tab[abs(os * (kkv - SC) + ov)];
                            const float2 t2 = make_float2(tu, tu);
                            const float2 lo = __fmul2_rn(t2, make_float2(d.x, d.y));
                            const float2 hi = __fmul2_rn(t2, make_float2(d.z, d.w));
                            ra[c] = make_float4(lo.x, lo.y, hi.x, hi.y);
                        }
                        tv[SUP] = 0.f;   // v class 7 does not exist (second row of g = 3)
                        rt[0] = make_float4(tv[0], tv[1], tv[2], tv[3]);
                        rt[1] = make_float4(tv[4], tv[5], tv[6], tv[7]);
                    } else {
#pragma unroll
                        for (int c = 0; c < SUP; ++c) ra[c] = make_float4(0.f, 0.f, 0.f, 0.f);
                        rt[0] = make_float4(0.f, 0.f, 0.f, 0.f);
                        rt[1] = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                    recC[lane] = m.x;
                    // a step whose cell differs from the cell of the latest step before it
                    // that has one (steps without a cell add zeros to whatever cells are
                    // current, so they do not end a run; the cells are absolute, so the
                    // previous chunk's last cell carries over even from another track)
                    unsigned last = m.x;   // the cell of this step or of the latest step before it that has one
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const unsigned t = __shfl_up_sync(0xffffffffu, last, o);
                        if (lane >= o && last == NO_CELL) last = t;
                    }
                    unsigned prev = __shfl_up_sync(0xffffffffu, last, 1);
                    if (lane == 0 || prev == NO_CELL) prev = carry;
                    chg = __ballot_sync(0xffffffffu, m.x != NO_CELL && m.x != prev);
                    const unsigned tail = __shfl_sync(0xffffffffu, last, 31);
                    if (tail != NO_CELL) carry = tail;
                }
                __syncwarp();
                // ---- consumer: the chunk's 32 steps, in runs between cell changes ----
                const float4 *pA = cA;
                const float2 *pT = cT;
                int st = 0;
                for (;;) {
                    const int nxt = chg ? __ffs(chg) - 1 : CH;
#pragma unroll 4
                    for (; st < nxt; ++st, pA += SUP, pT += RT / 2) {
                        const float4 A = *pA;
                        const float2 t = *pT;   // this lane's two v taps
                        const float2 T0 = make_float2(t.x, t.x), T1 = make_float2(t.y, t.y);
                        acc[0][0] = __ffma2_rn(make_float2(A.x, A.y), T0, acc[0][0]);
                        acc[1][0] = __ffma2_rn(make_float2(A.x, A.y), T1, acc[1][0]);
                        if constexpr (CPLX && NP > 1) {
                            acc[0][1] = __ffma2_rn(make_float2(A.z, A.w), T0, acc[0][1]);
                            acc[1][1] = __ffma2_rn(make_float2(A.z, A.w), T1, acc[1][1]);
                        }
                    }
                    if (nxt >= CH) break;
                    change(recC[nxt]);
                    chg &= chg - 1u;
                }
                // bound the register sums to two chunks (64 steps)
                if (++jl == 2) {
                    jl = 0;
                    flush(0); zero(0); flush(1); zero(1);
                }
                __syncwarp();   // the producer of the next chunk overwrites the records
            }
            flush(0);
            flush(1);
            compute_sync();   // every warp's cells are in the tile
        }

        // ---------------- write the tile ----------------
        const bool busy = e0 < e1;
        if (!(split && !busy)) {
            for (int e = tid; e < NP * TU * TV; e += NCT) {
                const int p = e / (TU * TV);
                const int r = (e / TV) % TU;
                const int cl = e % TV;
                const int u = u0 + r, v = v0 + cl;
                float2 val = make_float2(0.f, 0.f);
                if (busy) {
                    const int ad = tile_addr(r, cl);
                    if constexpr (CPLX) {
                        float *qr = acc_s + (2 * p) * TU * TV + ad, *qi = qr + TU * TV;
                        val = make_float2(*qr, *qi);
                        *qr = 0.f;
                        *qi = 0.f;
                    } else {
                        float *q = acc_s + p * TU * TV + ad;
                        val.x = *q;
                        *q = 0.f;
                    }
                }
                if (u < a.nu && v < a.nv) {
                    int du = u, dv = v;
                    if (FFTL) {  // (x - N/2) mod N for x in [0, N)
                        du = u < cu_c ? u + ((int)a.nu - cu_c) : u - cu_c;
                        dv = v < cv_c ? v + ((int)a.nv - cv_c) : v - cv_c;
                    }
                    const int64_t off = ((int64_t)cimg * a.P + a.p0 + p) * plane + (int64_t)du * a.nv + dv;
                    if (split) {
                        if (CPLX || FFTL) {
                            float *q = reinterpret_cast<float *>(reinterpret_cast<float2 *>(a.grid) + off);
                            if (val.x != 0.f) atomicAdd(q, val.x);
                            if (val.y != 0.f) atomicAdd(q + 1, val.y);
                        } else if (val.x != 0.f) {
                            atomicAdd(reinterpret_cast<float *>(a.grid) + off, val.x);
                        }
                    } else if (CPLX || FFTL) {
                        reinterpret_cast<float2 *>(a.grid)[off] = val;
                    } else {
                        reinterpret_cast<float *>(a.grid)[off] = val.x;
                    }
                }
            }
        }
        compute_sync();
    }
}

size_t tile_smem_bytes(int np, bool cplx, int tab_bytes) {
    const size_t acc = (size_t)(cplx ? 2 * np : np) * TU * TV * 4;
    const size_t tab = (size_t)((tab_bytes + 3) / 4) * 4;
    const size_t rec = (size_t)NWT * WARP_REC_BYTES;
    return acc + tab + rec + 8 + 8 + 16 + ZBUF;
}

template <int NP, bool CPLX, bool FFTL>
int launch_tiles(const TileArgs &ta, int64_t n_bound, cudaStream_t s) {
    const size_t smem = tile_smem_bytes(NP, CPLX, ta.tab_bytes);
    auto kern = k_tiles<NP, CPLX, FFTL>;
    NGG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    NGG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (NWT + 1) * 32, smem));
    if (per_sm < 1) return fail(NGG_ERR_UNSUPPORTED, "k_tiles does not fit on an SM");
    if (n_bound > 0) {
        const int64_t zb = n_bound < (int64_t)num_sms() * 16 ? n_bound : (int64_t)num_sms() * 16;
        k_zero_split<CPLX, FFTL><<<(unsigned)zb, 256, 0, s>>>(ta.bin_start, ta.bbox, ta.n_img, ta.ntv, n_bound,
                                                                    ta.grid, ta.P, ta.p0, NP, ta.nu, ta.nv);
        NGG_CHECK_LAUNCH("k_zero_split");
    }
    const int grid = num_sms() * per_sm;
    kern<<<grid, (NWT + 1) * 32, smem, s>>>(ta);
    NGG_CHECK_LAUNCH("k_tiles");
    return NGG_OK;
}

template <int NP>
int dispatch_tiles(const TileArgs &ta, int64_t n_bound, bool cplx, bool fftl, cudaStream_t s) {
    if (cplx) return fftl ? launch_tiles<NP, true, true>(ta, n_bound, s) : launch_tiles<NP, true, false>(ta, n_bound, s);
    return fftl ? launch_tiles<NP, false, true>(ta, n_bound, s) : launch_tiles<NP, false, false>(ta, n_bound, s);
}

__global__ void k_cell_indices(int64_t n_rows, int64_t C, const double *uvw, const double *freq, int64_t nu, int64_t nv,
                               double dl0, double dl1, int os, int mirror, unsigned long long osm, float margin0,
                               int32_t *idx, unsigned long long *nfb) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_rows * C) return;
    const int64_t r = id / C, c = id % C;
    double su, sv;
    uv_scale_dev(freq[c], dl0, dl1, nu, nv, su, sv);
    const Split a = split_double(su), b = split_double(sv);
    const double u = uvw[r * 3], v = uvw[r * 3 + 1];
    const Split x = split_double(u), y = split_double(v);
    int cu = 0, cv = 0, ou = 0, ov = 0;
    unsigned long long fb = 0;
    // the packing pass's chain: cell_half, then cell_pair, then FP64
    const int cu_c = (int)(nu / 2), cv_c = (int)(nv / 2);
    const float os2 = (float)(2 * os) * (mirror ? -1.f : 1.f);
    float s2uh, s2ul, s2vh, s2vl;
    scale_pair(a.hi, a.lo, os2, s2uh, s2ul);
    scale_pair(b.hi, b.lo, os2, s2vh, s2vl);
    const bool half_ok = os >= 1 && os < 65536 && (int64_t)(2 * cu_c + 1) * os < (1 << 24) &&
                         (int64_t)(2 * cv_c + 1) * os < (1 << 24);
    const int Ku = (2 * cu_c + 1) * os, Kv = (2 * cv_c + 1) * os;
    if (!(half_ok && cell_half(x.hi, x.lo, s2uh, s2ul, Ku, os, osm, margin0, cu, ou)) &&
        !cell_pair(x.hi, x.lo, a.hi, a.lo, mirror != 0, cu_c, os, cu, ou)) {
        long long i64, o64;
        cell_fp64(u, su, mirror != 0, (int)(nu / 2), os, i64, o64);
        cu = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
        ou = (int)max(min(o64, (long long)1 << 30), -((long long)1 << 30));
        ++fb;
    }
    if (!(half_ok && cell_half(y.hi, y.lo, s2vh, s2vl, Kv, os, osm, margin0, cv, ov)) &&
        !cell_pair(y.hi, y.lo, b.hi, b.lo, mirror != 0, cv_c, os, cv, ov)) {
        long long i64, o64;
        cell_fp64(v, sv, mirror != 0, (int)(nv / 2), os, i64, o64);
        cv = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
        ov = (int)max(min(o64, (long long)1 << 30), -((long long)1 << 30));
        ++fb;
    }
    idx[id * 4 + 0] = cu;
    idx[id * 4 + 1] = cv;
    idx[id * 4 + 2] = ou;
    idx[id * 4 + 3] = ov;
    if (fb && nfb) atomicAdd(nfb, fb);
}

__global__ void k_table(const double *cgk, int n, int npad, float *tab) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npad) tab[i] = i < n ? (float)cgk[i] : 0.f;
}

}  // namespace

struct Scratch {
    std::vector<void *> ptrs;
    cudaStream_t s;
    explicit Scratch(cudaStream_t st) : s(st) {}
    int get(void **p, size_t bytes) {
        int rc = scratch_alloc(p, bytes, s);
        if (rc == NGG_OK) ptrs.push_back(*p);
        return rc;
    }
    ~Scratch() {
        for (void *p : ptrs) scratch_free(p, s);
    }
};

struct Prof {
    bool on = false;
    bool valid = false;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
};
static thread_local Prof g_prof;

static void prof_record(int i, cudaStream_t s) {
    if (!g_prof.on) return;
    if (!g_prof.ev[i]) cudaEventCreate(&g_prof.ev[i]);
    cudaEventRecord(g_prof.ev[i], s);
    if (i == 2) g_prof.valid = true;
}

}  // namespace ngg

using namespace ngg;

extern "C" void ngg_set_profiling(int enable) {
    g_prof.on = enable != 0;
    g_prof.valid = false;
}

extern "C" int ngg_last_phase_ms(double *binning_ms, double *tiles_ms) {
    clear_error();
    if (!g_prof.valid) return fail(NGG_ERR_INVALID, "no profiled ngg_grid_ps call on this thread");
    NGG_CUDA(cudaEventSynchronize(g_prof.ev[2]));
    float a = 0.f, b = 0.f;
    NGG_CUDA(cudaEventElapsedTime(&a, g_prof.ev[0], g_prof.ev[1]));
    NGG_CUDA(cudaEventElapsedTime(&b, g_prof.ev[1], g_prof.ev[2]));
    if (binning_ms) *binning_ms = a;
    if (tiles_ms) *tiles_ms = b;
    return NGG_OK;
}

namespace {
// The device address through which a kernel reads p: device memory as is,
// pinned host memory through its mapping (read in place over the host link:
// no copy), NULL as NULL. Pageable host memory is refused.
int device_view(const void *p, const void **out, const char *what) {
    *out = p;
    if (!p) return NGG_OK;
    cudaPointerAttributes at;
    const cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(NGG_ERR_INVALID, std::string(what) + " is not a CUDA-visible pointer");
    }
    if (at.type == cudaMemoryTypeUnregistered)
        return fail(NGG_ERR_INVALID, std::string(what) + " is pageable host memory (pass device or pinned host memory)");
    if (at.type == cudaMemoryTypeHost) {
        if (!at.devicePointer) return fail(NGG_ERR_INVALID, std::string(what) + ": pinned memory without a device mapping");
        *out = at.devicePointer;
    }
    return NGG_OK;
}

int grid_ps_impl(const NggGridArgs *a, int64_t c_off, int64_t c_stride, const NggImagingWeights *iw, void *stream);
}  // namespace

extern "C" int ngg_grid_ps(const NggGridArgs *a, void *stream) {
    clear_error();
    if (!a) return fail(NGG_ERR_INVALID, "args is NULL");
    return grid_ps_impl(a, 0, a->n_chan, nullptr, stream);
}

extern "C" int ngg_grid_ps_chunk(const NggGridArgs *a, int64_t chan_offset, int64_t n_chan_total, void *stream) {
    clear_error();
    if (!a) return fail(NGG_ERR_INVALID, "args is NULL");
    if (chan_offset < 0 || a->n_chan < 0 || n_chan_total < chan_offset + a->n_chan)
        return fail(NGG_ERR_INVALID, "channel range outside the input arrays");
    return grid_ps_impl(a, chan_offset, n_chan_total, nullptr, stream);
}

extern "C" int ngg_grid_ps_weighted(const NggGridArgs *a, const NggImagingWeights *iw, void *stream) {
    clear_error();
    if (!a || !iw) return fail(NGG_ERR_INVALID, "args is NULL");
    if (iw->density) {
        if (!iw->factors) return fail(NGG_ERR_INVALID, "density without Briggs factors");
        if (iw->n_u < 1 || iw->n_v < 1 || iw->n_u > 65535 || iw->n_v > 65535)
            return fail(NGG_ERR_INVALID, "density grid size out of [1,65535]");
        if (a->n_pol > 2) return fail(NGG_ERR_UNSUPPORTED, "imaging weights from density: at most 2 pols");
    }
    return grid_ps_impl(a, 0, a->n_chan, iw, stream);
}

namespace {
int grid_ps_impl(const NggGridArgs *a, int64_t c_off, int64_t c_stride, const NggImagingWeights *iw, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (a->mode != NGG_MODE_DATA && a->mode != NGG_MODE_PSF) return fail(NGG_ERR_INVALID, "mode");
    if (a->chan_mode != NGG_CHAN_CUBE && a->chan_mode != NGG_CHAN_CONTINUUM) return fail(NGG_ERR_INVALID, "chan_mode");
    if (a->layout != NGG_LAYOUT_NATURAL && a->layout != NGG_LAYOUT_FFT) return fail(NGG_ERR_INVALID, "layout");
    if (a->support != SUP) return fail(NGG_ERR_UNSUPPORTED, "support must be 7");
    if (a->oversampling < 1 || a->oversampling > 1000) return fail(NGG_ERR_UNSUPPORTED, "oversampling out of [1,1000]");
    if (a->n_time < 0 || a->n_baseline < 0 || a->n_chan < 0 || a->n_pol < 1) return fail(NGG_ERR_INVALID, "negative dims");
    if (a->n_u < 1 || a->n_v < 1 || a->n_u > 65535 || a->n_v > 65535) return fail(NGG_ERR_INVALID, "grid size out of [1,65535]");
    if (!a->uvw && a->n_time * a->n_baseline > 0) return fail(NGG_ERR_INVALID, "uvw is NULL");
    if (!a->weight && a->n_time * a->n_baseline * a->n_chan > 0) return fail(NGG_ERR_INVALID, "weight is NULL");
    if (a->mode == NGG_MODE_DATA && !a->vis && a->n_time * a->n_baseline * a->n_chan > 0)
        return fail(NGG_ERR_INVALID, "vis is NULL in DATA mode");
    if (!a->grid || !a->sum_weight || !a->cgk_1D || (!a->freq && a->n_chan > 0)) return fail(NGG_ERR_INVALID, "NULL output/table");
    const int tab_len = a->oversampling * (a->support / 2 + 1);
    if (tab_len > MAX_TAB) return fail(NGG_ERR_UNSUPPORTED, "kernel table too long");

    const int64_t T = a->n_time, B = a->n_baseline, C = a->n_chan, P = a->n_pol;
    const void *vis_d = nullptr, *weight_d = nullptr;
    {
        int rc0 = device_view(a->mode == NGG_MODE_DATA ? a->vis : nullptr, &vis_d, "vis");
        if (rc0 == NGG_OK) rc0 = device_view(a->weight, &weight_d, "weight");
        if (rc0 != NGG_OK) return rc0;
    }
    const int n_img = a->chan_mode == NGG_CHAN_CONTINUUM ? 1 : (int)C;
    const bool cplx = a->mode == NGG_MODE_DATA;
    const bool fftl = a->layout == NGG_LAYOUT_FFT;
    const size_t elem = (cplx || fftl) ? 8 : 4;
    const int64_t nu = a->n_u, nv = a->n_v;
    const int ntu = (int)((nu + TU - 1) / TU), ntv = (int)((nv + TV - 1) / TV);
    const int nk = (int)((T + CH - 1) / CH);

    if (n_img == 0) return NGG_OK;
    g_prof.valid = false;
    prof_record(0, s);
    NGG_CUDA(cudaMemsetAsync(a->sum_weight, 0, sizeof(double) * (size_t)n_img * P, s));

    Scratch sc(s);
    int rc;
    const int tab_bytes = ((tab_len * 4 + 15) / 16) * 16;
    float *tab = nullptr;
    if ((rc = sc.get((void **)&tab, tab_bytes)) != NGG_OK) return rc;
    k_table<<<(tab_bytes / 4 + 255) / 256, 256, 0, s>>>(a->cgk_1D, tab_len, tab_bytes / 4, tab);
    NGG_CHECK_LAUNCH("k_table");

    ChanParms *chan = nullptr;
    float4 *uvs = nullptr, *bbox = nullptr;
    if (C > 0 && (rc = sc.get((void **)&chan, sizeof(ChanParms) * C)) != NGG_OK) return rc;
    const int64_t n_chunks = C * B * nk;
    if (n_chunks >= (int64_t)1 << 32) return fail(NGG_ERR_UNSUPPORTED, "more than 2^32 track chunks");
    int64_t n_keys = 0;
    unsigned long long *keys_sorted = nullptr;
    const int64_t n_bins = (int64_t)n_img * ntu * ntv;
    int64_t *bin_start = nullptr;
    if ((rc = sc.get((void **)&bin_start, sizeof(int64_t) * (n_bins + 1))) != NGG_OK) return rc;

    if (n_chunks > 0) {
        if ((rc = sc.get((void **)&uvs, sizeof(float4) * T * B)) != NGG_OK) return rc;
        if ((rc = sc.get((void **)&bbox, sizeof(float4) * B * nk)) != NGG_OK) return rc;
        k_chan<<<(int)((C + 127) / 128), 128, 0, s>>>(a->freq, (int)C, a->delta_lm[0], a->delta_lm[1], nu, nv, chan);
        NGG_CHECK_LAUNCH("k_chan");
        {
            int64_t warps = B * nk;
            k_uvw<<<(unsigned)((warps + 7) / 8), 256, 0, s>>>(a->uvw, T, B, nk, uvs, bbox);
            NGG_CHECK_LAUNCH("k_uvw");
        }
        unsigned *counts = nullptr;
        unsigned long long *offsets = nullptr;
        if ((rc = sc.get((void **)&counts, sizeof(unsigned) * (n_chunks + 1))) != NGG_OK) return rc;
        if ((rc = sc.get((void **)&offsets, sizeof(unsigned long long) * (n_chunks + 1))) != NGG_OK) return rc;
        const unsigned nb = (unsigned)((n_chunks + 255) / 256);
        k_count<<<nb, 256, 0, s>>>(bbox, chan, C, B, nk, nu, nv, ntu, ntv, counts);
        NGG_CHECK_LAUNCH("k_count");
        size_t tmp_bytes = 0;
        NGG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, counts, offsets, n_chunks + 1, s));
        void *tmp = nullptr;
        if ((rc = sc.get(&tmp, tmp_bytes)) != NGG_OK) return rc;
        NGG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, counts, offsets, n_chunks + 1, s));
        unsigned long long total = 0;
        NGG_CUDA(cudaMemcpyAsync(&total, offsets + n_chunks, sizeof(total), cudaMemcpyDeviceToHost, s));
        NGG_CUDA(cudaStreamSynchronize(s));
        n_keys = (int64_t)total;
        if (n_keys > 0) {
            unsigned long long *keys = nullptr;
            if ((rc = sc.get((void **)&keys, sizeof(unsigned long long) * n_keys)) != NGG_OK) return rc;
            if ((rc = sc.get((void **)&keys_sorted, sizeof(unsigned long long) * n_keys)) != NGG_OK) return rc;
            k_emit<<<nb, 256, 0, s>>>(bbox, chan, C, B, nk, nu, nv, ntu, ntv,
                                       a->chan_mode == NGG_CHAN_CONTINUUM, offsets, keys);
            NGG_CHECK_LAUNCH("k_emit");
            // k_emit writes each chunk's keys in chunk order, so a stable
            // sort on the tile bits alone (LSD radix sort is stable) leaves
            // every tile's chunks in (chan, baseline, time) order: sorted by
            // the whole key, bins (tile, image channel) in order
            int end_bit = 32;
            while (end_bit < 64 && ((unsigned long long)((int64_t)ntu * ntv) >> (end_bit - 32)) > 0) ++end_bit;
            size_t sort_bytes = 0;
            NGG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, keys, keys_sorted, n_keys, 32, end_bit, s));
            void *stmp = nullptr;
            if ((rc = sc.get(&stmp, sort_bytes)) != NGG_OK) return rc;
            NGG_CUDA(cub::DeviceRadixSort::SortKeys(stmp, sort_bytes, keys, keys_sorted, n_keys, 32, end_bit, s));
        }
    }
    k_bounds<<<(unsigned)((n_bins + 1 + 255) / 256), 256, 0, s>>>(
        keys_sorted, n_keys, n_bins, (int)n_img, a->chan_mode == NGG_CHAN_CONTINUUM ? 0 : B * (int64_t)nk, bin_start);
    NGG_CHECK_LAUNCH("k_bounds");

    int *counter = nullptr;
    if ((rc = sc.get((void **)&counter, sizeof(int) * 128)) != NGG_OK) return rc;
    NGG_CUDA(cudaMemsetAsync(counter, 0, sizeof(int) * 128, s));
    int *bbox_d = nullptr;
    if ((rc = sc.get((void **)&bbox_d, sizeof(int) * 4)) != NGG_OK) return rc;
    k_bbox_init<<<1, 1, 0, s>>>(bbox_d);
    k_bbox<<<(unsigned)((n_bins + 255) / 256), 256, 0, s>>>(bin_start, n_bins, (int)n_img, ntv, bbox_d);
    NGG_CHECK_LAUNCH("k_bbox");
    // tile work items: every (tile in the busy box, channel); bins with more
    // than MAXE entries become several items
    const int64_t n_bound = n_bins;   // box items <= bins
    int *nsub = nullptr, *soff = nullptr, *n_subs_d = nullptr;
    SubItem *subs = nullptr;
    if ((rc = sc.get((void **)&nsub, sizeof(int) * (n_bound + 1))) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&soff, sizeof(int) * (n_bound + 1))) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&n_subs_d, sizeof(int))) != NGG_OK) return rc;
    const int64_t max_subs = n_bound + n_keys / MAXE + 2;
    if (max_subs >= ((int64_t)1 << 31)) return fail(NGG_ERR_UNSUPPORTED, "too many tile work items");
    if ((rc = sc.get((void **)&subs, sizeof(SubItem) * max_subs)) != NGG_OK) return rc;
    k_nsub<<<(unsigned)((n_bound + 1 + 255) / 256), 256, 0, s>>>(bin_start, bbox_d, n_img, ntv, n_bound, nsub);
    NGG_CHECK_LAUNCH("k_nsub");
    {
        size_t tb = 0;
        NGG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, nsub, soff, n_bound + 1, s));
        void *tmp2 = nullptr;
        if ((rc = sc.get(&tmp2, tb)) != NGG_OK) return rc;
        NGG_CUDA(cub::DeviceScan::ExclusiveSum(tmp2, tb, nsub, soff, n_bound + 1, s));
    }
    k_fill_subs<<<(unsigned)((n_bound + 1 + 255) / 256), 256, 0, s>>>(nsub, soff, n_bound + 1, subs, n_subs_d);
    NGG_CHECK_LAUNCH("k_fill_subs");

    // packed steps, one pass per launch's pols (reused across launches)
    uint2 *meta = nullptr;
    float4 *wvp = nullptr;
    double *sw_part = nullptr;
    float *nsum = nullptr;
    const int64_t n_slots = C * B * (int64_t)nk * CH;
    if (n_chunks > 0) {
        if ((rc = sc.get((void **)&meta, sizeof(uint2) * n_slots)) != NGG_OK) return rc;
        if ((rc = sc.get((void **)&wvp, sizeof(float4) * n_slots)) != NGG_OK) return rc;
        if ((rc = sc.get((void **)&sw_part, sizeof(double) * 2 * C * B * nk)) != NGG_OK) return rc;
        if ((rc = sc.get((void **)&nsum, sizeof(float) * (a->oversampling + 1))) != NGG_OK) return rc;
        k_nsum<<<(a->oversampling + 1 + 127) / 128, 128, 0, s>>>(tab, tab_len, a->oversampling, nsum);
        NGG_CHECK_LAUNCH("k_nsum");
    }

    // imaging weights formed in the packing pass: per-channel scale of the density grid
    ChanParms *dchan = nullptr;
    const bool fused_w = iw && iw->density && n_chunks > 0;
    if (fused_w) {
        if ((rc = sc.get((void **)&dchan, sizeof(ChanParms) * C)) != NGG_OK) return rc;
        k_chan<<<(int)((C + 127) / 128), 128, 0, s>>>(a->freq, (int)C, a->delta_lm[0], a->delta_lm[1], iw->n_u,
                                                     iw->n_v, dchan);
        NGG_CHECK_LAUNCH("k_chan (density)");
    }

    TileArgs ta;
    ta.vis = (const float2 *)vis_d;
    ta.weight = (const float *)weight_d;
    ta.uvw = a->uvw;
    ta.uvs = uvs;
    ta.chan = chan;
    ta.tab_g = tab;
    ta.keys = keys_sorted;
    ta.bin_start = bin_start;
    ta.grid = a->grid;
    ta.sum_weight = a->sum_weight;
    ta.T = T; ta.B = B; ta.C = C; ta.P = P;
    ta.nu = nu; ta.nv = nv;
    ta.n_img = n_img; ta.ntu = ntu; ta.ntv = ntv; ta.nk = nk;
    ta.os = a->oversampling;
    ta.tab_len = tab_len;
    ta.tab_bytes = tab_bytes;
    ta.continuum = a->chan_mode == NGG_CHAN_CONTINUUM;
    ta.bbox = bbox_d;
    ta.subs = subs;
    ta.n_subs = n_subs_d;
    ta.bnk = (unsigned)(B * nk);
    (void)elem;
    for (int64_t p0 = 0, launch = 0; p0 < P; ++launch) {
        const int np = (P - p0) >= 2 ? 2 : 1;
        ta.p0 = (int)p0;
        ta.work_counter = counter + 2 * launch;
        ta.err = counter + 127;
        if (n_chunks > 0) {
            PackArgs pa;
            pa.vis = (const float2 *)vis_d;
            pa.weight = (const float *)weight_d;
            pa.uvw = a->uvw;
            pa.uvs = uvs;
            pa.chan = chan;
            pa.nsum = nsum;
            pa.meta = meta;
            pa.wvp = wvp;
            pa.sw_part = sw_part;
            pa.T = T; pa.B = B; pa.C = C; pa.P = P;
            pa.c_stride = c_stride; pa.c_off = c_off;
            pa.nu = nu; pa.nv = nv;
            pa.nk = nk; pa.p0 = (int)p0; pa.os = a->oversampling;
            {
                const int64_t ku = (2 * (nu / 2) + 1) * (int64_t)a->oversampling;
                const int64_t kv = (2 * (nv / 2) + 1) * (int64_t)a->oversampling;
                pa.half_ok = a->oversampling >= 1 && a->oversampling < 65536 && ku < (1 << 24) && kv < (1 << 24);
                pa.ku = (int)ku;
                pa.kv = (int)kv;
                pa.osm = os_magic(a->oversampling);
                pa.margin0 = half_margin(a->oversampling);
                pa.vec2 = np == 2 && P == 2 && p0 == 0 && ((uintptr_t)vis_d & 15) == 0 &&
                          ((uintptr_t)weight_d & 7) == 0;
            }
            pa.density = fused_w ? iw->density : nullptr;
            pa.factors = fused_w ? iw->factors : nullptr;
            pa.dchan = dchan;
            pa.flag = (iw && cplx) ? iw->flag : nullptr;
            pa.dnu = fused_w ? iw->n_u : 1;
            pa.dnv = fused_w ? iw->n_v : 1;
            pa.n_img = n_img;
            pa.continuum = a->chan_mode == NGG_CHAN_CONTINUUM;
            const dim3 pg((unsigned)B, (unsigned)nk, (unsigned)((C + 31) / 32)), pb(32, 8);
            // the imaging-weight / flag variant only where it is asked for (its
            // extra registers cost the plain pass a third of its speed)
            const bool fused = pa.density != nullptr || pa.flag != nullptr;
            if (np == 2) {
                if (cplx) {
                    if (fused) k_pack<2, true, true><<<pg, pb, 0, s>>>(pa); else k_pack<2, true, false><<<pg, pb, 0, s>>>(pa);
                } else {
                    if (fused) k_pack<2, false, true><<<pg, pb, 0, s>>>(pa); else k_pack<2, false, false><<<pg, pb, 0, s>>>(pa);
                }
            } else {
                if (cplx) {
                    if (fused) k_pack<1, true, true><<<pg, pb, 0, s>>>(pa); else k_pack<1, true, false><<<pg, pb, 0, s>>>(pa);
                } else {
                    if (fused) k_pack<1, false, true><<<pg, pb, 0, s>>>(pa); else k_pack<1, false, false><<<pg, pb, 0, s>>>(pa);
                }
            }
            NGG_CHECK_LAUNCH("k_pack");
            k_sw_reduce<<<(unsigned)(n_img * np), 256, 0, s>>>(sw_part, C, np, B * nk, ta.continuum, P, (int)p0,
                                                                a->sum_weight);
            NGG_CHECK_LAUNCH("k_sw_reduce");
        }
        ta.meta = meta;
        ta.wvp = wvp;
        if (launch == 0) prof_record(1, s);   // phases: binning + packing | tile pass
        rc = np == 2 ? dispatch_tiles<2>(ta, n_bound, cplx, fftl, s) : dispatch_tiles<1>(ta, n_bound, cplx, fftl, s);
        if (rc != NGG_OK) return rc;
        p0 += np;
        if (launch >= 62) return fail(NGG_ERR_UNSUPPORTED, "too many polarizations");
    }
    prof_record(2, s);
    // the tile kernel's bounded wait for its table copy: report a time-out
    int err = 0;
    NGG_CUDA(cudaMemcpyAsync(&err, counter + 127, sizeof(int), cudaMemcpyDeviceToHost, s));
    NGG_CUDA(cudaStreamSynchronize(s));
    if (err) return fail(NGG_ERR_TIMEOUT, "k_tiles: the kernel table copy did not complete in time");
    return NGG_OK;
}
}  // namespace

extern "C" int ngg_cell_indices(int64_t n_rows, int64_t C, const double *uvw, const double *freq, int64_t nu,
                                int64_t nv, const double delta_lm[2], int os, int mirror, int32_t *idx,
                                long long *n_fallback, void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (n_rows < 0 || C < 0 || nu < 1 || nv < 1 || os < 0 || os > 1000 || !delta_lm) return fail(NGG_ERR_INVALID, "dims");
    if (n_fallback) NGG_CUDA(cudaMemsetAsync(n_fallback, 0, sizeof(long long), s));
    if (n_rows * C == 0) return NGG_OK;
    if (!uvw || !freq || !idx) return fail(NGG_ERR_INVALID, "NULL pointer");
    const int64_t n = n_rows * C;
    k_cell_indices<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n_rows, C, uvw, freq, nu, nv, delta_lm[0], delta_lm[1],
                                                               os, mirror, os_magic(os), half_margin(os), idx,
                                                               (unsigned long long *)n_fallback);
    NGG_CHECK_LAUNCH("k_cell_indices");
    return NGG_OK;
}
