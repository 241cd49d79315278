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
//  Inside a busy tile each warp runs 8 track processors of 4 lanes. A lane
//  owns up to two of the 7 column residue classes (Romein's work
//  distribution) and, for each, the 7 rows of the current footprint in
//  registers; it adds tap*tap*datum in registers while its cells stay the
//  same and flushes a cell to shared memory (atomic add) when the track
//  moves off it or, at the latest, every second 32-step chunk. Taps come from the oversampled table, loaded into shared
//  memory by a TMA bulk copy. Cell and oversampling indices are certified to
//  equal the reference's FP64 results (see cell_pair).
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "ngg_internal.cuh"

namespace ngg {
namespace {

constexpr int TU = 64;      // tile rows (u)
constexpr int TV = 64;      // tile columns (v, contiguous)
constexpr int CH = 32;      // time steps per chunk
constexpr int NW = 8;       // warps per CTA
constexpr int NG = 8;       // track processors per warp (4 lanes each)
constexpr int ROUND = 8;    // producer round length (steps)
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
};

// One pass over the visibilities (time, baseline, chan, pol): per step its
// cell and oversampling offsets (the FP64 index chain, certified FP32 pairs),
// its weighted data and its sum_weight term, written track-major
// ([chan][baseline][time]) so that the tile kernel reads each 32-step chunk
// as one contiguous run however many tiles the chunk touches. A block is 32
// channels x 32 steps of one (baseline, chunk): the reads are contiguous over
// channels, a shared-memory transpose makes the writes contiguous over time.
template <int NP, bool CPLX>
__global__ void __launch_bounds__(256) k_pack(const PackArgs a) {
    __shared__ uint2 s_meta[32][33];
    __shared__ float4 s_wv[32][33];
    __shared__ float s_sw[NP][32][9];       // per channel: the 8 row-threads' partial sums
    __shared__ float s_nsum[MAX_OS + 1];
    const int x = threadIdx.x;
    const int64_t b = blockIdx.x;
    const int k = blockIdx.y;
    const int64_t c0 = (int64_t)blockIdx.z * 32;
    const int cu_c = (int)(a.nu / 2), cv_c = (int)(a.nv / 2);
    for (int i = threadIdx.y * 32 + x; i <= a.os; i += 256) s_nsum[i] = a.nsum[i];
    __syncthreads();
    float swc[NP];   // this thread's sum_weight terms over its 4 steps
#pragma unroll
    for (int p = 0; p < NP; ++p) swc[p] = 0.f;
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int64_t c = c0 + x, t = (int64_t)k * CH + y;
        uint2 meta = make_uint2(NO_CELL, 0u);
        float4 wv = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c < a.C && t < a.T) {
            const float4 us = a.uvs[b * a.T + t];
            if (!isnan(us.x) && !isnan(us.z)) {
                const ChanParms cp = a.chan[c];
                int cu, ou, cv, ov;
                if (!cell_pair(us.x, us.y, cp.suh, cp.sul, false, cu_c, a.os, cu, ou)) {
                    long long i64, o64;
                    cell_fp64(a.uvw[(t * a.B + b) * 3 + 0], cp.su, false, cu_c, a.os, i64, o64);
                    cu = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
                    ou = (int)o64;
                }
                if (!cell_pair(us.z, us.w, cp.svh, cp.svl, false, cv_c, a.os, cv, ov)) {
                    long long i64, o64;
                    cell_fp64(a.uvw[(t * a.B + b) * 3 + 1], cp.sv, false, cv_c, a.os, i64, o64);
                    cv = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
                    ov = (int)o64;
                }
                if (cu - SC >= 0 && cu + SC < a.nu && cv - SC >= 0 && cv + SC < a.nv) {
                    const int64_t base = ((t * a.B + b) * a.c_stride + a.c_off + c) * a.P + a.p0;
                    float w[NP];
                    bool pv[NP];
                    bool any = false;
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        w[p] = a.weight[base + p];
                        if constexpr (CPLX) {
                            const float2 vv = a.vis[base + p];
                            const float xr = vv.x * w[p], xi = vv.y * w[p];
                            pv[p] = !isnan(xr) && !isnan(xi) && (xr != 0.f || xi != 0.f);
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
    int64_t cimg = continuum ? 0 : c;
    int64_t NT = (int64_t)ntu * ntv;
    for (int tu = r.u0; tu <= r.u1; ++tu)
        for (int tv = r.v0; tv <= r.v1; ++tv) {
            unsigned long long bin = (unsigned long long)(cimg * NT + (int64_t)tu * ntv + tv);
            keys[o++] = (bin << 32) | (unsigned long long)ch;
        }
}

__global__ void k_bbox_init(int *bb) {
    bb[0] = 0x7fffffff; bb[1] = -1; bb[2] = 0x7fffffff; bb[3] = -1;
}

// range of tiles holding any chunk, over all image channels
__global__ void k_bbox(const int64_t *bin_start, int64_t n_bins, int64_t NT, int ntv, int *bb) {
    const int64_t bin = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (bin >= n_bins || bin_start[bin] == bin_start[bin + 1]) return;
    const int64_t tile = bin % NT;
    const int tu = (int)(tile / ntv), tv = (int)(tile % ntv);
    atomicMin(&bb[0], tu); atomicMax(&bb[1], tu);
    atomicMin(&bb[2], tv); atomicMax(&bb[3], tv);
}

__global__ void k_bounds(const unsigned long long *keys, int64_t n, int64_t n_bins, int64_t *bin_start) {
    int64_t bin = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (bin > n_bins) return;
    unsigned long long target = (unsigned long long)bin << 32;
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

__device__ __forceinline__ int mod7(int x) {
    int r = x % 7;
    return r < 0 ? r + 7 : r;
}

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
    int64_t NT;
    int ntv;
    __device__ __forceinline__ void map(int64_t item, int &tiu, int &tiv, int &cimg, int64_t &bin) const {
        const int64_t tix = item / n_img;
        cimg = (int)(item % n_img);
        tiu = bt0 + (int)(tix / nbv);
        tiv = bv0 + (int)(tix % nbv);
        bin = (int64_t)cimg * NT + (int64_t)tiu * ntv + tiv;
    }
};

__device__ __forceinline__ BoxMap box_map(const int *bbox, int n_img, int64_t NT, int ntv) {
    BoxMap m;
    const bool have = bbox[0] <= bbox[1] && bbox[2] <= bbox[3];
    m.bt0 = bbox[0];
    m.bv0 = bbox[2];
    m.nbu = have ? bbox[1] - bbox[0] + 1 : 0;
    m.nbv = have ? bbox[3] - bbox[2] + 1 : 0;
    m.n_img = n_img;
    m.NT = NT;
    m.ntv = ntv;
    return m;
}

// number of work items of every box item (0 beyond the box)
__global__ void k_nsub(const int64_t *bin_start, const int *bbox, int n_img, int64_t NT, int ntv, int64_t n_bound,
                       int *nsub) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n_bound) return;
    const BoxMap m = box_map(bbox, n_img, NT, ntv);
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
// their partial tiles with atomics)
template <bool CPLX, bool FFTL>
__global__ void k_zero_split(const int64_t *bin_start, const int *bbox, int n_img, int64_t NT, int ntv,
                             int64_t n_bound, void *grid, int64_t P, int p0, int np, int64_t nu, int64_t nv) {
    const int64_t i = blockIdx.x;
    if (i >= n_bound) return;
    const BoxMap m = box_map(bbox, n_img, NT, ntv);
    if (i >= (int64_t)m.nbu * m.nbv * n_img) return;
    int tiu, tiv, cimg;
    int64_t bin;
    m.map(i, tiu, tiv, cimg, bin);
    if (bin_start[bin + 1] - bin_start[bin] <= MAXE) return;
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
    asm volatile("cp.async.bulk.wait_group.read 32;" ::: "memory");   // bound the stores in flight
    return true;
}

// register accumulator of one (column, row) cell
template <bool CPLX>
struct Cell;
template <>
struct Cell<true> { float2 a, b; };   // (re, im) of pol 0 and pol 1
template <>
struct Cell<false> { float2 a; };     // (pol 0, pol 1) of a real grid

template <int NP, bool CPLX, bool FFTL>
__global__ void __launch_bounds__(NW * 32, 2) k_tiles(const TileArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    // layout: acc tile | table | norm sums | records | group info | misc
    constexpr int ACC_ELEM = CPLX ? 8 : 4;
    constexpr int NREC = NG * ROUND;   // records per warp
    float *acc_s = reinterpret_cast<float *>(smem);
    const size_t acc_bytes = (size_t)NP * TU * TV * ACC_ELEM;
    float *tab = reinterpret_cast<float *>(smem + acc_bytes);
    // per warp: the round's step records (taps, cell, info) and, double
    // buffered, the packed steps of this round and the next (cp.async)
    float4 *rec_tv = reinterpret_cast<float4 *>(tab + ((a.tab_bytes + 3) / 4));   // 2 per record
    unsigned *rec_cuv = reinterpret_cast<unsigned *>(rec_tv + 2 * NW * NREC);
    int *rec_info = reinterpret_cast<int *>(rec_cuv + NW * NREC);
    int4 *ginfo = reinterpret_cast<int4 *>(rec_info + NW * NREC);   // (c, b, t0, valid) per group
    float4 *raw_wv = reinterpret_cast<float4 *>(ginfo + NW * NG);    // [NW][2][NREC]
    uint2 *raw_meta = reinterpret_cast<uint2 *>(raw_wv + NW * 2 * NREC);
    unsigned long long *mbar = reinterpret_cast<unsigned long long *>(raw_meta + NW * 2 * NREC);
    int *s_item = reinterpret_cast<int *>(mbar + 1);   // [kind, item]
    float4 *zbuf = reinterpret_cast<float4 *>(
        (reinterpret_cast<uintptr_t>(s_item + 2) + 15) & ~static_cast<uintptr_t>(15));

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;

    // ---- stage the tap table with a TMA bulk copy -------------------------
    unsigned mbar_addr = (unsigned)__cvta_generic_to_shared(mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_addr) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        unsigned dst = (unsigned)__cvta_generic_to_shared(tab);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar_addr), "r"(a.tab_bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
            "l"(a.tab_g), "r"(a.tab_bytes), "r"(mbar_addr)
            : "memory");
    }
    const bool tma_ok = mbar_wait(mbar_addr, 0);
    if (!tma_ok) {  // the bounded wait ran out: fall back to plain loads
        for (int i = tid; i < a.tab_len; i += blockDim.x) tab[i] = a.tab_g[i];
    }
    __syncthreads();
    for (int i = tid; i < NP * TU * TV * (CPLX ? 2 : 1); i += blockDim.x) acc_s[i] = 0.f;
    for (int i = tid; i < ZBUF / 16; i += blockDim.x) zbuf[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // the bulk stores read zbuf
    __syncthreads();
    const unsigned zs = (unsigned)__cvta_generic_to_shared(zbuf);

    const int64_t NT = (int64_t)a.ntu * a.ntv;
    const int cu_c = (int)(a.nu / 2), cv_c = (int)(a.nv / 2);
    const int g = lane >> 2;            // track processor in the warp
    const int l4 = lane & 3;            // lane within the processor
    const int ncol = (l4 < 3) ? 2 : 1;  // column classes l4 and l4+4
    const int64_t plane = a.nu * a.nv;
    const BoxMap bm = box_map(a.bbox, a.n_img, NT, a.ntv);
    const int R0 = bm.nbu ? bm.bt0 * TU : 0, R1 = bm.nbu ? min((bm.bt0 + bm.nbu) * TU, (int)a.nu) : 0;
    const int V0 = bm.nbv ? bm.bv0 * TV : 0, V1 = bm.nbv ? min((bm.bv0 + bm.nbv) * TV, (int)a.nv) : 0;
    const int64_t n_tile_items = *a.n_subs;
    constexpr int ZR = 8;
    const int nrb = (int)((a.nu + ZR - 1) / ZR);
    const int64_t n_zero_items = (int64_t)a.n_img * NP * nrb;

    int4 *my_ginfo = ginfo + warp * NG;
    unsigned *my_cuv = rec_cuv + warp * NREC;
    int *my_info = rec_info + warp * NREC;
    float4 *my_tv = rec_tv + 2 * warp * NREC;
    float4 *my_raw_wv = raw_wv + warp * 2 * NREC;
    uint2 *my_raw_meta = raw_meta + warp * 2 * NREC;

    // Rows outside the busy box are zeroed by TMA bulk stores that lane 0 of
    // each warp issues, one block of rows at a time, just before the warp
    // waits at a tile barrier (the rest after the last tile): the grid write
    // they carry overlaps the tile work instead of taking CTAs away from it.
    const ZeroRows zr{a.grid, a.nu, a.nv, a.P, a.p0, nrb, n_zero_items, R0, R1, V0, V1, cu_c, cv_c, zs,
                      &a.work_counter[1]};
    bool zero_left = lane == 0;   // this warp's issuing lane: zero row blocks remain
    for (;;) {
        if (tid == 0) {
            const long long it = atomicAdd(&a.work_counter[0], 1);
            s_item[0] = it < n_tile_items ? 0 : -1;
            s_item[1] = (int)it;
        }
        __syncthreads();
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
            // ---------------- busy tile ----------------
            const int64_t n = e1 - e0;
            const int gi = warp * NG + g;
            const int64_t rs = e0 + (n * gi) / (NW * NG);
            const int64_t re = e0 + (n * (gi + 1)) / (NW * NG);
            int jmax = (int)(re - rs);
            for (int o = 16; o > 0; o >>= 1) jmax = max(jmax, __shfl_xor_sync(0xffffffffu, jmax, o));
            int prev_cu = -(1 << 28), prev_cv = -(1 << 28);
            int col[2] = {-(1 << 28), -(1 << 28)};
            bool colv[2] = {false, false};
            Cell<CPLX> acc[2][SUP];
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int d = 0; d < SUP; ++d) {
                    acc[j][d].a = make_float2(0.f, 0.f);
                    if constexpr (CPLX) acc[j][d].b = make_float2(0.f, 0.f);
                }

            auto flush_cell = [&](int j, int d) {
                const int row = prev_cv - SC + d;
                if (!colv[j] || row < v0 || row >= v0 + TV || row >= a.nv) return;
                const int lu = col[j] - u0, lv = row - v0;
                if constexpr (CPLX) {
                    const float2 x = acc[j][d].a;
                    if (x.x != 0.f || x.y != 0.f) {
                        float *q = acc_s + 2 * ((size_t)lu * TV + lv);
                        atomicAdd(q, x.x);
                        atomicAdd(q + 1, x.y);
                    }
                    if (NP > 1) {
                        const float2 y = acc[j][d].b;
                        if (y.x != 0.f || y.y != 0.f) {
                            float *q = acc_s + 2 * (((size_t)TU + lu) * TV + lv);
                            atomicAdd(q, y.x);
                            atomicAdd(q + 1, y.y);
                        }
                    }
                } else {
                    const float2 x = acc[j][d].a;
                    if (x.x != 0.f) atomicAdd(acc_s + (size_t)lu * TV + lv, x.x);
                    if (NP > 1 && x.y != 0.f) atomicAdd(acc_s + ((size_t)TU + lu) * TV + lv, x.y);
                }
            };
            auto zero_cell = [&](int j, int d) {
                acc[j][d].a = make_float2(0.f, 0.f);
                if constexpr (CPLX) acc[j][d].b = make_float2(0.f, 0.f);
            };

            // chunk j of each group -> my_ginfo (lanes 0..NG-1)
            auto decode = [&](int j) {
                if (lane < NG) {
                    const int ggi = warp * NG + lane;
                    const int64_t grs = e0 + (n * ggi) / (NW * NG);
                    const int64_t gre = e0 + (n * (ggi + 1)) / (NW * NG);
                    int4 gi4 = make_int4(0, 0, 0, 0);
                    if (grs + j < gre) {
                        const unsigned chu = (unsigned)(a.keys[grs + j] & 0xffffffffull);
                        const unsigned cq = chu / a.bnk;
                        const unsigned rem = chu - cq * a.bnk;
                        const unsigned bq = rem / (unsigned)a.nk;
                        gi4 = make_int4((int)cq, (int)bq, (int)((rem - bq * (unsigned)a.nk) * CH), 1);
                    }
                    my_ginfo[lane] = gi4;
                }
                __syncwarp();
            };
            // start the copies of round rnd of the current chunks into buffer buf:
            // each lane its two packed steps (meta 8 bytes, data 16 bytes)
            auto prefetch = [&](int rnd, int buf) {
#pragma unroll
                for (int k2 = 0; k2 < 2; ++k2) {
                    // record q = s*NG + gg: the processors' records of one step are adjacent
                    const int r = lane + 32 * k2;
                    const int gg = r % NG, s = r / NG;
                    const int4 gi4 = my_ginfo[gg];
                    uint2 *dm = my_raw_meta + buf * NREC + r;
                    if (gi4.w) {
                        const int64_t ri = ((int64_t)gi4.x * a.B + gi4.y) * ((int64_t)a.nk * CH) + gi4.z +
                                           rnd * ROUND + s;
                        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                                         (unsigned)__cvta_generic_to_shared(dm)),
                                     "l"(a.meta + ri)
                                     : "memory");
                        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                                         (unsigned)__cvta_generic_to_shared(my_raw_wv + buf * NREC + r)),
                                     "l"(a.wvp + ri)
                                     : "memory");
                    } else {
                        *dm = make_uint2(NO_CELL, 0u);
                    }
                }
            };
            if (jmax > 0) {
                decode(0);
                prefetch(0, 0);
            }
            asm volatile("cp.async.commit_group;" ::: "memory");

            for (int j = 0; j < jmax; ++j) {
                for (int rnd = 0; rnd < CH / ROUND; ++rnd) {
                    const int buf = rnd & 1;   // CH / ROUND is even: round parity continues across chunks
                    // copies of the next round overlap this one
                    if (rnd + 1 < CH / ROUND) {
                        prefetch(rnd + 1, buf ^ 1);
                    } else if (j + 1 < jmax) {
                        decode(j + 1);
                        prefetch(0, buf ^ 1);
                    }
                    asm volatile("cp.async.commit_group;" ::: "memory");
                    asm volatile("cp.async.wait_group 1;" ::: "memory");   // this round's copies are in
                    // ---- producer: taps of this lane's two steps ----
#pragma unroll
                    for (int k2 = 0; k2 < 2; ++k2) {
                        const int r = lane + 32 * k2;
                        const uint2 m = my_raw_meta[buf * NREC + r];
                        unsigned cuv = 0;
                        int info = 0;
                        float4 tva = make_float4(0.f, 0.f, 0.f, 0.f), tvb = tva;
                        if (m.x != NO_CELL) {
                            const int ou = (int)(m.y & 0xffffu) - 32768, ov = (int)(m.y >> 16) - 32768;
                            cuv = m.x;
                            info = 1 | ((ou + 1024) << 1);
                            float tv[SUP];
#pragma unroll
                            for (int d = 0; d < SUP; ++d) tv[d] = tab[abs(a.os * (d - SC) + ov)];
                            tva = make_float4(tv[0], tv[1], tv[2], tv[3]);
                            tvb = make_float4(tv[4], tv[5], tv[6], 0.f);
                        }
                        my_cuv[r] = cuv;
                        my_info[r] = info;
                        my_tv[r] = tva;
                        my_tv[NREC + r] = tvb;
                    }
                    __syncwarp();
                    // ---- consumer: ROUND steps of this processor's chunk ----
                    for (int s = 0; s < ROUND; ++s) {
                        const int ri = s * NG + g;
                        const int info = my_info[ri];
                        if (!(info & 1)) continue;
                        const unsigned cuv = my_cuv[ri];
                        const int cu = (int)(cuv >> 16), cv = (int)(cuv & 0xffffu);
                        const int ou = ((info >> 1) & 2047) - 1024;
                        if (cu != prev_cu) {
#pragma unroll
                            for (int jj = 0; jj < 2; ++jj) {
                                if (jj < ncol) {
                                    const int nc = cu - SC + mod7(l4 + 4 * jj - (cu - SC));
                                    if (nc != col[jj]) {
#pragma unroll
                                        for (int d = 0; d < SUP; ++d) { flush_cell(jj, d); zero_cell(jj, d); }
                                        col[jj] = nc;
                                        colv[jj] = (nc >= u0 && nc < u0 + TU && nc < a.nu);
                                    }
                                }
                            }
                            prev_cu = cu;
                        }
                        if (cv != prev_cv) {
                            int delta = cv - prev_cv;
                            if (delta >= SUP || delta <= -SUP) {
#pragma unroll
                                for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                                    for (int d = 0; d < SUP; ++d) { flush_cell(jj, d); zero_cell(jj, d); }
                                prev_cv = cv;
                            } else {
                                while (delta > 0) {
#pragma unroll
                                    for (int jj = 0; jj < 2; ++jj) {
                                        flush_cell(jj, 0);
#pragma unroll
                                        for (int d = 0; d < SUP - 1; ++d) acc[jj][d] = acc[jj][d + 1];
                                        zero_cell(jj, SUP - 1);
                                    }
                                    ++prev_cv;
                                    --delta;
                                }
                                while (delta < 0) {
#pragma unroll
                                    for (int jj = 0; jj < 2; ++jj) {
                                        flush_cell(jj, SUP - 1);
#pragma unroll
                                        for (int d = SUP - 1; d > 0; --d) acc[jj][d] = acc[jj][d - 1];
                                        zero_cell(jj, 0);
                                    }
                                    --prev_cv;
                                    ++delta;
                                }
                            }
                        }
                        const float4 wv = my_raw_wv[buf * NREC + ri];
                        const float4 tva = my_tv[ri], tvb = my_tv[NREC + ri];
                        const float tv[SUP] = {tva.x, tva.y, tva.z, tva.w, tvb.x, tvb.y, tvb.z};
#pragma unroll
                        for (int jj = 0; jj < 2; ++jj) {
                            if (jj < ncol) {
                                const float tu = tab[abs(a.os * (col[jj] - cu) + ou)];
                                const float2 tu2 = make_float2(tu, tu);
                                const float2 A0 = __fmul2_rn(tu2, make_float2(wv.x, wv.y));
                                if constexpr (CPLX) {
                                    const float2 A1 = __fmul2_rn(tu2, make_float2(wv.z, wv.w));
#pragma unroll
                                    for (int d = 0; d < SUP; ++d) {
                                        const float2 t2 = make_float2(tv[d], tv[d]);
                                        acc[jj][d].a = __ffma2_rn(A0, t2, acc[jj][d].a);
                                        if (NP > 1) acc[jj][d].b = __ffma2_rn(A1, t2, acc[jj][d].b);
                                    }
                                } else {
#pragma unroll
                                    for (int d = 0; d < SUP; ++d)
                                        acc[jj][d].a = __ffma2_rn(A0, make_float2(tv[d], tv[d]), acc[jj][d].a);
                                }
                            }
                        }
                    }
                    __syncwarp();
                }
                // A slow track keeps adding to the same cells chunk after chunk;
                // an FP32 running sum of hundreds of like-sized terms drifts (its
                // rounding errors stop cancelling), so register sums are bounded
                // to two chunks (64 steps) and the long sums run in the tile.
                if (j & 1) {
#pragma unroll
                    for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                        for (int d = 0; d < SUP; ++d) { flush_cell(jj, d); zero_cell(jj, d); }
                }
            }
#pragma unroll
            for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                for (int d = 0; d < SUP; ++d) flush_cell(jj, d);
            if (zero_left) zero_left = zero_next<NP, (CPLX || FFTL) ? 8 : 4, FFTL>(zr);
            __syncthreads();   // every warp's cells are in the tile
        }

        // ---------------- write the tile ----------------
        const bool busy = e0 < e1;
        if (!(split && !busy)) {
            for (int e = tid; e < NP * TU * TV; e += blockDim.x) {
                const int p = e / (TU * TV);
                const int r = (e / TV) % TU;
                const int cl = e % TV;
                const int u = u0 + r, v = v0 + cl;
                float2 val = make_float2(0.f, 0.f);
                if (busy) {
                    if constexpr (CPLX) {
                        float2 *q = reinterpret_cast<float2 *>(acc_s) + e;
                        val = *q;
                        *q = make_float2(0.f, 0.f);
                    } else {
                        val.x = acc_s[e];
                        acc_s[e] = 0.f;
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
        if (zero_left) zero_left = zero_next<NP, (CPLX || FFTL) ? 8 : 4, FFTL>(zr);
        __syncthreads();
    }
    if (lane == 0) {
        while (zero_left) zero_left = zero_next<NP, (CPLX || FFTL) ? 8 : 4, FFTL>(zr);
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");   // the zero rows are written
    }
}

size_t tile_smem_bytes(int np, bool cplx, int tab_bytes, int os) {
    size_t acc = (size_t)np * TU * TV * (cplx ? 8 : 4);
    size_t tab = (size_t)((tab_bytes + 3) / 4) * 4;
    size_t rec = (size_t)NW * NG * ROUND * (32 + 4 + 4);       // taps, cell, info
    size_t raw = (size_t)NW * 2 * NG * ROUND * (16 + 8);       // packed steps, two rounds
    size_t gin = (size_t)NW * NG * 16;
    size_t misc = 8 + 8;
    (void)os;
    return acc + tab + rec + gin + raw + misc + 16 + ZBUF;
}

template <int NP, bool CPLX, bool FFTL>
int launch_tiles(const TileArgs &ta, int64_t n_bound, cudaStream_t s) {
    size_t smem = tile_smem_bytes(NP, CPLX, ta.tab_bytes, ta.os);
    auto kern = k_tiles<NP, CPLX, FFTL>;
    NGG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    NGG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NW * 32, smem));
    if (per_sm < 1) return fail(NGG_ERR_UNSUPPORTED, "k_tiles does not fit on an SM");
    if (n_bound > 0) {
        k_zero_split<CPLX, FFTL><<<(unsigned)n_bound, 256, 0, s>>>(ta.bin_start, ta.bbox, ta.n_img,
                                                                    (int64_t)ta.ntu * ta.ntv, ta.ntv, n_bound,
                                                                    ta.grid, ta.P, ta.p0, NP, ta.nu, ta.nv);
        NGG_CHECK_LAUNCH("k_zero_split");
    }
    const int grid = num_sms() * per_sm;
    kern<<<grid, NW * 32, smem, s>>>(ta);
    NGG_CHECK_LAUNCH("k_tiles");
    return NGG_OK;
}

template <int NP>
int dispatch_tiles(const TileArgs &ta, int64_t n_bound, bool cplx, bool fftl, cudaStream_t s) {
    if (cplx) return fftl ? launch_tiles<NP, true, true>(ta, n_bound, s) : launch_tiles<NP, true, false>(ta, n_bound, s);
    return fftl ? launch_tiles<NP, false, true>(ta, n_bound, s) : launch_tiles<NP, false, false>(ta, n_bound, s);
}

__global__ void k_cell_indices(int64_t n_rows, int64_t C, const double *uvw, const double *freq, int64_t nu, int64_t nv,
                               double dl0, double dl1, int os, int mirror, int32_t *idx, unsigned long long *nfb) {
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
    if (!cell_pair(x.hi, x.lo, a.hi, a.lo, mirror != 0, (int)(nu / 2), os, cu, ou)) {
        long long i64, o64;
        cell_fp64(u, su, mirror != 0, (int)(nu / 2), os, i64, o64);
        cu = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
        ou = (int)max(min(o64, (long long)1 << 30), -((long long)1 << 30));
        ++fb;
    }
    if (!cell_pair(y.hi, y.lo, b.hi, b.lo, mirror != 0, (int)(nv / 2), os, cv, ov)) {
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

int grid_ps_impl(const NggGridArgs *a, int64_t c_off, int64_t c_stride, void *stream);
}  // namespace

extern "C" int ngg_grid_ps(const NggGridArgs *a, void *stream) {
    clear_error();
    if (!a) return fail(NGG_ERR_INVALID, "args is NULL");
    return grid_ps_impl(a, 0, a->n_chan, stream);
}

extern "C" int ngg_grid_ps_chunk(const NggGridArgs *a, int64_t chan_offset, int64_t n_chan_total, void *stream) {
    clear_error();
    if (!a) return fail(NGG_ERR_INVALID, "args is NULL");
    if (chan_offset < 0 || a->n_chan < 0 || n_chan_total < chan_offset + a->n_chan)
        return fail(NGG_ERR_INVALID, "channel range outside the input arrays");
    return grid_ps_impl(a, chan_offset, n_chan_total, stream);
}

namespace {
int grid_ps_impl(const NggGridArgs *a, int64_t c_off, int64_t c_stride, void *stream) {
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
            int end_bit = 32;
            while (end_bit < 64 && ((unsigned long long)n_bins >> (end_bit - 32)) > 0) ++end_bit;
            size_t sort_bytes = 0;
            NGG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, keys, keys_sorted, n_keys, 0, end_bit, s));
            void *stmp = nullptr;
            if ((rc = sc.get(&stmp, sort_bytes)) != NGG_OK) return rc;
            NGG_CUDA(cub::DeviceRadixSort::SortKeys(stmp, sort_bytes, keys, keys_sorted, n_keys, 0, end_bit, s));
        }
    }
    k_bounds<<<(unsigned)((n_bins + 1 + 255) / 256), 256, 0, s>>>(keys_sorted, n_keys, n_bins, bin_start);
    NGG_CHECK_LAUNCH("k_bounds");

    int *counter = nullptr;
    if ((rc = sc.get((void **)&counter, sizeof(int) * 128)) != NGG_OK) return rc;
    NGG_CUDA(cudaMemsetAsync(counter, 0, sizeof(int) * 128, s));
    int *bbox_d = nullptr;
    if ((rc = sc.get((void **)&bbox_d, sizeof(int) * 4)) != NGG_OK) return rc;
    k_bbox_init<<<1, 1, 0, s>>>(bbox_d);
    k_bbox<<<(unsigned)((n_bins + 255) / 256), 256, 0, s>>>(bin_start, n_bins, (int64_t)ntu * ntv, ntv, bbox_d);
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
    k_nsub<<<(unsigned)((n_bound + 1 + 255) / 256), 256, 0, s>>>(bin_start, bbox_d, n_img, (int64_t)ntu * ntv, ntv,
                                                                n_bound, nsub);
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
            const dim3 pg((unsigned)B, (unsigned)nk, (unsigned)((C + 31) / 32)), pb(32, 8);
            if (np == 2) {
                if (cplx) k_pack<2, true><<<pg, pb, 0, s>>>(pa); else k_pack<2, false><<<pg, pb, 0, s>>>(pa);
            } else {
                if (cplx) k_pack<1, true><<<pg, pb, 0, s>>>(pa); else k_pack<1, false><<<pg, pb, 0, s>>>(pa);
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
        if (launch >= 63) return fail(NGG_ERR_UNSUPPORTED, "too many polarizations");
    }
    prof_record(2, s);
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
                                                               os, mirror, idx, (unsigned long long *)n_fallback);
    NGG_CHECK_LAUNCH("k_cell_indices");
    return NGG_OK;
}
