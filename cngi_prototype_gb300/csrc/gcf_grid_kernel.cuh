// k_grid_gcf<DATA, S>: mosaic gridding with the reorganised GCF table (see
// gcf.cu). Included by gcf_grid_lo.cu, gcf_grid_mid.cu and gcf_grid_hi.cu,
// which instantiate it for the odd supports 1-15, 17-23 and 25-31.
//
// One warp per (channel, baseline, 128-step chunk, pol). Lanes decode one
// visibility each, 32 at a time; then the warp walks them in track order.
// Lane l < S owns the grid columns = l (mod S) (Romein) and keeps the S rows
// of its current column in registers, row class i in acc[i]. Per
// visibility a lane adds S taps: tab[...][S - m + i][col] * W, one coalesced
// load and two FMAs each (the table row run is stored twice so the rotation
// by m = (cv - S/2) mod S is a base offset; W carries the visibility's part of
// the phase gradient). A cell leaves the registers when the track moves:
//  * one row (cv +-1): the leaving row class is warp-uniform -> a switch;
//  * one column (cu +-1): the leaving lane is warp-uniform -> its registers
//    are transposed across the warp with shuffles and flushed in parallel;
//  * larger jumps and field changes flush all registers.
// A flushed cell is rotated by its position's phase (Gx[u] Gy[v]) and added
// to the grid with one 64-bit float2 atomic. Full flushes go through a
// per-warp shared-memory stage so the kernel holds only three copies of that
// epilogue (instruction-cache footprint).
#pragma once
#include "gcf_grid.cuh"

namespace ngg {
namespace {

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulcf(float2 a, float2 b) {   // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ int pmod(int x, int m) {
    int r = x % m;
    return r < 0 ? r + m : r;
}

template <bool DATA, int S>
__global__ void __launch_bounds__(128, 4) k_grid_gcf(const GArgs a) {
    constexpr int sc = S / 2;
    // per warp: S x 32 staging cells for flushes, 32 for the column transpose
    __shared__ float2 s_stage[4][S * 32];
    __shared__ float2 s_trans[4][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t item = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    if (item >= a.C * a.B * a.nk * a.P) return;
    const int p = (int)(item % a.P);
    const int64_t k = (item / a.P) % a.nk;
    const int64_t b = (item / (a.P * a.nk)) % a.B;
    const int64_t c = item / (a.P * a.nk * a.B);
    const int64_t cimg = a.continuum ? 0 : c;
    const int cfb = a.cfb_map[b], cfc = a.cfc_map[c], cfp = a.cfp_map[p];
    if (cfb < 0 || cfb >= a.ncfb || cfc < 0 || cfc >= a.ncfc || cfp < 0 || cfp >= a.ncfp) return;
    const int64_t cf = ((int64_t)cfb * a.ncfc + cfc) * a.ncfp + cfp;
    const GChan cp = a.chan[c];
    const int cu_c = (int)(a.nu / 2), cv_c = (int)(a.nv / 2);
    float2 *plane = a.grid + (cimg * a.P + p) * a.nu * a.nv;
    const float *tab = a.ckt + cf * (int64_t)(a.os0 + 1) * (a.os1 + 1) * (2 * S) * SP;
    const bool active = lane < S;
    const int fftl = a.fftl;
    float2 *stage = s_stage[wib];
    float2 *trans = s_trans[wib];

    float2 acc[S];
#pragma unroll
    for (int i = 0; i < S; ++i) acc[i] = make_float2(0.f, 0.f);
    int prev_cu = -(1 << 28), prev_cv = -(1 << 28), cur_f = 0;
    int mycol = -(1 << 28);
    double swl = 0.0;

    // add cell (u, v) of field cur_f; skips empty cells and cells off the grid
    auto emit = [&](float2 x, int u, int v) {
        if ((x.x == 0.f && x.y == 0.f) || u < 0 || u >= a.nu || v < 0 || v >= a.nv) return;
        x = cmulf(cmulf(x, a.gx[(int64_t)cur_f * a.nu + u]), a.gy[(int64_t)cur_f * a.nv + v]);
        if (fftl) {
            u = u < cu_c ? u + ((int)a.nu - cu_c) : u - cu_c;
            v = v < cv_c ? v + ((int)a.nv - cv_c) : v - cv_c;
        }
        atomicAdd(plane + (int64_t)u * a.nv + v, x);
    };
    // register i holds row cv - sc + ((i - (cv - sc)) mod S)
    auto row_of = [&](int i, int cv) { return cv - sc + pmod(i - (cv - sc), S); };
    // this lane's column, all rows: registers -> own staging slots -> one rolled
    // emit loop (no cross-lane traffic, so no warp barrier; callable divergently)
    auto flush_mine = [&]() {
#pragma unroll
        for (int i = 0; i < S; ++i) {
            stage[i * 32 + lane] = acc[i];
            acc[i] = make_float2(0.f, 0.f);
        }
#pragma unroll 1
        for (int i = 0; i < S; ++i) emit(stage[i * 32 + lane], mycol, row_of(i, prev_cv));
    };

    for (int r0 = 0; r0 < GCH; r0 += 32) {
        // ---- producer: one visibility per lane ----
        const int64_t t = k * GCH + r0 + lane;
        unsigned cuv = 0, oo = 0;
        int fidx = 0;
        float2 W = make_float2(0.f, 0.f);
        if (t < a.T) {
            const int64_t row = t * a.B + b;
            fidx = a.field_index[row];
            const float4 us = a.uvs[row];
            if (fidx >= 0 && fidx < a.nf && !isnan(us.x) && !isnan(us.z)) {
                int cu, ou, cv, ov;
                if (!cell_pair(us.x, us.y, cp.suh, cp.sul, false, cu_c, a.os0, cu, ou)) {
                    long long i64, o64;
                    cell_fp64(a.uvw[row * 3 + 0], cp.su, false, cu_c, a.os0, i64, o64);
                    cu = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
                    ou = (int)o64;
                }
                if (!cell_pair(us.z, us.w, cp.svh, cp.svl, false, cv_c, a.os1, cv, ov)) {
                    long long i64, o64;
                    cell_fp64(a.uvw[row * 3 + 1], cp.sv, false, cv_c, a.os1, i64, o64);
                    cv = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
                    ov = (int)o64;
                }
                if (cu + a.maxsup < a.nu && cv + a.maxsup < a.nv && cu - a.maxsup >= 0 && cv - a.maxsup >= 0) {
                    const int64_t base = (row * a.C + c) * a.P + p;
                    const float w = a.weight[base];
                    float2 wd;
                    bool ok;
                    if (DATA) {
                        const float2 v = a.vis[base];
                        wd = make_float2(v.x * w, v.y * w);
                        ok = !isnan(wd.x) && !isnan(wd.y) && (wd.x != 0.f || wd.y != 0.f);
                    } else {
                        wd = make_float2(w, 0.f);
                        ok = !isnan(w) && w != 0.f;
                    }
                    const int oui = ou + a.os0 / 2, ovi = ov + a.os1 / 2;
                    ok = ok && oui >= 0 && oui <= a.os0 && ovi >= 0 && ovi <= a.os1;
                    if (ok) {
                        cuv = ((unsigned)cu << 16) | (unsigned)cv;
                        oo = 1u | ((unsigned)oui << 1) | ((unsigned)ovi << 12);
                        const float2 h = cmulf(a.hx[(int64_t)fidx * (a.os0 + 1) + oui],
                                               a.hy[(int64_t)fidx * (a.os1 + 1) + ovi]);
                        const float2 g = cmulf(a.gx[(int64_t)fidx * a.nu + cu], a.gy[(int64_t)fidx * a.nv + cv]);
                        W = cmulcf(cmulf(wd, h), g);
                        const double2 n = a.nrm[((int64_t)fidx * a.ncf + cf) * (a.os0 + 1) * (a.os1 + 1) +
                                                (int64_t)oui * (a.os1 + 1) + ovi];
                        swl += DATA ? (double)w * (n.x * n.x - n.y * n.y) : (double)w * n.x;
                    }
                }
            }
        }

        // ---- consumer: the warp walks the 32 visibilities (all lanes, uniform control) ----
        for (int s = 0; s < 32; ++s) {
            const unsigned oos = __shfl_sync(0xffffffffu, oo, s);
            if (!(oos & 1u)) continue;
            const unsigned cuvs = __shfl_sync(0xffffffffu, cuv, s);
            const int fs = __shfl_sync(0xffffffffu, fidx, s);
            const float wx = __shfl_sync(0xffffffffu, W.x, s);
            const float wy = __shfl_sync(0xffffffffu, W.y, s);
            const int cu = (int)(cuvs >> 16), cv = (int)(cuvs & 0xffffu);
            const int oui = (int)((oos >> 1) & 2047u), ovi = (int)((oos >> 12) & 2047u);
            const int dcu = cu - prev_cu, dcv = cv - prev_cv;
            const bool small_move = dcu >= -1 && dcu <= 1 && dcv >= -1 && dcv <= 1;
            if (fs != cur_f || !small_move) {
                // field change (cells carry their field's rotation) or a jump: flush all
                if (active) {
                    flush_mine();
                    mycol = cu - sc + pmod(lane - (cu - sc), S);
                }
                cur_f = fs;
            } else {
                if (dcu != 0) {
                    // one column leaves: lane src (uniform) takes the new one; its
                    // registers are spread over the warp and flushed in parallel
                    const int oldcol = dcu > 0 ? prev_cu - sc : prev_cu + sc;
                    const int src = pmod(oldcol, S);
                    if (lane == src) {
#pragma unroll
                        for (int i = 0; i < S; ++i) {
                            trans[i] = acc[i];
                            acc[i] = make_float2(0.f, 0.f);
                        }
                        mycol = dcu > 0 ? prev_cu + sc + 1 : prev_cu - sc - 1;
                    }
                    __syncwarp();
                    if (active) emit(trans[lane], oldcol, row_of(lane, prev_cv));
                    __syncwarp();
                }
                if (dcv != 0) {
                    // one row leaves: its register class (uniform) is flushed by every lane
                    const int ro = dcv > 0 ? prev_cv - sc : prev_cv + sc;
                    float2 x = make_float2(0.f, 0.f);
                    switch (pmod(ro, S)) {
#define NGG_ROW_CASE(I)                               \
    case I:                                           \
        if (I < S) {                                  \
            x = acc[I < S ? I : 0];                   \
            acc[I < S ? I : 0] = make_float2(0.f, 0.f); \
        }                                             \
        break;
                        NGG_ROW_CASE(0) NGG_ROW_CASE(1) NGG_ROW_CASE(2) NGG_ROW_CASE(3) NGG_ROW_CASE(4)
                        NGG_ROW_CASE(5) NGG_ROW_CASE(6) NGG_ROW_CASE(7) NGG_ROW_CASE(8) NGG_ROW_CASE(9)
                        NGG_ROW_CASE(10) NGG_ROW_CASE(11) NGG_ROW_CASE(12) NGG_ROW_CASE(13) NGG_ROW_CASE(14)
                        NGG_ROW_CASE(15) NGG_ROW_CASE(16) NGG_ROW_CASE(17) NGG_ROW_CASE(18) NGG_ROW_CASE(19)
                        NGG_ROW_CASE(20) NGG_ROW_CASE(21) NGG_ROW_CASE(22) NGG_ROW_CASE(23) NGG_ROW_CASE(24)
                        NGG_ROW_CASE(25) NGG_ROW_CASE(26) NGG_ROW_CASE(27) NGG_ROW_CASE(28) NGG_ROW_CASE(29)
                        NGG_ROW_CASE(30)
#undef NGG_ROW_CASE
                        default: break;
                    }
                    if (active) emit(x, mycol, ro);
                }
            }
            prev_cu = cu;
            prev_cv = cv;
            if (active) {
                const int m = pmod(cv - sc, S);
                // register i takes tap row (i - m) mod S: row S - m + i of the doubled run
                const float *q = tab + ((int64_t)oui * (a.os1 + 1) + ovi) * (2 * S) * SP + (S - m) * SP +
                                 (mycol - cu + sc);
                const float2 w2 = make_float2(wx, wy);
#pragma unroll
                for (int i = 0; i < S; ++i) {
                    const float kk = __ldg(q + i * SP);
                    acc[i] = __ffma2_rn(make_float2(kk, kk), w2, acc[i]);   // (re, im) in one paired FMA
                }
            }
        }
    }
    if (active) flush_mine();
    for (int o = 16; o > 0; o >>= 1) swl += __shfl_xor_sync(0xffffffffu, swl, o);
    if (lane == 0 && swl != 0.0) atomicAdd(a.sum_weight + cimg * a.P + p, swl);
}

template <int S>
void launch_one(const GArgs &a, bool data, unsigned blocks, cudaStream_t s) {
    if (data) k_grid_gcf<true, S><<<blocks, 128, 0, s>>>(a);
    else k_grid_gcf<false, S><<<blocks, 128, 0, s>>>(a);
}

}  // namespace
}  // namespace ngg
