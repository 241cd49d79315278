// Learned-GCF network on the tcgen05 tensor cores: the four 64x64 layers of a
// 128-sample tile run as tcgen05.mma (kind::f16, BF16 A and B from shared
// memory, FP32 accumulator in tensor memory), issued by one thread and
// completed through an mbarrier; the tile's 4 warps read their 32
// accumulator rows back with tcgen05.ld, add the bias, apply SiLU in FP32 and
// write the next layer's operand. Fourier features and the output layer are
// FP32 on the CUDA cores.
//
// A CTA holds one copy of the weights and NG = 4 tile groups of 4 warps, each
// with its own activation buffer, 64 TMEM columns, mbarrier and named
// barrier: while one group's MMAs run on the tensor pipe the other groups do
// their SiLU / feature work, so the tensor pipe and the CUDA cores overlap
// (the CUDA-core work per tile is far larger than the MMAs').
//
// Split BF16: every operand is stored as hi = bf16(v) and lo = bf16(v - hi),
// and each K-step issues hi*hi + lo*hi + hi*lo into the FP32 accumulator
// (the lo*lo term, ~2^-16 relative, is dropped). Products of BF16 values are
// exact in FP32, so a layer is computed to about FP32 accuracy on the BF16
// tensor cores; single-BF16 operands gave 2-3x the network's own fit error.
//
// Operand layout (no swizzle, K-major): an 8-row x 16-byte core matrix holds
// 8 rows x 8 BF16 of K; core matrix (row group g, K group j) sits at
// g*1024 + j*128 bytes, so the descriptor's leading-dimension offset (next
// core matrix along K) is 128 B and its stride offset (next 8-row group) is
// 1024 B; one MMA consumes K = 16 (two core matrices), the next starts 256 B
// further.
#include <cuda_bf16.h>

#include "ngg_internal.cuh"
#include "mlp.cuh"

namespace ngg {
namespace {

constexpr int NGRP = 4;                      // tile groups per CTA
constexpr int TC_THREADS = 128 * NGRP;
constexpr int SMEM_A1 = 2 * 128 * 64 * 2;    // one group's activations, hi and lo: 32 KB
constexpr int SMEM_A = NGRP * SMEM_A1;
constexpr int SMEM_B = 2 * 4 * 64 * 64 * 2;  // hi, lo of W1..W4: 64 KB
constexpr int SMEM_F = (4 * 64 + 64 + 8) * 4;
constexpr int SMEM_TOTAL = SMEM_A + SMEM_B + SMEM_F + 128;
constexpr uint32_t TMEM_COLS = 64 * NGRP;
// instruction descriptor, kind::f16: D F32 (bit 4), A BF16 (bits 7-9), B BF16
// (bits 10-12), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
constexpr int WAIT_LIMIT = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version for tcgen05
    return d;                 // base offset 0, no swizzle
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(IDESC), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// bounded wait for phase `parity` of the barrier; false on timeout
__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (int it = 0; it < WAIT_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred P1;\nmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
            "selp.b32 %0, 1, 0, P1;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

#define NGG_TMEM_LD16(taddr, r)                                                                                   \
    asm volatile(                                                                                                 \
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n" \
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),          \
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])      \
        : "r"(taddr)                                                                                              \
        : "memory")

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ float bf16_lo(float v) { return v - __bfloat162float(__float2bfloat16_rn(v)); }

// 8 consecutive K values of one row (hi and lo parts) into K-major operand tiles
__device__ __forceinline__ void store8(uint8_t *hi, uint8_t *lo, int off, const float *v) {
    uint4 q, r;
    q.x = pack_bf16(v[0], v[1]);
    q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]);
    q.w = pack_bf16(v[6], v[7]);
    r.x = pack_bf16(bf16_lo(v[0]), bf16_lo(v[1]));
    r.y = pack_bf16(bf16_lo(v[2]), bf16_lo(v[3]));
    r.z = pack_bf16(bf16_lo(v[4]), bf16_lo(v[5]));
    r.w = pack_bf16(bf16_lo(v[6]), bf16_lo(v[7]));
    *reinterpret_cast<uint4 *>(hi + off) = q;
    *reinterpret_cast<uint4 *>(lo + off) = r;
}

// row `row` (64 values) into the hi / lo K-major operand tiles
__device__ __forceinline__ void store_row(uint8_t *hi, uint8_t *lo, int row, const float *v) {
#pragma unroll
    for (int j = 0; j < 8; ++j) store8(hi, lo, (row >> 3) * 1024 + j * 128 + (row & 7) * 16, v + 8 * j);
}

// SiLU with the fast exponential and division (each within a few ulps; the
// split-BF16 operands carry ~2^-16 relative error): the argument of the
// exponential is capped so 1 + e stays below 2^126, where __fdividef is exact
__device__ __forceinline__ float silu_f(float a) { return __fdividef(a, 1.0f + __expf(fminf(-a, 80.0f))); }

// (sin, cos)(2 pi d): reduced to t = d - rint(d) in [-1/2, 1/2] first (exact),
// so the hardware sine and cosine see arguments in [-pi, pi], where their
// absolute error is ~2^-21
__device__ __forceinline__ void sincos_turns(float d, float *sv, float *cv) {
    const float t = d - rintf(d);
    __sincosf(6.283185307179586f * t, sv, cv);
}

// samples from an array: z[s] -> y[s]
struct GenArray {
    const float *z;
    float *y;
    __device__ bool point(int64_t s, float &x, float &yv, float &f) const {
        x = z[s * 3];
        yv = z[s * 3 + 1];
        f = z[s * 3 + 2];
        return true;
    }
    __device__ void store(int64_t s, float v) const { y[s] = v; }
};

// samples of the reorganised GCF table of the mosaic gridder: for every
// channel c, offset class (oui, ovi) and tap (dv, du) of the S x S footprint,
// value = net(x * xs, y * ys, (f_c - f0) * fs) * out_scale with
// x = os0*(du - S/2) + oui - os0/2, y likewise; stored at tap rows dv and
// dv + S (the doubled run), column du; zero outside the channel's support.
struct GenTable {
    const double *freq;
    const int32_t *support;   // (C, 2)
    float *ckt;
    int os0, os1, S;
    double xs, ys, f0, fs, out_scale;
    __device__ void decode(int64_t s, int &c, int &oui, int &ovi, int &dv, int &du) const {
        du = (int)(s % S);
        int64_t r = s / S;
        dv = (int)(r % S);
        r /= S;
        const int no = (os0 + 1) * (os1 + 1);
        const int o = (int)(r % no);
        c = (int)(r / no);
        oui = o / (os1 + 1);
        ovi = o % (os1 + 1);
    }
    __device__ bool point(int64_t s, float &x, float &y, float &f) const {
        int c, oui, ovi, dv, du;
        decode(s, c, oui, ovi, dv, du);
        const int sc = S / 2;
        x = (float)((double)(os0 * (du - sc) + oui - os0 / 2) * xs);
        y = (float)((double)(os1 * (dv - sc) + ovi - os1 / 2) * ys);
        f = (float)((freq[c] - f0) * fs);
        return true;
    }
    __device__ void store(int64_t s, float v) const {
        int c, oui, ovi, dv, du;
        decode(s, c, oui, ovi, dv, du);
        const int sc = S / 2;
        const int su = support[c * 2], sv = support[c * 2 + 1];
        const int iu = du - sc, iv = dv - sc;
        const bool in = iu >= -(su / 2) && iu < su - su / 2 && iv >= -(sv / 2) && iv < sv - sv / 2;
        const float val = in ? (float)((double)v * out_scale) : 0.f;
        float *blk = ckt + (((int64_t)c * (os0 + 1) + oui) * (os1 + 1) + ovi) * (2 * S) * SP_TABLE;
        blk[dv * SP_TABLE + du] = val;
        blk[(dv + S) * SP_TABLE + du] = val;
    }
};

__device__ __forceinline__ void group_sync(int grp) {
    asm volatile("bar.sync %0, 128;" ::"r"(grp + 1) : "memory");
}

template <class Gen>
__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_tc(const float *params, Gen gen, int64_t n, int *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int grp = tid >> 7, gt = tid & 127;       // tile group, thread within the group
    uint8_t *sA = smem + grp * SMEM_A1, *sAl = sA + SMEM_A1 / 2;   // this group's activations hi / lo
    uint8_t *sB = smem + SMEM_A, *sBl = smem + SMEM_A + SMEM_B / 2;  // weights hi / lo
    float *sb = reinterpret_cast<float *>(smem + SMEM_A + SMEM_B);  // b1..b4 [4][64], Wo [64], bo
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + SMEM_A + SMEM_B + SMEM_F);   // [NGRP]
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(bars + NGRP);
    int *s_fail = reinterpret_cast<int *>(bars + NGRP + 1);                             // [NGRP]
    uint64_t *bar = bars + grp;

    // weights as B operands (N = output, K = input), biases, output layer
    for (int e = tid; e < 4 * 64 * 8; e += TC_THREADS) {
        const int k = e / 512, o = (e / 8) % 64, j = e % 8;
        float w[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) w[q] = params[k * MLP_LAYER + o * 64 + j * 8 + q];
        store8(sB + k * 8192, sBl + k * 8192, (o >> 3) * 1024 + j * 128 + (o & 7) * 16, w);
    }
    for (int e = tid; e < 4 * 64; e += TC_THREADS) sb[e] = params[(e / 64) * MLP_LAYER + 4096 + e % 64];
    for (int e = tid; e < 65; e += TC_THREADS) sb[256 + e] = params[MLP_OFF_WO + e];
    if (tid < NGRP) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bars + tid)) : "memory");
        s_fail[tid] = 0;
    }
    if (tid == 0) asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tbase = *s_tmem;
    const uint32_t tcol = tbase + (uint32_t)(64 * grp);                 // this group's accumulator
    const uint32_t trow = tcol + ((uint32_t)((warp & 3) * 32) << 16);   // this warp's 32 lanes
    const float *Bf = params + MLP_OFF_B;
    uint32_t parity = 0;
    bool failed = false;

    for (int64_t tile = (int64_t)blockIdx.x * NGRP + grp; tile * 128 < n && !failed;
         tile += (int64_t)gridDim.x * NGRP) {
        const int64_t s = tile * 128 + gt;
        float h[64];
        {
            float x = 0.f, y = 0.f, f = 0.f;
            if (s < n) gen.point(s, x, y, f);
            const float r = sqrtf(x * x + y * y);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const float d = Bf[j * 4] * x + Bf[j * 4 + 1] * y + Bf[j * 4 + 2] * r + Bf[j * 4 + 3] * f;
                sincos_turns(d, &h[j], &h[32 + j]);
            }
            store_row(sA, sAl, gt, h);
        }
        fence_async_smem();
        fence_before();
        group_sync(grp);
        fence_after();
        for (int layer = 0; layer < 4; ++layer) {
            if (gt == 0) {
                const uint32_t a0 = smem_u32(sA), a1 = smem_u32(sAl);
                const uint32_t b0 = smem_u32(sB + layer * 8192), b1 = smem_u32(sBl + layer * 8192);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const uint64_t ah = sdesc(a0 + kk * 256, 128, 1024), al = sdesc(a1 + kk * 256, 128, 1024);
                    const uint64_t bh = sdesc(b0 + kk * 256, 128, 1024), bl = sdesc(b1 + kk * 256, 128, 1024);
                    mma_bf16(tcol, ah, bh, kk > 0 ? 1u : 0u);
                    mma_bf16(tcol, al, bh, 1u);
                    mma_bf16(tcol, ah, bl, 1u);
                }
                commit(bar);
            }
            if (!bar_wait(bar, parity)) {
                s_fail[grp] = 1;
                atomicExch(err, 1);
            }
            parity ^= 1u;
            fence_after();
            uint32_t acc[64];
            NGG_TMEM_LD16(trow + 0, (&acc[0]));
            NGG_TMEM_LD16(trow + 16, (&acc[16]));
            NGG_TMEM_LD16(trow + 32, (&acc[32]));
            NGG_TMEM_LD16(trow + 48, (&acc[48]));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 64; ++j) h[j] = silu_f(__uint_as_float(acc[j]) + sb[layer * 64 + j]);
            if (layer < 3) {
                store_row(sA, sAl, gt, h);
                fence_async_smem();
            }
            fence_before();
            group_sync(grp);
            fence_after();
            if (s_fail[grp]) {
                failed = true;
                break;
            }
        }
        if (failed) break;
        float out = sb[256 + 64];
#pragma unroll
        for (int j = 0; j < 64; ++j) out = fmaf(sb[256 + j], h[j], out);
        if (s < n) gen.store(s, out);
    }
    if (failed && gt == 0) bar_wait(bar, parity ^ 1u);   // the timed-out MMAs' phase, another bounded wait
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TMEM_COLS) : "memory");
}

template <class Gen>
int launch_tc(const float *params, const Gen &gen, int64_t n, cudaStream_t s) {
    static bool attr_set[64] = {};
    int dev = 0;
    NGG_CUDA(cudaGetDevice(&dev));
    if (dev < 64 && !attr_set[dev]) {
        NGG_CUDA(cudaFuncSetAttribute(k_mlp_tc<Gen>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_TOTAL));
        attr_set[dev] = true;
    }
    ScratchList sc(s);
    int *err = nullptr;
    int rc;
    if ((rc = sc.get((void **)&err, sizeof(int))) != NGG_OK) return rc;
    NGG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    const int64_t tiles = (n + 127) / 128;
    const int64_t groups = (tiles + NGRP - 1) / NGRP;   // one CTA (NGRP tile groups) per SM
    const int64_t grid = groups < (int64_t)num_sms() ? groups : (int64_t)num_sms();
    k_mlp_tc<Gen><<<(unsigned)grid, TC_THREADS, SMEM_TOTAL, s>>>(params, gen, n, err);
    NGG_CHECK_LAUNCH("k_mlp_tc");
    int herr = 0;
    NGG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    NGG_CUDA(cudaStreamSynchronize(s));
    if (herr) return fail(NGG_ERR_TIMEOUT, "k_mlp_tc: tensor-core barrier wait timed out");
    return NGG_OK;
}

}  // namespace

int mlp_synth_table(const float *params, const NggMlpScale *scale, const double *freq, int64_t C, int os0, int os1,
                    int S, const int32_t *support, float *ckt, cudaStream_t s) {
    GenTable g;
    g.freq = freq;
    g.support = support;
    g.ckt = ckt;
    g.os0 = os0;
    g.os1 = os1;
    g.S = S;
    g.xs = scale->x_scale;
    g.ys = scale->y_scale;
    g.f0 = scale->f_center;
    g.fs = scale->f_scale;
    g.out_scale = scale->out_scale;
    const int64_t n = C * (int64_t)(os0 + 1) * (os1 + 1) * S * S;
    NGG_CUDA(cudaMemsetAsync(ckt, 0, sizeof(float) * C * (os0 + 1) * (os1 + 1) * 2 * S * SP_TABLE, s));
    if (n == 0) return NGG_OK;
    return launch_tc(params, g, n, s);
}

}  // namespace ngg

using namespace ngg;

extern "C" int ngg_mlp_forward_tc(const float *params, const float *z, int64_t n, float *y, void *stream) {
    clear_error();
    if (!params || n < 0 || (n > 0 && (!z || !y))) return fail(NGG_ERR_INVALID, "ngg_mlp_forward_tc arguments");
    if (n == 0) return NGG_OK;
    GenArray g;
    g.z = z;
    g.y = y;
    return launch_tc(params, g, n, (cudaStream_t)stream);
}
