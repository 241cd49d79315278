// Degridder: the exact adjoint of the standard gridder (DATA mode).
//
// ngg_grid_ps maps weighted visibilities to the grid,
//     grid[cell] += conv_u(iu) * conv_v(iv) * weight * vis,
// over the 7x7 footprint whose cells and oversampling offsets follow the
// reference's rounding (_standard_grid.py:299-359). Its adjoint (complex
// inner product) reads the same footprint back:
//     vis = weight * sum_{iv,iu} conv_u(iu) * conv_v(iv) * grid[cell].
// The reference has no visibility degridder (_standard_grid.py:429-430).
// One thread per (time, baseline, channel) row, channels fastest so weight
// and visibility accesses are coalesced; the 7 rows of a footprint are 7
// contiguous 56-byte runs of the grid.
#include <mutex>
#include <string>

#include "ngg_internal.cuh"

namespace ngg {
namespace {

constexpr int SUP = 7, SC = 3;

struct DChan {
    double su, sv;
    float suh, sul, svh, svl;
};

__global__ void k_dchan(const double *freq, int C, double dl0, double dl1, int64_t nu, int64_t nv, DChan *out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    double su, sv;
    uv_scale_dev(freq[c], dl0, dl1, nu, nv, su, sv);
    Split a = split_double(su), b = split_double(sv);
    out[c] = DChan{su, sv, a.hi, a.lo, b.hi, b.lo};
}

__global__ void k_dsplit(const double *uvw, int64_t T, int64_t B, float4 *uvs) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= T * B) return;
    Split a = split_double(uvw[id * 3 + 0]), c = split_double(uvw[id * 3 + 1]);
    uvs[id] = make_float4(a.hi, a.lo, c.hi, c.lo);  // time-major, as uvw
}

// NORM: prediction (ngg_predict_ps) divides each visibility by its kernel
// sum (sum_iu conv_u)(sum_iv conv_v), so a flat grid predicts itself.
template <bool FFTL, bool NORM>
__global__ void __launch_bounds__(256, 2) k_degrid(const float2 *grid, const double *uvw, const float4 *uvs,
                                                const float *weight, const DChan *chan, const double *cgk,
                                                int tab_len, int os, int64_t T, int64_t B, int64_t C, int64_t P,
                                                int64_t nu, int64_t nv, int continuum, float2 *vis) {
    __shared__ float tab[4096];
    for (int i = threadIdx.x; i < tab_len; i += blockDim.x) tab[i] = (float)cgk[i];
    __syncthreads();
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= T * B * C) return;
    // consecutive threads follow one (channel, baseline) track in time: their
    // 7x7 footprints overlap (a track moves less than a cell per step), so
    // most grid reads hit L1 instead of gathering from 32 different planes
    const int64_t c = id / (B * T);
    const int64_t rem = id - c * (B * T);
    const int64_t b = rem / T, t = rem - (rem / T) * T;
    const int64_t row = t * B + b;
    const int64_t base = (row * C + c) * P;
    const int64_t cimg = continuum ? 0 : c;
    const DChan cp = chan[c];
    const float4 us = uvs[row];
    const int cu_c = (int)(nu / 2), cv_c = (int)(nv / 2);
    bool ok = !isnan(us.x) && !isnan(us.z);
    int cu = 0, cv = 0, ou = 0, ov = 0;
    if (ok) {
        if (!cell_pair(us.x, us.y, cp.suh, cp.sul, false, cu_c, os, cu, ou)) {
            long long i64, o64;
            cell_fp64(uvw[row * 3 + 0], cp.su, false, cu_c, os, i64, o64);
            cu = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
            ou = (int)o64;
        }
        if (!cell_pair(us.z, us.w, cp.svh, cp.svl, false, cv_c, os, cv, ov)) {
            long long i64, o64;
            cell_fp64(uvw[row * 3 + 1], cp.sv, false, cv_c, os, i64, o64);
            cv = (int)max(min(i64, (long long)1 << 30), -((long long)1 << 30));
            ov = (int)o64;
        }
        ok = cu - SC >= 0 && cu + SC < nu && cv - SC >= 0 && cv + SC < nv;
    }
    if (!ok) {
        for (int64_t p = 0; p < P; ++p) vis[base + p] = make_float2(0.f, 0.f);
        return;
    }
    float tu[SUP], tv[SUP];
    float su = 0.f, sv = 0.f;
#pragma unroll
    for (int d = 0; d < SUP; ++d) {
        tu[d] = tab[abs(os * (d - SC) + ou)];
        tv[d] = tab[abs(os * (d - SC) + ov)];
        su += tu[d];
        sv += tv[d];
    }
    const float scale = NORM ? 1.0f / (su * sv) : 1.0f;
    const int64_t plane = nu * nv;
    for (int64_t p = 0; p < P; ++p) {
        const float w = weight ? weight[base + p] : 1.0f;
        if (isnan(w)) {
            vis[base + p] = make_float2(0.f, 0.f);
            continue;
        }
        const float2 *g = grid + (cimg * P + p) * plane;
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int iu = 0; iu < SUP; ++iu) {
            int u = cu + iu - SC;
            if (FFTL) u = u < cu_c ? u + (int)(nu - cu_c) : u - cu_c;
            float2 racc = make_float2(0.f, 0.f);
#pragma unroll
            for (int iv = 0; iv < SUP; ++iv) {
                int v = cv + iv - SC;
                if (FFTL) v = v < cv_c ? v + (int)(nv - cv_c) : v - cv_c;
                const float2 x = __ldg(g + (int64_t)u * nv + v);
                racc.x = fmaf(tv[iv], x.x, racc.x);
                racc.y = fmaf(tv[iv], x.y, racc.y);
            }
            acc.x = fmaf(tu[iu], racc.x, acc.x);
            acc.y = fmaf(tu[iu], racc.y, acc.y);
        }
        vis[base + p] = make_float2(acc.x * (w * scale), acc.y * (w * scale));
    }
}

template <bool FFTL, bool NORM>
void launch_degrid_t(const NggDegridArgs *a, const float4 *uvs, const DChan *chan, int tab_len, int cont,
                     cudaStream_t s) {
    const int64_t n = a->n_time * a->n_baseline * a->n_chan;
    k_degrid<FFTL, NORM><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        (const float2 *)a->grid, a->uvw, uvs, a->weight, chan, a->cgk_1D, tab_len, a->oversampling, a->n_time,
        a->n_baseline, a->n_chan, a->n_pol, a->n_u, a->n_v, cont, (float2 *)a->vis);
}

void launch_degrid(const NggDegridArgs *a, const float4 *uvs, const DChan *chan, int tab_len, int cont,
                   bool normalize, cudaStream_t s) {
    const bool fftl = a->layout == NGG_LAYOUT_FFT;
    if (fftl && normalize) launch_degrid_t<true, true>(a, uvs, chan, tab_len, cont, s);
    else if (fftl) launch_degrid_t<true, false>(a, uvs, chan, tab_len, cont, s);
    else if (normalize) launch_degrid_t<false, true>(a, uvs, chan, tab_len, cont, s);
    else launch_degrid_t<false, false>(a, uvs, chan, tab_len, cont, s);
}

}  // namespace
}  // namespace ngg

using namespace ngg;

namespace {
// Body of ngg_degrid_ps and ngg_predict_ps (normalize: divide by the kernel sum).
int degrid_alloc(const NggDegridArgs *a, void *stream, bool normalize) {
    clear_error();
    if (!a) return fail(NGG_ERR_INVALID, "args is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    if (a->chan_mode != NGG_CHAN_CUBE && a->chan_mode != NGG_CHAN_CONTINUUM) return fail(NGG_ERR_INVALID, "chan_mode");
    if (a->layout != NGG_LAYOUT_NATURAL && a->layout != NGG_LAYOUT_FFT) return fail(NGG_ERR_INVALID, "layout");
    if (a->support != SUP) return fail(NGG_ERR_UNSUPPORTED, "support must be 7");
    if (a->oversampling < 1 || a->oversampling > 1000) return fail(NGG_ERR_UNSUPPORTED, "oversampling out of [1,1000]");
    const int64_t T = a->n_time, B = a->n_baseline, C = a->n_chan, P = a->n_pol;
    if (T < 0 || B < 0 || C < 0 || P < 1 || a->n_u < 1 || a->n_v < 1 || a->n_u > 65535 || a->n_v > 65535)
        return fail(NGG_ERR_INVALID, "dims");
    if (T * B * C == 0) return NGG_OK;
    if (!a->grid || !a->uvw || !a->freq || !a->cgk_1D || !a->vis) return fail(NGG_ERR_INVALID, "NULL pointer");
    const int tab_len = a->oversampling * (a->support / 2 + 1);
    if (tab_len > 4096) return fail(NGG_ERR_UNSUPPORTED, "kernel table too long");
    DChan *chan = nullptr;
    float4 *uvs = nullptr;
    int rc = scratch_alloc((void **)&chan, sizeof(DChan) * C, s);
    if (rc != NGG_OK) return rc;
    rc = scratch_alloc((void **)&uvs, sizeof(float4) * T * B, s);
    if (rc != NGG_OK) { scratch_free(chan, s); return rc; }
    k_dchan<<<(unsigned)((C + 127) / 128), 128, 0, s>>>(a->freq, (int)C, a->delta_lm[0], a->delta_lm[1], a->n_u, a->n_v, chan);
    k_dsplit<<<(unsigned)((T * B + 255) / 256), 256, 0, s>>>(a->uvw, T, B, uvs);
    const int cont = a->chan_mode == NGG_CHAN_CONTINUUM;
    launch_degrid(a, uvs, chan, tab_len, cont, normalize, s);
    cudaError_t e = cudaGetLastError();
    scratch_free(uvs, s);
    scratch_free(chan, s);
    if (e != cudaSuccess) return cuda_fail(e, "k_degrid");
    return NGG_OK;
}
}  // namespace

extern "C" int ngg_degrid_ps(const NggDegridArgs *a, void *stream) { return degrid_alloc(a, stream, false); }

extern "C" int ngg_predict_ps(const NggDegridArgs *a, void *stream) { return degrid_alloc(a, stream, true); }

// ---------------------------------------------------------------------------
// Degridding without any device allocation.
//
// Some programs embed this library inside a host application that owns all
// device memory: the application sizes its pools up front and forbids
// allocations it did not make (they could exceed the budget it enforces or
// fail mid-run, where it cannot recover). ngg_degrid_ps allocates two small
// scratch arrays per call; this variant keeps them instead in one fixed
// device array that is part of the library image. The array exists on every
// GPU that loads the library, for the life of the process.
//
// Limits: n_time*n_baseline <= NGG_NOALLOC_MAX_ROWS uvw rows and
// n_chan <= NGG_NOALLOC_MAX_CHAN channels (16.5 MiB in total).
// All calls share the array. Every byte a call reads from it is written by
// that same call first, so nothing has to start at zero, but two calls whose
// work overlaps on the GPU (different streams, or devices sharing a context)
// overwrite each other's scratch and give wrong results.
// ---------------------------------------------------------------------------
namespace ngg {
namespace {
constexpr int64_t kNoAllocRows = NGG_NOALLOC_MAX_ROWS;
constexpr int64_t kNoAllocChan = NGG_NOALLOC_MAX_CHAN;
constexpr size_t kNoAllocBytes = sizeof(float4) * kNoAllocRows + sizeof(DChan) * kNoAllocChan;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
struct NoAllocSlot {
    unsigned long long ctx_id;   // context the address belongs to (0: none cached)
    void *ptr;
};
NoAllocSlot g_noalloc_slot[64] = {};

// The driver's context calls, reached through the runtime so that the library
// does not link libcuda (it must load on machines without a GPU driver).
typedef int (*CtxGetCurrentFn)(void **ctx);
typedef int (*CtxGetIdFn)(void *ctx, unsigned long long *id);

// Unique id of the context current on this thread (0 if none, or if the
// driver does not offer context ids: then the address is looked up per call).
unsigned long long current_ctx_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of g_noalloc_scratch in the current device's context. The
// host-side symbol is not a device address; the address is looked up with
// cudaGetSymbolAddress once per (device, context) and looked up again when
// the context changes (after cudaDeviceReset the old address is invalid).
int noalloc_scratch(void **out) {
    int dev = 0;
    NGG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(NGG_ERR_UNSUPPORTED, "device index >= 64");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocSlot &sl = g_noalloc_slot[dev];
    const unsigned long long id = current_ctx_id();
    if (id == 0 || sl.ctx_id != id || !sl.ptr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);   // makes the context current if needed
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        sl.ptr = p;
        sl.ctx_id = current_ctx_id();
    }
    *out = sl.ptr;
    return NGG_OK;
}
}  // namespace
}  // namespace ngg

extern "C" int ngg_degrid_ps_noalloc(const NggDegridArgs *a, void *stream) {
    clear_error();
    if (!a) return fail(NGG_ERR_INVALID, "args is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    if (a->chan_mode != NGG_CHAN_CUBE && a->chan_mode != NGG_CHAN_CONTINUUM) return fail(NGG_ERR_INVALID, "chan_mode");
    if (a->layout != NGG_LAYOUT_NATURAL && a->layout != NGG_LAYOUT_FFT) return fail(NGG_ERR_INVALID, "layout");
    if (a->support != SUP) return fail(NGG_ERR_UNSUPPORTED, "support must be 7");
    if (a->oversampling < 1 || a->oversampling > 1000) return fail(NGG_ERR_UNSUPPORTED, "oversampling out of [1,1000]");
    const int64_t T = a->n_time, B = a->n_baseline, C = a->n_chan, P = a->n_pol;
    if (T < 0 || B < 0 || C < 0 || P < 1 || a->n_u < 1 || a->n_v < 1 || a->n_u > 65535 || a->n_v > 65535)
        return fail(NGG_ERR_INVALID, "dims");
    if (T * B > kNoAllocRows)
        return fail(NGG_ERR_INVALID, "ngg_degrid_ps_noalloc: n_time*n_baseline = " + std::to_string(T * B) +
                                         " exceeds the fixed scratch limit of " + std::to_string(kNoAllocRows) +
                                         " uvw rows (use ngg_degrid_ps)");
    if (C > kNoAllocChan)
        return fail(NGG_ERR_INVALID, "ngg_degrid_ps_noalloc: n_chan = " + std::to_string(C) +
                                         " exceeds the fixed scratch limit of " + std::to_string(kNoAllocChan) +
                                         " channels (use ngg_degrid_ps)");
    if (T * B * C == 0) return NGG_OK;
    if (!a->grid || !a->uvw || !a->freq || !a->cgk_1D || !a->vis) return fail(NGG_ERR_INVALID, "NULL pointer");
    const int tab_len = a->oversampling * (a->support / 2 + 1);
    if (tab_len > 4096) return fail(NGG_ERR_UNSUPPORTED, "kernel table too long");
    void *base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc != NGG_OK) return rc;
    float4 *uvs = reinterpret_cast<float4 *>(base);
    DChan *chan = reinterpret_cast<DChan *>(reinterpret_cast<unsigned char *>(base) + sizeof(float4) * kNoAllocRows);
    k_dchan<<<(unsigned)((C + 127) / 128), 128, 0, s>>>(a->freq, (int)C, a->delta_lm[0], a->delta_lm[1], a->n_u, a->n_v, chan);
    k_dsplit<<<(unsigned)((T * B + 255) / 256), 256, 0, s>>>(a->uvw, T, B, uvs);
    const int cont = a->chan_mode == NGG_CHAN_CONTINUUM;
    launch_degrid(a, uvs, chan, tab_len, cont, false, s);
    NGG_CHECK_LAUNCH("k_degrid (noalloc)");
    return NGG_OK;
}
