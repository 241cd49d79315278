// Learned GCF: a coordinate MLP (Fourier features of (x, y, r, f), 4 hidden
// SiLU layers of width 64, scalar output) trained on GCF tables in FP32 with
// these hand-written forward / backward / Adam kernels. The reference has no
// learned component; the tables it learns are the CONV_KERNEL values of
// make_gridding_convolution_function (make_gridding_convolution_function.py:
// 164-311), which the network replaces in ngg_grid_gcf_learned.
//
// Layout of the flat float32 parameter vector (NGG_MLP_NPARAM values):
//   W1[64][64] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64][64] b4[64]
//   Wo[64] bo[1] B[32][4]   (B: Fourier-feature matrix, fixed)
// Activations of a batch live in scratch as [sample][64] float32.
#include <vector>

#include "ngg_internal.cuh"
#include "mlp.cuh"

namespace ngg {
namespace {

constexpr int TS = 64;   // samples per dense-layer tile

// features phi[s] = [sin(2 pi B c), cos(2 pi B c)], c = (x, y, r, f)
__global__ void k_features(const float *params, const float *z, int64_t n, float *phi) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n * 32) return;
    const int64_t s = id / 32;
    const int j = (int)(id % 32);
    const float *B = params + MLP_OFF_B + j * 4;
    const float x = z[s * 3], y = z[s * 3 + 1], f = z[s * 3 + 2];
    const float r = sqrtf(x * x + y * y);
    const float d = B[0] * x + B[1] * y + B[2] * r + B[3] * f;
    float sv, cv;
    sincospif(2.0f * d, &sv, &cv);
    phi[s * 64 + j] = sv;
    phi[s * 64 + 32 + j] = cv;
}

__device__ __forceinline__ float silu(float a) { return a / (1.0f + __expf(-a)); }
__device__ __forceinline__ float silu_grad(float a) {
    const float s = 1.0f / (1.0f + __expf(-a));
    return s * (1.0f + a * (1.0f - s));
}

// A = X W^T + b, H = silu(A). X [n][64], W [64][64]. 256 threads: thread t
// computes sample t/4, outputs 16*(t%4) .. +15.
__global__ void __launch_bounds__(256) k_dense_fwd(const float *X, const float *W, const float *b, int64_t n, float *A,
                                                   float *H) {
    __shared__ float sx[TS][65];
    __shared__ float sw[64][65];
    const int64_t s0 = (int64_t)blockIdx.x * TS;
    for (int i = threadIdx.x; i < TS * 64; i += 256) {
        const int r = i / 64, c = i % 64;
        sx[r][c] = (s0 + r < n) ? X[(s0 + r) * 64 + c] : 0.f;
        sw[r][c] = W[i];
    }
    __syncthreads();
    const int r = threadIdx.x / 4, o0 = (threadIdx.x % 4) * 16;
    float acc[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j] = b[o0 + j];
    for (int k = 0; k < 64; ++k) {
        const float xv = sx[r][k];
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[j] = fmaf(xv, sw[o0 + j][k], acc[j]);
    }
    if (s0 + r < n) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            A[(s0 + r) * 64 + o0 + j] = acc[j];
            H[(s0 + r) * 64 + o0 + j] = silu(acc[j]);
        }
    }
}

// y = Wo . H4 + bo; optional loss and dA4 = (2 (y - t) / n) Wo silu'(A4)
__global__ void k_out(const float *params, const float *H4, const float *A4, const float *t, int64_t n, float *y,
                      float *dy, float *dA4, double *loss) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (s < n) {
        const float *Wo = params + MLP_OFF_WO;
        float acc = params[MLP_OFF_BO];
        for (int k = 0; k < 64; ++k) acc = fmaf(Wo[k], H4[s * 64 + k], acc);
        if (y) y[s] = acc;
        if (t) {
            const float r = acc - t[s];
            l = (double)r * (double)r;
            const float g = 2.0f * r / (float)n;
            dy[s] = g;
            for (int k = 0; k < 64; ++k) dA4[s * 64 + k] = g * Wo[k] * silu_grad(A4[s * 64 + k]);
        }
    }
    if (loss) {
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l / (double)n);
    }
}

// dAp = (dA W) * silu'(Ap). dA [n][64], W [64][64] (out, in).
__global__ void __launch_bounds__(256) k_dense_bwd_data(const float *dA, const float *W, const float *Ap, int64_t n,
                                                        float *dAp) {
    __shared__ float sd[TS][65];
    __shared__ float sw[64][65];
    const int64_t s0 = (int64_t)blockIdx.x * TS;
    for (int i = threadIdx.x; i < TS * 64; i += 256) {
        const int r = i / 64, c = i % 64;
        sd[r][c] = (s0 + r < n) ? dA[(s0 + r) * 64 + c] : 0.f;
        sw[r][c] = W[i];
    }
    __syncthreads();
    const int r = threadIdx.x / 4, i0 = (threadIdx.x % 4) * 16;
    float acc[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j] = 0.f;
    for (int o = 0; o < 64; ++o) {
        const float dv = sd[r][o];
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[j] = fmaf(dv, sw[o][i0 + j], acc[j]);
    }
    if (s0 + r < n) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int64_t q = (s0 + r) * 64 + i0 + j;
            dAp[q] = acc[j] * silu_grad(Ap[q]);
        }
    }
}

// gW += dA^T Hp, gb += sum dA over a chunk of samples (atomics across chunks)
constexpr int WCH = 256;
__global__ void __launch_bounds__(256) k_dense_bwd_weight(const float *dA, const float *Hp, int64_t n, float *gW,
                                                          float *gb) {
    __shared__ float sd[32][65];
    __shared__ float sh[32][65];
    const int64_t s0 = (int64_t)blockIdx.x * WCH;
    const int o = threadIdx.x / 4, i0 = (threadIdx.x % 4) * 16;   // row o of W, columns i0..i0+15
    float acc[16];
    float accb = 0.f;
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j] = 0.f;
    for (int c0 = 0; c0 < WCH; c0 += 32) {
        __syncthreads();
        for (int i = threadIdx.x; i < 32 * 64; i += 256) {
            const int r = i / 64, c = i % 64;
            const int64_t s = s0 + c0 + r;
            sd[r][c] = s < n ? dA[s * 64 + c] : 0.f;
            sh[r][c] = s < n ? Hp[s * 64 + c] : 0.f;
        }
        __syncthreads();
        for (int r = 0; r < 32; ++r) {
            const float dv = sd[r][o];
            accb += (i0 == 0) ? dv : 0.f;
#pragma unroll
            for (int j = 0; j < 16; ++j) acc[j] = fmaf(dv, sh[r][i0 + j], acc[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) atomicAdd(gW + o * 64 + i0 + j, acc[j]);
    if (i0 == 0) atomicAdd(gb + o, accb);
}

// gWo += sum dy H4, gbo += sum dy
__global__ void k_out_bwd_weight(const float *dy, const float *H4, int64_t n, float *g) {
    const int k = threadIdx.x;   // 64 threads: Wo[k]; thread 0 also bo
    const int64_t s0 = (int64_t)blockIdx.x * WCH;
    float acc = 0.f, accb = 0.f;
    for (int r = 0; r < WCH; ++r) {
        const int64_t s = s0 + r;
        if (s >= n) break;
        acc = fmaf(dy[s], H4[s * 64 + k], acc);
        accb += dy[s];
    }
    atomicAdd(g + MLP_OFF_WO + k, acc);
    if (k == 0) atomicAdd(g + MLP_OFF_BO, accb);
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// random batch: sample i of step `step` is row hash(seed, step, i) mod n_all
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}
__global__ void k_gather(const float *z, const float *t, int64_t n_all, uint64_t seed, int64_t step, int64_t nb,
                         float *zb, float *tb) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const uint64_t h = mix64(seed ^ mix64((uint64_t)step * 0x9e3779b97f4a7c15ull + (uint64_t)i));
    const int64_t r = (int64_t)(h % (uint64_t)n_all);
    zb[i * 3] = z[r * 3];
    zb[i * 3 + 1] = z[r * 3 + 1];
    zb[i * 3 + 2] = z[r * 3 + 2];
    tb[i] = t[r];
}

struct Work {
    float *phi, *A[4], *H[4], *dA, *dA2, *dy;
};

int work_alloc(Work &w, int64_t n, ScratchList &sc) {
    int rc;
    if ((rc = sc.get((void **)&w.phi, sizeof(float) * n * 64)) != NGG_OK) return rc;
    for (int k = 0; k < 4; ++k) {
        if ((rc = sc.get((void **)&w.A[k], sizeof(float) * n * 64)) != NGG_OK) return rc;
        if ((rc = sc.get((void **)&w.H[k], sizeof(float) * n * 64)) != NGG_OK) return rc;
    }
    if ((rc = sc.get((void **)&w.dA, sizeof(float) * n * 64)) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&w.dA2, sizeof(float) * n * 64)) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&w.dy, sizeof(float) * (n > 0 ? n : 1))) != NGG_OK) return rc;
    return NGG_OK;
}

void forward(const float *params, const float *z, int64_t n, Work &w, cudaStream_t s) {
    k_features<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(params, z, n, w.phi);
    const unsigned nb = (unsigned)((n + TS - 1) / TS);
    const float *X = w.phi;
    for (int k = 0; k < 4; ++k) {
        k_dense_fwd<<<nb, 256, 0, s>>>(X, params + MLP_OFF_W[k], params + MLP_OFF_b[k], n, w.A[k], w.H[k]);
        X = w.H[k];
    }
}

void backward(const float *params, const float *t, int64_t n, Work &w, float *grad, double *loss, cudaStream_t s) {
    k_out<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(params, w.H[3], w.A[3], t, n, nullptr, w.dy, w.dA, loss);
    const unsigned nw = (unsigned)((n + WCH - 1) / WCH);
    k_out_bwd_weight<<<nw, 64, 0, s>>>(w.dy, w.H[3], n, grad);
    float *dA = w.dA, *dA2 = w.dA2;
    const unsigned nb = (unsigned)((n + TS - 1) / TS);
    for (int k = 3; k >= 0; --k) {
        const float *Hp = k > 0 ? w.H[k - 1] : w.phi;
        k_dense_bwd_weight<<<nw, 256, 0, s>>>(dA, Hp, n, grad + MLP_OFF_W[k], grad + MLP_OFF_b[k]);
        if (k > 0) {
            k_dense_bwd_data<<<nb, 256, 0, s>>>(dA, params + MLP_OFF_W[k], w.A[k - 1], n, dA2);
            float *tmp = dA;
            dA = dA2;
            dA2 = tmp;
        }
    }
}

}  // namespace
}  // namespace ngg

using namespace ngg;

extern "C" int ngg_mlp_forward(const float *params, const float *z, int64_t n, float *y, void *stream) {
    clear_error();
    if (!params || n < 0 || (n > 0 && (!z || !y))) return fail(NGG_ERR_INVALID, "ngg_mlp_forward arguments");
    if (n == 0) return NGG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    ScratchList sc(s);
    Work w;
    int rc;
    if ((rc = work_alloc(w, n, sc)) != NGG_OK) return rc;
    forward(params, z, n, w, s);
    k_out<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(params, w.H[3], w.A[3], nullptr, n, y, nullptr, nullptr, nullptr);
    NGG_CHECK_LAUNCH("ngg_mlp_forward");
    return NGG_OK;
}

extern "C" int ngg_mlp_loss_grad(const float *params, const float *z, const float *target, int64_t n, float *grad,
                                 double *loss, void *stream) {
    clear_error();
    if (!params || !grad || !loss || n < 1 || !z || !target) return fail(NGG_ERR_INVALID, "ngg_mlp_loss_grad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    NGG_CUDA(cudaMemsetAsync(grad, 0, sizeof(float) * NGG_MLP_NPARAM, s));
    NGG_CUDA(cudaMemsetAsync(loss, 0, sizeof(double), s));
    ScratchList sc(s);
    Work w;
    int rc;
    if ((rc = work_alloc(w, n, sc)) != NGG_OK) return rc;
    forward(params, z, n, w, s);
    backward(params, target, n, w, grad, loss, s);
    NGG_CHECK_LAUNCH("ngg_mlp_loss_grad");
    return NGG_OK;
}

extern "C" int ngg_mlp_adam(float *params, const float *grad, float *m, float *v, float lr, float beta1, float beta2,
                            float eps, int step, void *stream) {
    clear_error();
    if (!params || !grad || !m || !v || step < 1) return fail(NGG_ERR_INVALID, "ngg_mlp_adam arguments");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    const int64_t n = MLP_N_TRAINED;
    k_adam<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, n, lr, beta1, beta2, eps,
                                                                          c1, c2);
    NGG_CHECK_LAUNCH("k_adam");
    return NGG_OK;
}

extern "C" int ngg_mlp_train(float *params, float *m, float *v, const float *z, const float *target, int64_t n_samples,
                             int64_t batch, int n_steps, int step0, float lr0, float lr1, uint64_t seed,
                             double *loss_history, void *stream) {
    clear_error();
    if (!params || !m || !v || !z || !target || n_samples < 1 || batch < 1 || n_steps < 0 || step0 < 0)
        return fail(NGG_ERR_INVALID, "ngg_mlp_train arguments");
    cudaStream_t s = (cudaStream_t)stream;
    ScratchList sc(s);
    Work w;
    float *zb = nullptr, *tb = nullptr, *grad = nullptr;
    double *lossbuf = nullptr;
    int rc;
    if ((rc = work_alloc(w, batch, sc)) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&zb, sizeof(float) * batch * 3)) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&tb, sizeof(float) * batch)) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&grad, sizeof(float) * NGG_MLP_NPARAM)) != NGG_OK) return rc;
    if ((rc = sc.get((void **)&lossbuf, sizeof(double) * (n_steps > 0 ? n_steps : 1))) != NGG_OK) return rc;
    if (n_steps > 0) NGG_CUDA(cudaMemsetAsync(lossbuf, 0, sizeof(double) * n_steps, s));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < n_steps; ++it) {
        const int step = step0 + it + 1;
        // cosine decay from lr0 to lr1 over the n_steps of this call
        const float fr = n_steps > 1 ? (float)it / (float)(n_steps - 1) : 1.f;
        const float lr = lr1 + 0.5f * (lr0 - lr1) * (1.f + cosf(3.14159265f * fr));
        k_gather<<<(unsigned)((batch + 255) / 256), 256, 0, s>>>(z, target, n_samples, seed, step, batch, zb, tb);
        NGG_CUDA(cudaMemsetAsync(grad, 0, sizeof(float) * NGG_MLP_NPARAM, s));
        forward(params, zb, batch, w, s);
        backward(params, tb, batch, w, grad, lossbuf + it, s);
        const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
        k_adam<<<(unsigned)((MLP_N_TRAINED + 255) / 256), 256, 0, s>>>(params, grad, m, v, MLP_N_TRAINED, lr, b1, b2,
                                                                       eps, c1, c2);
    }
    NGG_CHECK_LAUNCH("ngg_mlp_train");
    if (loss_history && n_steps > 0)
        NGG_CUDA(cudaMemcpyAsync(loss_history, lossbuf, sizeof(double) * n_steps, cudaMemcpyDeviceToDevice, s));
    return NGG_OK;
}
