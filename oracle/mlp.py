"""numpy restatement of the learned-GCF coordinate MLP (test infrastructure).

The reference has no learned component; this is the CPU oracle for the
network the library trains and evaluates on the GPU, used to check its
forward pass, its hand-written backward pass (gradients) and its Adam step.

Network (parameter layout of the flat float32 vector, in order):
  W1[64][64] b1[64]  W2[64][64] b2[64]  W3[64][64] b3[64]  W4[64][64] b4[64]
  Wo[64] bo[1]  B[32][4]   (B: Fourier-feature matrix, fixed, not trained)
Input z = (x, y, f) already scaled to about [-1, 1]; c = (x, y, r, f) with
r = sqrt(x^2 + y^2); features phi = [sin(2 pi B c), cos(2 pi B c)] (64);
h_k = silu(W_k h_{k-1} + b_k), k = 1..4, h_0 = phi; output y = Wo . h4 + bo.
Loss = mean((y - t)^2).
"""
import numpy as np

WIDTH = 64
NFREQ = 32
SIZES = [(64, 64), (64,), (64, 64), (64,), (64, 64), (64,), (64, 64), (64,), (64,), (1,), (32, 4)]
NPARAM = int(sum(np.prod(s) for s in SIZES))
N_TRAINED = NPARAM - 32 * 4


def unpack(params):
    out, o = [], 0
    for s in SIZES:
        n = int(np.prod(s))
        out.append(params[o:o + n].reshape(s))
        o += n
    return out


def init_params(seed, feature_sigma=(6.0, 6.0, 12.0, 1.0)):
    """He-style init for the dense layers, Gaussian Fourier matrix with a
    per-coordinate scale for (x, y, r, f)."""
    rng = np.random.default_rng(seed)
    parts = []
    for s in SIZES[:8]:
        if len(s) == 2:
            parts.append(rng.standard_normal(s) * np.sqrt(2.0 / s[1]))
        else:
            parts.append(np.zeros(s))
    parts.append(rng.standard_normal(64) * np.sqrt(1.0 / 64))
    parts.append(np.zeros(1))
    parts.append(rng.standard_normal((32, 4)) * np.asarray(feature_sigma)[None, :])
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


def silu(a):
    return a / (1.0 + np.exp(-a))


def silu_grad(a):
    s = 1.0 / (1.0 + np.exp(-a))
    return s * (1.0 + a * (1.0 - s))


def features(z, B):
    x, y, f = z[:, 0], z[:, 1], z[:, 2]
    c = np.stack([x, y, np.sqrt(x * x + y * y), f], axis=1)
    p = 2 * np.pi * (c @ B.T)
    return np.concatenate([np.sin(p), np.cos(p)], axis=1)


def forward(params, z, dtype=np.float64):
    """Returns (y, cache). Computed in `dtype`."""
    P = [np.asarray(p, dtype=dtype) for p in unpack(np.asarray(params, dtype=np.float64))]
    W = [P[0], P[2], P[4], P[6]]
    b = [P[1], P[3], P[5], P[7]]
    Wo, bo, B = P[8], P[9], P[10]
    h = features(np.asarray(z, dtype=dtype), B).astype(dtype)
    hs, As = [h], []
    for k in range(4):
        a = h @ W[k].T + b[k]
        h = silu(a)
        As.append(a)
        hs.append(h)
    y = h @ Wo + bo[0]
    return y, (hs, As, W, Wo)


def loss_grad(params, z, t, dtype=np.float64):
    """mean squared error and its gradient w.r.t. the flat parameter vector
    (zero for the fixed Fourier matrix)."""
    y, (hs, As, W, Wo) = forward(params, z, dtype)
    n = len(t)
    r = y - np.asarray(t, dtype=dtype)
    loss = float(np.mean(r * r))
    dy = 2.0 * r / n
    g_Wo = hs[4].T @ dy
    g_bo = np.array([dy.sum()])
    dh = np.outer(dy, Wo)
    gW, gb = [None] * 4, [None] * 4
    for k in range(3, -1, -1):
        da = dh * silu_grad(As[k])
        gW[k] = da.T @ hs[k]
        gb[k] = da.sum(axis=0)
        dh = da @ W[k]
    parts = [gW[0], gb[0], gW[1], gb[1], gW[2], gb[2], gW[3], gb[3], g_Wo, g_bo, np.zeros((32, 4))]
    return loss, np.concatenate([p.ravel() for p in parts])


def adam(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (bias-corrected), trained parameters only."""
    p = params.astype(np.float64).copy()
    g = grad.astype(np.float64)
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    p[:N_TRAINED] -= (lr * mh / (np.sqrt(vh) + eps))[:N_TRAINED]
    return p, m, v
