"""Learned gridding convolution function for mosaic imaging.

A coordinate MLP stands in for the oversampled CONV_KERNEL table that
make_gridding_convolution_function builds (make_gridding_convolution_function.py:
164-311): input (x, y, f) -- the table offset from its centre along u and v
(oversampled units) and the frequency, scaled to about [-1, 1] -- Fourier
features of (x, y, r = |(x, y)|, f), four SiLU layers of width 64, one linear
output (the reference's CONV_KERNEL is real: the real part of the pattern's
FFT, :273). The phase gradient of each pointing is an exact plane wave and is
applied in closed form by the gridder, as on the table path, so the network
only has to represent the aperture kernel and its frequency dependence.

Training data are the GCFs the method itself generates (ngg_gcf_kernels at
n_freq frequencies spanning the band, cropped and normalised as
make_gridding_convolution_function does), every table point of the gridder's
footprint. The network is trained in FP32 on the GPU by libngg's own forward,
backward and Adam kernels (ngg_mlp_train) and evaluated in BF16 on the
tcgen05 tensor cores to synthesise one table per channel at that channel's
exact frequency (ngg_grid_gcf_learned). The table path (ngg_grid_gcf) stays
the fallback and the yardstick for the learned path's image error.
"""
import time

import numpy as np

from .. import _lib
from .make_gridding_convolution_function import gcf_tables

SPATIAL_SIGMA = (3.0, 3.0, 6.0)   # Fourier-feature scales for (x, y, r)
FREQ_ROWS = (0.1, 0.2)            # frequency-only features: cycles per unit of scaled frequency
WIDTH = 64


def init_params(seed, spatial_sigma=SPATIAL_SIGMA, freq_rows=FREQ_ROWS):
    """Initial parameter vector (layout of ngg.h): He-normal dense layers,
    zero biases, and a structured Fourier matrix B (32 x 4): the first rows
    Gaussian in (x, y, r) with no frequency term, the last len(freq_rows)
    rows pure frequency features. Mixing frequency into the spatial features
    makes every spatial feature's phase frequency-dependent, which the
    network then has to undo; separate rows keep the kernel's slow frequency
    dependence a smooth modulation."""
    rng = np.random.default_rng(seed)
    parts = []
    for _ in range(4):
        parts.append(rng.standard_normal((WIDTH, WIDTH)) * np.sqrt(2.0 / WIDTH))
        parts.append(np.zeros(WIDTH))
    parts.append(rng.standard_normal(WIDTH) * np.sqrt(1.0 / WIDTH))
    parts.append(np.zeros(1))
    B = np.zeros((32, 4))
    ns = 32 - len(freq_rows)
    B[:ns, :3] = rng.standard_normal((ns, 3)) * np.asarray(spatial_sigma, dtype=np.float64)[None, :]
    B[ns:, 3] = freq_rows
    parts.append(B)
    p = np.concatenate([q.ravel() for q in parts]).astype(np.float32)
    assert p.size == _lib.MLP_NPARAM
    return p


class LearnedGCF:
    """A trained network and what the gridder needs with it."""

    def __init__(self, params, scale, train_freq, train_support, oversampling, max_support, info=None):
        self.params = params                       # CUDA float32 (NGG_MLP_NPARAM)
        self.scale = dict(scale)                   # NggMlpScale fields
        self.train_freq = np.asarray(train_freq, dtype=np.float64)
        self.train_support = np.asarray(train_support, dtype=np.int32)   # (n_freq, 2)
        self.oversampling = np.asarray(oversampling).astype(int)
        self.max_support = np.asarray(max_support).astype(int)
        self.info = dict(info or {})

    @property
    def conv_size(self):
        return (self.max_support + 1) * self.oversampling

    # ---- training -------------------------------------------------------
    @staticmethod
    def training_set(function, dish, blockage, freqs, grid_parms, oversampling, max_support, support_cut_level=0.025):
        """(z, target, scale, support, tables): every table point of the
        gridder's footprint at each frequency, as CUDA float32 arrays."""
        import torch
        os_ = np.asarray(oversampling).astype(int)
        ck, _, sup = gcf_tables(function, [dish], [blockage], np.array([[0, 0]]), freqs, grid_parms, os_,
                                max_support, support_cut_level)
        S = int(sup.max()) | 1
        w = (os_ * (S // 2) + os_ // 2).astype(int)          # largest |x|, |y| the gridder reads
        R = np.asarray(ck.shape[-2:])
        c = R // 2
        sub = ck[0, :, 0, c[0] - w[0]:c[0] + w[0] + 1, c[1] - w[1]:c[1] + w[1] + 1]   # (n_f, 2w+1, 2w+1)
        out_scale = float(sub.abs().max())
        f = np.asarray(freqs, dtype=np.float64)
        f0 = 0.5 * (f.max() + f.min())
        fs = 2.0 / (f.max() - f.min()) if f.max() > f.min() else 1.0
        scale = {'x_scale': 1.0 / w[0], 'y_scale': 1.0 / w[1], 'f_center': f0, 'f_scale': fs, 'out_scale': out_scale}
        xs = torch.arange(-int(w[0]), int(w[0]) + 1, device='cuda', dtype=torch.float64) * scale['x_scale']
        ys = torch.arange(-int(w[1]), int(w[1]) + 1, device='cuda', dtype=torch.float64) * scale['y_scale']
        fz = torch.as_tensor((f - f0) * fs, device='cuda', dtype=torch.float64)
        F, X, Y = torch.meshgrid(fz, xs, ys, indexing='ij')
        z = torch.stack([X, Y, F], dim=-1).reshape(-1, 3).float().contiguous()
        t = (sub / out_scale).reshape(-1).float().contiguous()
        return z, t, scale, sup[0, :, 0], ck

    @classmethod
    def fit(cls, function, dish, blockage, freq_band, grid_parms, oversampling, max_support, support_cut_level=0.025,
            n_freq=32, steps=8000, batch=65536, lr=(3e-3, 1e-5), seed=0, chunk=2000):
        """Generate the training set on the GPU and train the network there."""
        import torch
        t0 = time.perf_counter()
        freqs = np.linspace(freq_band[0], freq_band[1], n_freq)
        z, t, scale, sup, _ = cls.training_set(function, dish, blockage, freqs, grid_parms, oversampling,
                                               max_support, support_cut_level)
        torch.cuda.synchronize()
        t_data = time.perf_counter() - t0
        params = torch.as_tensor(init_params(seed), device='cuda')
        m = torch.zeros(_lib.MLP_NTRAINED, dtype=torch.float32, device='cuda')
        v = torch.zeros_like(m)
        hist = []
        t1 = time.perf_counter()
        done = 0
        while done < steps:
            k = min(chunk, steps - done)
            # one cosine schedule over all steps, applied piecewise per call
            fa, fb = done / max(steps - 1, 1), (done + k - 1) / max(steps - 1, 1)
            lra = lr[1] + 0.5 * (lr[0] - lr[1]) * (1 + np.cos(np.pi * fa))
            lrb = lr[1] + 0.5 * (lr[0] - lr[1]) * (1 + np.cos(np.pi * fb))
            hist.append(_lib.mlp_train(params, m, v, z, t, k, step0=done, batch=batch, lr0=lra, lr1=lrb,
                                       seed=seed + 17).cpu().numpy())
            done += k
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t1
        hist = np.concatenate(hist) if hist else np.zeros(0)
        info = {'n_samples': int(z.shape[0]), 'n_freq': n_freq, 'steps': steps, 'batch': batch,
                'data_s': t_data, 'train_s': t_train, 'final_loss': float(hist[-100:].mean()) if len(hist) else None,
                'loss_history': hist}
        return cls(params, scale, freqs, sup, oversampling, max_support, info)

    # ---- evaluation -------------------------------------------------------
    def support_for(self, freq):
        """Per-channel support: that of the nearest training frequency."""
        f = freq.detach().cpu().numpy() if hasattr(freq, 'detach') else np.asarray(freq)
        f = f.astype(np.float64).ravel()
        idx = np.abs(f[:, None] - self.train_freq[None, :]).argmin(axis=1)
        return np.ascontiguousarray(self.train_support[idx]).astype(np.int32)

    def table(self, freq, tensor_cores=True):
        """The network's table at one frequency over the trained footprint,
        (2w+1, 2w+1) float64 numpy, in table units (times out_scale)."""
        import torch
        w0, w1 = int(round(1 / self.scale['x_scale'])), int(round(1 / self.scale['y_scale']))
        xs = torch.arange(-w0, w0 + 1, device='cuda', dtype=torch.float64) * self.scale['x_scale']
        ys = torch.arange(-w1, w1 + 1, device='cuda', dtype=torch.float64) * self.scale['y_scale']
        X, Y = torch.meshgrid(xs, ys, indexing='ij')
        fz = torch.full_like(X, (float(freq) - self.scale['f_center']) * self.scale['f_scale'])
        z = torch.stack([X, Y, fz], dim=-1).reshape(-1, 3).float().contiguous()
        y = _lib.mlp_forward(self.params, z, tensor_cores=tensor_cores)
        return (y.double() * self.scale['out_scale']).reshape(X.shape).cpu().numpy()

    def grid(self, vis, uvw, weight, freq, field_index, phase_slope, n_uv, delta_lm, mode='data', chan_mode='cube',
             layout='natural'):
        """Mosaic gridding with the synthesised per-channel tables."""
        return _lib.grid_gcf_learned(vis, uvw, weight, freq, field_index, self.support_for(freq), phase_slope,
                                     self.params, self.scale, self.conv_size, n_uv, delta_lm, self.oversampling,
                                     mode=mode, chan_mode=chan_mode, layout=layout)
