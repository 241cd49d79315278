"""GPU imaging pipeline shared by the public API functions.

Channel chunking replaces the reference's dask graph: channels are gridded in
chunks sized to a device-memory budget (cube mode: image channels are
independent), each chunk gridded straight into FFT-ordered planes, inverse
transformed and cropped/corrected on the device; only the image returns to
the host.
"""
import numpy as np

from ... import _lib
from ._gridding_convolutional_kernels import _create_prolate_spheroidal_kernel, \
    _create_prolate_spheroidal_kernel_1D
from ._remove_padding import _remove_padding

OVERSAMPLING = 100   # make_image.py:106-107 / make_psf.py hard-code these
SUPPORT = 7
GRID_BUDGET_BYTES = 16 << 30


def _arr(x):
    return x.data if hasattr(x, 'dims') and hasattr(x, 'data') else x


def _slice_chan(a, c0, c1):
    if hasattr(a, 'detach'):
        return a[:, :, c0:c1].contiguous()
    return np.ascontiguousarray(np.asarray(a)[:, :, c0:c1])


def chan_chunks(n_chan, n_pol, npad, chan_mode, budget=GRID_BUDGET_BYTES):
    if chan_mode == 'continuum' or n_chan == 0:
        return [(0, n_chan)]
    per = int(n_pol) * int(npad[0]) * int(npad[1]) * 8
    k = max(1, int(budget // max(per, 1)))
    return [(c0, min(n_chan, c0 + k)) for c0 in range(0, n_chan, k)]


AUTO_FFT64_CELLS = 1 << 26


def fft_precision(grid_parms, n_img, n_pol, npad):
    """The inverse transform's precision: grid_parms['fft_precision'], with
    'auto' (the default) resolved to 'double' while the cube's padded planes
    hold at most AUTO_FFT64_CELLS cells (the FP64 transform then costs a few
    ms and removes the FP32 transform's error in the image corners, where
    the correction image is small) and to 'single' above."""
    p = grid_parms.get('fft_precision', 'auto')
    if p == 'auto':
        return 'double' if n_img * n_pol * int(npad[0]) * int(npad[1]) <= AUTO_FFT64_CELLS else 'single'
    return p


def image_cube(vis, uvw, imaging_weight, freq, grid_parms, do_psf, normalize=True):
    """Dirty image or PSF (N0, N1, C_img, P) float64 and sum_weight (C_img, P).

    normalize=False leaves out the division by sum_weight (the image is
    Re(FFT^-1 grid) * Nu*Nv / correction): partial images of disjoint row
    sets then add up to the image of their union times its sum_weight."""
    import torch
    npad = np.asarray(grid_parms['image_size_padded'])
    image_size = np.asarray(grid_parms['image_size'])
    cell = np.asarray(grid_parms['cell_size'], dtype=np.float64)
    chan_mode = grid_parms.get('chan_mode', 'cube')
    _, corr = _create_prolate_spheroidal_kernel(OVERSAMPLING, SUPPORT, npad)
    corr = np.ascontiguousarray(_remove_padding(corr, image_size))
    cgk = _create_prolate_spheroidal_kernel_1D(OVERSAMPLING, SUPPORT)
    w = _arr(imaging_weight)
    T, B, C, P = w.shape
    freq = np.asarray(freq, dtype=np.float64)
    uvw_d = _lib._dev(_arr(uvw), torch.float64, 'uvw')
    cgk_d = _lib._dev(cgk, torch.float64, 'cgk_1D')
    corr_d = _lib._dev(corr, torch.float64, 'correction')
    n_img = 1 if chan_mode == 'continuum' else C
    precision = fft_precision(grid_parms, n_img, P, npad)
    image = np.empty((int(image_size[0]), int(image_size[1]), n_img, P), dtype=np.float64)
    sum_weight = np.empty((n_img, P), dtype=np.float64)
    for c0, c1 in chan_chunks(C, P, npad, chan_mode):
        wv = _slice_chan(w, c0, c1) if (c0, c1) != (0, C) else w
        vv = None
        if not do_psf:
            v = _arr(vis)
            vv = _slice_chan(v, c0, c1) if (c0, c1) != (0, C) else v
        g, sw = _lib.grid_ps(vv, uvw_d, wv, freq[c0:c1], cgk_d, npad, cell, mode='psf' if do_psf else 'data',
                             chan_mode=chan_mode, layout='fft', support=SUPPORT, oversampling=OVERSAMPLING)
        img = _lib.fft_correct(g, sw if normalize else torch.ones_like(sw), corr_d, image_size, precision=precision)
        del g
        if chan_mode == 'continuum':
            image[:, :, 0:1] = img.cpu().numpy()
            sum_weight[0:1] = sw.cpu().numpy()
        else:
            image[:, :, c0:c1] = img.cpu().numpy()
            sum_weight[c0:c1] = sw.cpu().numpy()
    return image, sum_weight


def imaging_weights(uvw, weight, freq, grid_parms, imaging_weights_parms, density_reduce=None):
    """Uniform/Briggs imaging weights (T,B,C,P) float32 on the GPU (torch tensor).

    density_reduce(density, sum_weight) -> (density, sum_weight), when given,
    replaces the local weight-density grid and its sum before the Briggs
    factors are taken (the sum over row shards in continuum mode)."""
    import torch
    cell = np.asarray(grid_parms['cell_size'], dtype=np.float64)
    image_size = np.asarray(grid_parms['image_size'])
    chan_mode = grid_parms.get('chan_mode', 'cube')
    uvw_d = _lib._dev(_arr(uvw), torch.float64, 'uvw')
    w_d = _lib._dev(_arr(weight), torch.float32, 'weight')
    f_d = _lib._dev(np.asarray(freq, dtype=np.float64), torch.float64, 'freq')
    dens, dsw = _lib.grid_density(uvw_d, w_d, f_d, image_size, cell, chan_mode)
    if density_reduce is not None:
        dens, dsw = density_reduce(dens, dsw)
    fac = _lib.briggs_factors(dens, dsw, imaging_weights_parms['weighting'], imaging_weights_parms.get('robust', 0.5),
                              imaging_weights_parms.get('briggs_abs_noise', 1.0))
    return _lib.weight_lookup(uvw_d, w_d, f_d, dens, fac, cell, chan_mode)
