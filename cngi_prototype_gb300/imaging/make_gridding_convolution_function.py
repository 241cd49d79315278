"""make_gridding_convolution_function -- same signature and outputs as
ngcasa/imaging/make_gridding_convolution_function.py:36-313 (the a-term GCF:
Airy / CASA-Airy primary-beam products per antenna-type pair and PB
frequency, their FFTs, supports, normalisation and the per-field phase
gradient), with the patterns and FFTs computed on the GPU in FP64
(ngg_gcf_kernels) and cropped and normalised on the device.
"""
import copy

import numpy as np

from .. import _lib
from ..xds import Dataset
from ._imaging_utils._check_imaging_parms import _check_gcf_parms, _check_grid_parms
from ._imaging_utils._sel import _check_sel_parms


def create_cf_baseline_map(unique_ant_indx, basline_ant, n_unique_ant):
    """Antenna-type pairs (i <= j, row-major) and each baseline's pair index
    (make_gridding_convolution_function.py:522-539)."""
    n_pairs = int((n_unique_ant ** 2 + n_unique_ant) / 2)
    pairs = np.array([[i, j] for i in range(n_unique_ant) for j in range(i, n_unique_ant)], dtype=int)
    pairs = pairs.reshape(n_pairs, 2)
    uai = np.asarray(unique_ant_indx)
    ba = np.asarray(basline_ant)
    t0, t1 = uai[ba[:, 0]], uai[ba[:, 1]]
    cf_map = np.zeros(ba.shape[0], dtype=int)
    for k, (i, j) in enumerate(pairs):
        cf_map[(t0 == i) & (t1 == j)] = k
    return cf_map, pairs


def create_cf_chan_map(freq_chan, chan_tolerance_factor):
    """PB frequencies, one per `chan_tolerance_factor` of fractional bandwidth
    (at least one, each channel its own when there are fewer channels), and
    each channel's nearest one (make_gridding_convolution_function.py:546-575)."""
    freq_chan = np.asarray(freq_chan, dtype=np.float64)
    n_chan = len(freq_chan)
    lo, hi = np.min(freq_chan), np.max(freq_chan)
    n_pb = int(np.floor((hi - lo) / (hi * chan_tolerance_factor)) + 0.5)
    n_pb = max(n_pb, 1)
    if n_pb >= n_chan:
        return np.arange(n_chan), freq_chan
    step = (hi - lo) / n_pb
    pb_freq = np.arange(n_pb) * step + lo + step / 2
    return np.array([int(np.argmin(np.abs(pb_freq - f))) for f in freq_chan]), pb_freq


def calc_conv_size(centre_row, centre_col, amin, amax, imsize, support_cut_level, oversampling, max_support):
    """Odd support of one weight kernel (make_gridding_convolution_function.py:
    412-459): walk +x along the centre column and +y along the centre row
    until the kernel is no longer above support_cut_level * max|kernel|;
    support = (int(0.5 + walk / os) + 1) * 2 + 1; both axes take the larger.
    centre_row[i] = kernel[i, n1//2], centre_col[j] = kernel[n0//2, j]."""
    cut = support_cut_level * amax
    if not amin < cut:
        raise AssertionError('######### ERROR: support_cut_level too small or imsize too small.')
    sup = []
    for ax, line in ((0, centre_row), (1, centre_col)):
        c = imsize[ax] // 2
        i = c
        while line[i] > cut:
            i += 1
            if not i < imsize[ax]:
                raise AssertionError('######### ERROR: support_cut_level too small or imsize too small.')
        sup.append((int(0.5 + (i - c) / oversampling[ax]) + 1) * 2 + 1)
    if not (sup[0] < max_support[0] and sup[1] < max_support[1]):
        raise AssertionError('######### ERROR: support_cut_level too small or imsize too small.'
                             + f'{sup[0]},*,{max_support[0]}')
    s = max(sup)
    return [s, s]


def sin_pixel_offsets(field_phase_dir, phase_center, cell_size):
    """Field-centre offsets in pixels from the phase centre under the SIN
    (orthographic) projection of the image grid -- what make_phase_gradient
    obtains from an RA---SIN/DEC--SIN world-to-pixel transform
    (make_gridding_convolution_function.py:331-347): direction cosines
    l = cos d sin(a - a0), m = sin d cos d0 - cos d sin d0 cos(a - a0), in
    degrees, divided by the cell size in degrees."""
    a0, d0 = float(phase_center[0]), float(phase_center[1])
    f = np.asarray(field_phase_dir, dtype=np.float64).reshape(-1, 2)
    a, d = f[:, 0], f[:, 1]
    l = np.cos(d) * np.sin(a - a0)
    m = np.sin(d) * np.cos(d0) - np.cos(d) * np.sin(d0) * np.cos(a - a0)
    cdelt = np.asarray(cell_size, dtype=np.float64) * (180 / np.pi)
    return np.stack([np.rad2deg(l) / cdelt[0], np.rad2deg(m) / cdelt[1]], axis=1)


def _phase_slopes(field_phase_dir, phase_center, grid_parms, oversampling):
    pix = sin_pixel_offsets(field_phase_dir, phase_center, grid_parms['cell_size'])
    return -pix * 2 * np.pi / (np.asarray(grid_parms['image_size_padded']) * np.asarray(oversampling))


def _phase_gradient(slopes, conv_size):
    """exp(i (x px + y py)) over the table offsets from its centre, on the GPU."""
    import torch
    cs = np.asarray(conv_size)
    c = cs // 2
    x = torch.arange(-int(c[0]), int(cs[0] - c[0]), dtype=torch.float64, device='cuda')
    y = torch.arange(-int(c[1]), int(cs[1] - c[1]), dtype=torch.float64, device='cuda')
    s = torch.as_tensor(slopes, dtype=torch.float64, device='cuda')
    ph = x[None, :, None] * s[:, 0, None, None] + y[None, None, :] * s[:, 1, None, None]
    return torch.polar(torch.ones_like(ph), ph)


def gcf_tables(function, dish, blockage, pairs, pb_freq, grid_parms, oversampling, max_support, support_cut_level,
               freq_chunk=8):
    """CONV_KERNEL and WEIGHT_CONV_KERNEL (n_pair, n_freq, 1, R0, R1) float64 CUDA
    tensors and SUPPORT (n_pair, n_freq, 1, 2) (make_gridding_convolution_function.py:
    164-274 and resize_and_calc_support, :360-390): patterns and FFTs on the GPU
    (ngg_gcf_kernels) in chunks of PB frequencies; the support walk on the
    kernels' centre row and column; crop to (max_support + 1) * os and division
    by the sum over the (support + 1) * os window / (os0 * os1) on the device."""
    import torch
    os_ = np.asarray(oversampling)
    max_sup = np.asarray(max_support)
    rs = (max_sup + 1) * os_
    npad = np.asarray(grid_parms['image_size_padded'])
    cell = np.asarray(grid_parms['cell_size']) * os_
    pb_freq = np.asarray(pb_freq, dtype=np.float64)
    n_pair, n_freq = len(pairs), len(pb_freq)
    c0, c1 = int(npad[0] // 2), int(npad[1] // 2)
    st = npad // 2 - rs // 2
    support = np.zeros((n_pair, n_freq, 1, 2), dtype=int)
    ck = torch.empty((n_pair, n_freq, 1, int(rs[0]), int(rs[1])), dtype=torch.float64, device='cuda')
    wk = torch.empty_like(ck)
    for f0 in range(0, n_freq, freq_chunk):
        fr = pb_freq[f0:f0 + freq_chunk]
        ck_full, wk_full = _lib.gcf_kernels(function, dish, blockage, pairs, fr, npad, cell, npad // 2)
        awk = wk_full.abs()
        amax = awk.amax(dim=(2, 3)).cpu().numpy()
        amin = awk.amin(dim=(2, 3)).cpu().numpy()
        rows = wk_full[:, :, :, c1].cpu().numpy()
        cols = wk_full[:, :, c0, :].cpu().numpy()
        for q in range(n_pair):
            for j in range(len(fr)):
                f = f0 + j
                support[q, f, 0] = calc_conv_size(rows[q, j], cols[q, j], amin[q, j], amax[q, j], npad,
                                                  support_cut_level, os_, max_sup)
                es = (support[q, f, 0] + 1) * os_
                e0 = rs // 2 - es // 2
                for src, dst in ((ck_full, ck), (wk_full, wk)):
                    crop = src[q, j, st[0]:st[0] + rs[0], st[1]:st[1] + rs[1]]
                    nf = crop[e0[0]:e0[0] + es[0], e0[1]:e0[1] + es[1]].sum() / float(os_[0] * os_[1])
                    dst[q, f, 0] = crop / nf
        del ck_full, wk_full, awk
    return ck, wk, support


def _baseline_ant(vis):
    a1 = np.asarray(vis['ANTENNA1'].values)
    a2 = np.asarray(vis['ANTENNA2'].values)
    if a1.ndim == 2:   # (time, baseline): the antennas of each baseline
        a1, a2 = a1.max(axis=0), a2.max(axis=0)
    return np.stack([a1, a2], axis=1).astype(int)


def make_gridding_convolution_function(mxds, gcf_parms, grid_parms, sel_parms):
    """A-term gridding convolution functions for mosaic imaging.

    gcf_parms: function ('casa_airy' | 'airy'), list_dish_diameters,
    list_blockage_diameters, unique_ant_indx, phase_center (radians; also
    accepted as image_phase_center), oversampling [10, 10], max_support
    [15, 15], support_cut_level 0.025, chan_tolerance_factor 0.005.
    grid_parms: image_size, cell_size (arcsec), fft_padding.

    Returns a dataset with CF_BASELINE_MAP, CF_CHAN_MAP, CF_POL_MAP,
    CONV_KERNEL and WEIGHT_CONV_KERNEL (conv_baseline, conv_chan, conv_pol,
    u, v), SUPPORT (..., xy), PHASE_GRADIENT (field_id, u, v) and
    PS_CORR_IMAGE (l, m), attrs cell_uv and oversampling, and phase_slope
    (n_field, 2) -- the (px, py) of PHASE_GRADIENT = exp(i (x px + y py)),
    which the mosaic gridder applies separably.
    """
    import torch
    _gcf = copy.deepcopy(gcf_parms)
    _gp = copy.deepcopy(grid_parms)
    _sel = copy.deepcopy(sel_parms)
    assert 'xds' in _sel, '######### ERROR: xds must be specified in sel_parms'
    vis = mxds.attrs[_sel['xds']]
    _check_sel_parms(vis, _sel)
    _gcf['basline_ant'] = _baseline_ant(vis)
    _gcf['freq_chan'] = vis.coords['chan'].values
    _gcf['pol'] = vis.coords['pol'].values
    field = mxds.attrs['FIELD'] if 'FIELD' in mxds.attrs else mxds['FIELD']
    pd = np.asarray(field['PHASE_DIR'].values)
    _gcf['field_phase_dir'] = pd[:, 0, :] if pd.ndim == 3 else pd
    field_id = np.asarray(field['field_id'].values)
    if 'phase_center' not in _gcf and 'image_phase_center' in _gcf:
        _gcf['phase_center'] = _gcf['image_phase_center']
    assert _check_gcf_parms(_gcf), '######### ERROR: gcf_parms checking failed'
    assert _check_grid_parms(_gp), '######### ERROR: grid_parms checking failed'
    if 'phase_center' not in _gcf:
        raise AssertionError('######### ERROR: gcf_parms phase_center must be specified')

    os_ = np.asarray(_gcf['oversampling'])
    max_sup = np.asarray(_gcf['max_support'])
    rs = (max_sup + 1) * os_
    npad = np.asarray(_gp['image_size_padded'])
    n_types = len(_gcf['list_dish_diameters'])
    cf_baseline_map, pairs = create_cf_baseline_map(_gcf['unique_ant_indx'], _gcf['basline_ant'], n_types)
    cf_chan_map, pb_freq = create_cf_chan_map(_gcf['freq_chan'], _gcf['chan_tolerance_factor'])
    cf_pol_map = np.zeros(len(_gcf['pol']), dtype=int)

    ck, wk, support = gcf_tables(_gcf['function'], _gcf['list_dish_diameters'], _gcf['list_blockage_diameters'],
                                 pairs, pb_freq, _gp, os_, max_sup, _gcf['support_cut_level'])

    slopes = _phase_slopes(_gcf['field_phase_dir'], _gcf['phase_center'], _gp, os_)
    pg = _phase_gradient(slopes, rs)
    image_size = np.asarray(_gp['image_size'])
    coords = {'u': ('u', np.arange(rs[0])), 'v': ('v', np.arange(rs[1])), 'xy': ('xy', np.arange(2)),
              'field_id': ('field_id', field_id), 'l': ('l', np.arange(image_size[0])),
              'm': ('m', np.arange(image_size[1]))}
    dv = {'CF_BASELINE_MAP': (('baseline',), cf_baseline_map), 'CF_CHAN_MAP': (('chan',), cf_chan_map),
          'CF_POL_MAP': (('pol',), cf_pol_map),
          'CONV_KERNEL': (('conv_baseline', 'conv_chan', 'conv_pol', 'u', 'v'), ck.cpu().numpy()),
          'WEIGHT_CONV_KERNEL': (('conv_baseline', 'conv_chan', 'conv_pol', 'u', 'v'), wk.cpu().numpy()),
          'SUPPORT': (('conv_baseline', 'conv_chan', 'conv_pol', 'xy'), support),
          'PHASE_GRADIENT': (('field_id', 'u', 'v'), pg.cpu().numpy()),
          'PS_CORR_IMAGE': (('l', 'm'), np.ones(tuple(image_size)))}
    ds = Dataset(dv, coords)
    ds.attrs['cell_uv'] = 1 / (npad * _gp['cell_size'] * os_)
    ds.attrs['oversampling'] = os_
    ds.attrs['phase_slope'] = slopes
    ds.attrs['pb_freq'] = np.asarray(pb_freq)
    return ds
