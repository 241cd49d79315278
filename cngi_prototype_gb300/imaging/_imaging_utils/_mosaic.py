"""GPU mosaic (GCF-table) pipeline shared by make_mosaic_pb, make_image_with_gcf
and make_psf_with_gcf.

Replaces _graph_aperture_grid (ngcasa/imaging/_imaging_utils/_aperture_grid.py:
21-143): instead of a dask graph of per-chunk numba gridders and a tree sum,
channels are gridded in chunks sized to a device-memory budget straight into
FFT-ordered planes (ngg_grid_gcf / ngg_grid_gcf_weight), inverse transformed
and cropped on the device (ngg_fft_correct with a correction of ones, which
leaves Re(FFT^-1 grid) * Nu*Nv / sum_weight), then normalised in place
(ngg_mosaic_normalize).
"""
import numpy as np

from ... import _lib
from ._pipeline import GRID_BUDGET_BYTES, _arr, _slice_chan, chan_chunks


def field_indices(field, field_id):
    """FIELD_ID (T, B) -> index into the GCF's field list, -1 for rows without
    a field (the reference skips FIELD_ID <= -1 and looks the others up with
    np.where(field_id == FIELD_ID)[0][0], _aperture_grid.py:447-449)."""
    f = np.asarray(_arr(field))
    fid = np.asarray(field_id).ravel()
    out = np.full(f.shape, -1, dtype=np.int32)
    for v in np.unique(f[f > -1]):
        hit = np.where(fid == v)[0]
        if len(hit) == 0:
            raise ValueError(f'FIELD_ID {v} is not in the gridding convolution function field list')
        out[f == v] = hit[0]
    return out


def phase_slopes(gcf_xds):
    """Per-field (px, py) of PHASE_GRADIENT = exp(i (x px + y py)): the
    attribute make_gridding_convolution_function stores, or, for a table
    built elsewhere, the phase step along each axis at the table centre."""
    if 'phase_slope' in gcf_xds.attrs:
        return np.asarray(gcf_xds.attrs['phase_slope'], dtype=np.float64).reshape(-1, 2)
    pg = np.asarray(gcf_xds['PHASE_GRADIENT'].values)
    c0, c1 = pg.shape[1] // 2, pg.shape[2] // 2
    px = np.angle(pg[:, c0 + 1, c1] / pg[:, c0, c1])
    py = np.angle(pg[:, c0, c1 + 1] / pg[:, c0, c1])
    return np.stack([px, py], axis=1)


def gcf_planes(kind, vis, uvw, imaging_weight, field, freq, gcf_xds, grid_parms):
    """Mosaic image planes before normalisation.

    kind: 'data' (make_image_with_gcf), 'psf' (make_psf_with_gcf) or
    'weight' (make_mosaic_pb). When gcf_xds.attrs['learned_gcf'] holds a
    LearnedGCF, the data / PSF grids use its per-channel tables (the weight
    grid keeps WEIGHT_CONV_KERNEL). Returns (image (l, m, Cimg, P) float64 CUDA
    tensor = Re(FFT^-1 grid) * Nu*Nv / sum_weight, sum_weight (Cimg, P)
    float64 numpy).
    """
    import torch
    npad = np.asarray(grid_parms['image_size_padded'])
    image_size = np.asarray(grid_parms['image_size'])
    cell = np.asarray(grid_parms['cell_size'], dtype=np.float64)
    chan_mode = grid_parms.get('chan_mode', 'cube')
    os_ = np.asarray(gcf_xds.attrs['oversampling']).astype(int)
    w = _arr(imaging_weight)
    T, B, C, P = w.shape
    freq = np.asarray(freq, dtype=np.float64)
    uvw_d = _lib._dev(_arr(uvw), torch.float64, 'uvw')
    fidx = _lib._dev(field_indices(field, gcf_xds['field_id'].values), torch.int32, 'field_index')
    table = gcf_xds['WEIGHT_CONV_KERNEL' if kind == 'weight' else 'CONV_KERNEL'].values
    ck_d = _lib._dev(np.asarray(table, dtype=np.float64), torch.float64, 'conv_kernel')
    sup_d = _lib._dev(np.asarray(gcf_xds['SUPPORT'].values, dtype=np.int32), torch.int32, 'support')
    slope_d = _lib._dev(phase_slopes(gcf_xds), torch.float64, 'phase_slope')
    cfb = np.asarray(gcf_xds['CF_BASELINE_MAP'].values, dtype=np.int32)
    cfc = np.asarray(gcf_xds['CF_CHAN_MAP'].values, dtype=np.int32)
    cfp = np.asarray(gcf_xds['CF_POL_MAP'].values, dtype=np.int32)
    ones = torch.ones((int(image_size[0]), int(image_size[1])), dtype=torch.float64, device='cuda')
    n_img = 1 if chan_mode == 'continuum' else C
    image = torch.empty((int(image_size[0]), int(image_size[1]), n_img, P), dtype=torch.float64, device='cuda')
    sum_weight = np.empty((n_img, P), dtype=np.float64)
    # continuum: one image accumulates every channel, so grid them in one call
    for c0, c1 in chan_chunks(C, P, npad, chan_mode, GRID_BUDGET_BYTES):
        wv = _slice_chan(w, c0, c1) if (c0, c1) != (0, C) else w
        common = (uvw_d, wv, freq[c0:c1], fidx, cfb, cfc[c0:c1], cfp, ck_d, sup_d, slope_d)
        learned = gcf_xds.attrs.get('learned_gcf') if hasattr(gcf_xds, 'attrs') else None
        if kind == 'weight':
            g, sw = _lib.grid_gcf_weight(*common, npad, cell, os_, chan_mode=chan_mode, layout='fft')
        elif learned is not None:
            vv = None
            if kind == 'data':
                v = _arr(vis)
                vv = _slice_chan(v, c0, c1) if (c0, c1) != (0, C) else v
            g, sw = learned.grid(vv, uvw_d, wv, freq[c0:c1], fidx, slope_d, npad, cell, mode=kind,
                                 chan_mode=chan_mode, layout='fft')
        else:
            vv = None
            if kind == 'data':
                v = _arr(vis)
                vv = _slice_chan(v, c0, c1) if (c0, c1) != (0, C) else v
            g, sw = _lib.grid_gcf(vv, *common, npad, cell, os_, mode=kind, chan_mode=chan_mode, layout='fft')
        img = _lib.fft_correct(g, sw, ones, image_size)
        del g
        dst = slice(0, 1) if chan_mode == 'continuum' else slice(c0, c1)
        image[:, :, dst] = img
        sum_weight[dst] = sw.cpu().numpy()
    return image, sum_weight
