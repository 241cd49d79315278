"""Per-chunk mosaic (GCF-table) gridding functions, backed by libngg on the GPU.

Same names, arguments and return values as the per-chunk functions the
reference's _graph_aperture_grid calls (ngcasa/imaging/_imaging_utils/
_aperture_grid.py): numpy arrays in, numpy arrays out.

* _aperture_grid_numpy_wrap(vis_data, uvw, imaging_weight, field,
  cf_baseline_map, cf_chan_map, cf_pol_map, conv_kernel, weight_support,
  phase_gradient, freq_chan, grid_parms) -> (grid[C,P,Nu,Nv] complex128,
  sum_weight[C,P])                                                   (:294-331)
* _aperture_psf_grid_numpy_wrap(uvw, imaging_weight, field, ...) (PSF)  (:334-373)
* _aperture_weight_grid_numpy_wrap(uvw, imaging_weight, field, ...,
  weight_conv_kernel, ...) (weight grid at the grid centre)            (:146-178)

grid_parms carries image_size_padded, cell_size (radians, [0] negated),
oversampling, chan_mode and field_id (the FIELD_ID of each phase-gradient
plane). The phase gradient must be the separable exp(i (x px + y py)) of
make_gridding_convolution_function; its (px, py) are read off the table.
Grids are accumulated in FP32 (complex64) and returned as complex128.
"""
import numpy as np

from ... import _lib
from ..._lib import NggError
from ._mosaic import field_indices
from ._pipeline import _arr


def _slopes(phase_gradient):
    pg = np.asarray(phase_gradient)
    c0, c1 = pg.shape[1] // 2, pg.shape[2] // 2
    return np.stack([np.angle(pg[:, c0 + 1, c1] / pg[:, c0, c1]), np.angle(pg[:, c0, c1 + 1] / pg[:, c0, c1])],
                    axis=1)


def _run(kind, vis_data, uvw, imaging_weight, field, cf_baseline_map, cf_chan_map, cf_pol_map, table,
         weight_support, phase_gradient, freq_chan, grid_parms):
    n_uv = np.asarray(grid_parms['image_size_padded']).astype(np.int64)
    dl = np.asarray(grid_parms['cell_size'], dtype=np.float64)
    os_ = np.asarray(grid_parms['oversampling']).astype(int)
    fidx = field_indices(field, grid_parms['field_id'])
    args = (uvw, np.asarray(imaging_weight, dtype=np.float32), np.asarray(freq_chan, dtype=np.float64), fidx,
            np.asarray(cf_baseline_map), np.asarray(cf_chan_map), np.asarray(cf_pol_map),
            np.asarray(table, dtype=np.float64), np.asarray(weight_support), _slopes(phase_gradient))
    cm = grid_parms.get('chan_mode', 'cube')
    if np.iscomplexobj(table) and np.abs(np.imag(table)).max() > 0:
        raise NggError('the GCF table must be real (the phase gradient carries the complex part)')
    if kind == 'weight':
        g, sw = _lib.grid_gcf_weight(*args, n_uv, dl, os_, chan_mode=cm)
    else:
        g, sw = _lib.grid_gcf(vis_data, *args, n_uv, dl, os_, mode=kind, chan_mode=cm)
    return g.cpu().numpy().astype(np.complex128), sw.cpu().numpy()


def _aperture_grid_numpy_wrap(vis_data, uvw, imaging_weight, field, cf_baseline_map, cf_chan_map, cf_pol_map,
                              conv_kernel, weight_support, phase_gradient, freq_chan, grid_parms):
    return _run('data', vis_data, uvw, imaging_weight, field, cf_baseline_map, cf_chan_map, cf_pol_map, conv_kernel,
                weight_support, phase_gradient, freq_chan, grid_parms)


def _aperture_psf_grid_numpy_wrap(uvw, imaging_weight, field, cf_baseline_map, cf_chan_map, cf_pol_map, conv_kernel,
                                  weight_support, phase_gradient, freq_chan, grid_parms):
    return _run('psf', None, uvw, imaging_weight, field, cf_baseline_map, cf_chan_map, cf_pol_map, conv_kernel,
                weight_support, phase_gradient, freq_chan, grid_parms)


def _aperture_weight_grid_numpy_wrap(uvw, imaging_weight, field, cf_baseline_map, cf_chan_map, cf_pol_map,
                                     weight_conv_kernel, weight_support, phase_gradient, freq_chan, grid_parms):
    return _run('weight', None, uvw, imaging_weight, field, cf_baseline_map, cf_chan_map, cf_pol_map,
                weight_conv_kernel, weight_support, phase_gradient, freq_chan, grid_parms)


def _graph_aperture_grid(vis_dataset, gcf_dataset, grid_parms, sel_parms):
    """_graph_aperture_grid (_aperture_grid.py:25-143): [grid (u, v, C_img, P),
    sum_weight (C_img, P)] of the mosaic gridder for the dataset's data group
    with the GCF dataset's tables and maps; grid_parms['grid_weights'] selects
    the weight grid (WEIGHT_CONV_KERNEL), grid_parms['do_psf'] the PSF grid.
    One GPU call instead of the reference's dask graph and tree sum."""
    gin = sel_parms['data_group_in']
    grid_parms = dict(grid_parms)
    grid_parms['field_id'] = gcf_dataset['field_id'].values   # as the reference (:59); oversampling from grid_parms
    uvw = _arr(vis_dataset[gin['uvw']])
    weight = _arr(vis_dataset[gin['imaging_weight']])
    field = _arr(vis_dataset['FIELD_ID'])
    maps = (gcf_dataset['CF_BASELINE_MAP'].values, gcf_dataset['CF_CHAN_MAP'].values, gcf_dataset['CF_POL_MAP'].values)
    support = gcf_dataset['SUPPORT'].values
    phase_gradient = gcf_dataset['PHASE_GRADIENT'].values
    freq = vis_dataset.coords['chan'].values
    if grid_parms.get('grid_weights', False):
        grid, sw = _aperture_weight_grid_numpy_wrap(uvw, weight, field, *maps, gcf_dataset['WEIGHT_CONV_KERNEL'].values,
                                                    support, phase_gradient, freq, grid_parms)
    elif grid_parms.get('do_psf', False):
        grid, sw = _aperture_psf_grid_numpy_wrap(uvw, weight, field, *maps, gcf_dataset['CONV_KERNEL'].values, support,
                                                 phase_gradient, freq, grid_parms)
    else:
        grid, sw = _aperture_grid_numpy_wrap(_arr(vis_dataset[gin['data']]), uvw, weight, field, *maps,
                                             gcf_dataset['CONV_KERNEL'].values, support, phase_gradient, freq,
                                             grid_parms)
    return [np.moveaxis(grid, [0, 1], [-2, -1]), np.moveaxis(sw, [0, 1], [-2, -1])]
