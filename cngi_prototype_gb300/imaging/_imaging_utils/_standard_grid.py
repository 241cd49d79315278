"""Per-chunk standard gridding functions, backed by libngg on the GPU.

Same names, arguments and return values as the per-chunk functions the
reference's dask graph builders call (ngcasa/imaging/_imaging_utils/
_standard_grid.py): numpy arrays in, numpy arrays out.

* _standard_grid_numpy_wrap(vis_data, uvw, weight, freq_chan, cgk_1D,
  grid_parms) -> (grid[C,P,Nu,Nv] complex, sum_weight[C,P])       (:123-177)
* _standard_grid_psf_numpy_wrap(uvw, weight, freq_chan, cgk_1D, grid_parms)
  -> (grid[C,P,Nu,Nv] real, sum_weight[C,P]); with
  grid_parms['do_imaging_weight'] the weight-density grid            (:180-236)
* _standard_imaging_weight_degrid_numpy_wrap(grid_imaging_weight[u,v,C,P],
  uvw, natural_imaging_weight, briggs_factors[2,C,P], freq_chan, grid_parms)
  -> imaging_weight[T,B,C,P]                                         (:443-464)

Differences, by design: grids are accumulated in FP32 (complex64 / float32)
and returned as complex128 / float64 arrays for drop-in compatibility;
weights are used as float32.
"""
import numpy as np

from ... import _lib
from ._pipeline import _arr


def _dims(grid_parms):
    return (np.asarray(grid_parms['image_size_padded']).astype(np.int64),
            np.asarray(grid_parms['cell_size'], dtype=np.float64))


def _standard_grid_numpy_wrap(vis_data, uvw, weight, freq_chan, cgk_1D, grid_parms):
    n_uv, dl = _dims(grid_parms)
    cplx = grid_parms.get('complex_grid', True)
    mode = 'data' if not grid_parms.get('do_psf', False) else 'psf'
    grid, sw = _lib.grid_ps(vis_data, uvw, weight, freq_chan, cgk_1D, n_uv, dl, mode=mode,
                            chan_mode=grid_parms.get('chan_mode', 'cube'),
                            support=int(grid_parms['support']), oversampling=int(grid_parms['oversampling']))
    g = grid.cpu().numpy()
    g = g.astype(np.complex128) if (cplx and mode == 'data') else g.astype(np.float64 if not cplx else np.complex128)
    return g, sw.cpu().numpy()


def _standard_grid_psf_numpy_wrap(uvw, weight, freq_chan, cgk_1D, grid_parms):
    n_uv, dl = _dims(grid_parms)
    chan_mode = grid_parms.get('chan_mode', 'cube')
    if grid_parms.get('do_imaging_weight', False):
        dens, dsw = _lib.grid_density(uvw, weight, freq_chan, n_uv, dl, chan_mode)
        P = np.shape(weight)[3]
        d = dens.cpu().numpy().astype(np.float64)
        s = dsw.cpu().numpy()
        return np.repeat(d[:, None], P, axis=1), np.repeat(s[:, None], P, axis=1)
    grid, sw = _lib.grid_ps(None, uvw, weight, freq_chan, cgk_1D, n_uv, dl, mode='psf', chan_mode=chan_mode,
                            support=int(grid_parms['support']), oversampling=int(grid_parms['oversampling']))
    return grid.cpu().numpy().astype(np.float64), sw.cpu().numpy()


def _standard_imaging_weight_degrid_numpy_wrap(grid_imaging_weight, uvw, natural_imaging_weight, briggs_factors,
                                               freq_chan, grid_parms):
    import torch
    n_uv, dl = _dims(grid_parms)
    dens = np.ascontiguousarray(np.moveaxis(np.asarray(grid_imaging_weight), (2, 3), (0, 1))[:, 0])  # (C,N,N)
    f = np.ascontiguousarray(np.asarray(briggs_factors, dtype=np.float64)[:, :, 0])                 # (2,C)
    out = _lib.weight_lookup(uvw, natural_imaging_weight, freq_chan,
                             torch.as_tensor(dens, dtype=torch.float32, device='cuda'),
                             torch.as_tensor(f, device='cuda'), dl, grid_parms.get('chan_mode', 'cube'))
    return out.cpu().numpy().astype(np.float64)


def _graph_standard_grid(vis_dataset, cgk_1D, grid_parms, sel_parms):
    """_graph_standard_grid (_standard_grid.py:23-106): [grid (u, v, C_img, P),
    sum_weight (C_img, P)] of the dataset's data group. The reference builds a
    dask graph of per-(time, baseline, chan) chunk gridders merged by a tree
    sum; here the whole cube is one GPU call (channel-chunked by the caller
    when it exceeds device memory), so the result is returned computed.
    grid_parms['do_psf'] selects the PSF (real) grid."""
    gin = sel_parms['data_group_in']
    uvw = vis_dataset[gin['uvw']]
    weight = vis_dataset[gin['imaging_weight']]
    freq = vis_dataset.coords['chan'].values
    if grid_parms.get('do_psf', False):
        grid, sw = _standard_grid_psf_numpy_wrap(_arr(uvw), _arr(weight), freq, cgk_1D, grid_parms)
    else:
        grid, sw = _standard_grid_numpy_wrap(_arr(vis_dataset[gin['data']]), _arr(uvw), _arr(weight), freq, cgk_1D,
                                             grid_parms)
    return [np.moveaxis(grid, [0, 1], [-2, -1]), np.moveaxis(sw, [0, 1], [-2, -1])]
