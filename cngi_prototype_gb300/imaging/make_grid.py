"""make_grid -- same signature and semantics as ngcasa/imaging/make_grid.py:27-142:
the gridded visibilities themselves (no FFT), from the GPU gridder."""
import copy

import numpy as np

from ..xds import set_var
from ._imaging_utils._check_imaging_parms import _check_grid_parms
from ._imaging_utils._gridding_convolutional_kernels import _create_prolate_spheroidal_kernel_1D
from ._imaging_utils._sel import _check_sel_parms, _register_group
from ._imaging_utils._standard_grid import _graph_standard_grid
from .make_image import _image_coords


def make_grid(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms):
    """Grid the visibilities of the selected data group with the
    prolate-spheroidal kernel (oversampling 100, support 7).

    Adds GRID (u, v, time, chan, pol) complex128 -- the padded uv-grid of
    make_image before its FFT -- and SUM_WEIGHT (time, chan, pol) to a copy of
    img_xds. The data group must name 'data' and 'imaging_weight' (as after
    make_imaging_weight). Inputs are not modified.
    """
    _mxds = vis_mxds.copy(deep=False)
    _img = img_xds.copy(deep=False)
    _vsp = copy.deepcopy(vis_sel_parms)
    _isp = copy.deepcopy(img_sel_parms)
    _gp = copy.deepcopy(grid_parms)
    assert _check_grid_parms(_gp), '######### ERROR: grid_parms checking failed'
    assert 'xds' in _vsp, '######### ERROR: xds must be specified in sel_parms'
    _vis = _mxds.attrs[_vsp['xds']]
    _check_sel_parms(_vis, _vsp)
    _check_sel_parms(_img, _isp, new_or_modified_data_variables={'sum_weight': 'SUM_WEIGHT', 'grid': 'GRID'},
                     append_to_in_id=True)
    gin = _vsp['data_group_in']
    if 'imaging_weight' not in gin:
        gin['imaging_weight'] = gin['weight']
    _gp['oversampling'] = 100
    _gp['support'] = 7
    _gp['complex_grid'] = True
    _gp['do_psf'] = False
    cgk_1D = _create_prolate_spheroidal_kernel_1D(_gp['oversampling'], _gp['support'])
    grid, sw = _graph_standard_grid(_vis, cgk_1D, _gp, _vsp)
    gout = _isp['data_group_out']
    _img = _image_coords(_img, _gp, _vis, _gp['chan_mode'])
    set_var(_img, gout['sum_weight'], np.asarray(sw)[None, :, :], ('time', 'chan', 'pol'))
    set_var(_img, gout['grid'], np.asarray(grid)[:, :, None, :, :], ('u', 'v', 'time', 'chan', 'pol'))
    _register_group(_img, gout)
    return _img
