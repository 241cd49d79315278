"""make_imaging_weight -- same signature and semantics as
ngcasa/imaging/make_imaging_weight.py:20-115 (density grid, Briggs factors
and nearest-cell lookup run on the GPU)."""
import copy

from ..xds import set_var
from ._imaging_utils._check_imaging_parms import _check_grid_parms, _check_imaging_weights_parms
from ._imaging_utils import _pipeline
from ._imaging_utils._sel import _check_sel_parms, _register_group


def make_imaging_weight(vis_mxds, imaging_weights_parms, grid_parms, sel_parms):
    """Create the imaging-weight variable (time, baseline, chan, pol).

    weighting 'natural' reuses the input weight (no new array, as in the
    reference); 'uniform', 'briggs' (robust in [-2, 2]) and 'briggs_abs' grid
    the weight density on the unpadded grid and divide each weight by
    f0*W+f1 at its cell. Inputs are not modified; a new mxds is returned.
    """
    return _make_imaging_weight(vis_mxds, imaging_weights_parms, grid_parms, sel_parms)


def _make_imaging_weight(vis_mxds, imaging_weights_parms, grid_parms, sel_parms, density_reduce=None):
    _mxds = vis_mxds.copy(deep=False)
    _iwp = copy.deepcopy(imaging_weights_parms)
    _gp = copy.deepcopy(grid_parms)
    _sp = copy.deepcopy(sel_parms)
    assert 'xds' in _sp, '######### ERROR: xds must be specified in sel_parms'
    _vis = _mxds.attrs[_sp['xds']].copy(deep=False)
    _mxds.attrs[_sp['xds']] = _vis
    assert _vis.dims['pol'] <= 2, 'Full polarization is not supported.'
    _check_sel_parms(_vis, _sp, new_or_modified_data_variables={'imaging_weight': 'IMAGING_WEIGHT'},
                     append_to_in_id=True)
    assert _check_imaging_weights_parms(_iwp), '######### ERROR: imaging_weights_parms checking failed'
    gin, gout = _sp['data_group_in'], _sp['data_group_out']
    if _iwp['weighting'] == 'natural':
        gout['imaging_weight'] = gin['weight']
        _register_group(_vis, gout)
        return _mxds
    assert _check_grid_parms(_gp), '######### ERROR: grid_parms checking failed'
    iw = _pipeline.imaging_weights(_vis[gin['uvw']], _vis[gin['weight']], _vis.coords['chan'].values, _gp, _iwp,
                                   density_reduce=density_reduce)
    set_var(_vis, gout['imaging_weight'], iw.cpu().numpy(), _vis[gin['weight']].dims)
    _register_group(_vis, gout)
    return _mxds
