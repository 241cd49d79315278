"""make_mosaic_pb -- same signature and outputs as
ngcasa/imaging/make_mosaic_pb.py:30-176: the weight grid of every
visibility's weight GCF placed at the grid centre (ngg_grid_gcf_weight),
inverse FFT, WEIGHT_PB = image / sum_weight and PB = sqrt(|WEIGHT_PB|), on
the GPU."""
import copy

from .. import _lib
from ..xds import set_var
from ._imaging_utils._check_imaging_parms import _check_grid_parms
from ._imaging_utils._mosaic import gcf_planes
from ._imaging_utils._sel import _check_sel_parms, _register_group
from .make_image import _image_coords


def make_mosaic_pb(mxds, gcf_dataset, img_dataset, vis_sel_parms, img_sel_parms, grid_parms):
    """Adds PB and WEIGHT_PB (l, m, time, chan, pol) and WEIGHT_PB_SUM_WEIGHT
    (time, chan, pol) to img_dataset (a copy)."""
    _img = img_dataset.copy(deep=False)
    _vsp = copy.deepcopy(vis_sel_parms)
    _isp = copy.deepcopy(img_sel_parms)
    _gp = copy.deepcopy(grid_parms)
    assert 'xds' in _vsp, '######### ERROR: xds must be specified in sel_parms'
    vis = mxds.attrs[_vsp['xds']]
    assert _check_grid_parms(_gp), '######### ERROR: grid_parms checking failed'
    _check_sel_parms(vis, _vsp)
    _check_sel_parms(_img, _isp, new_or_modified_data_variables={'pb': 'PB', 'weight_pb': 'WEIGHT_PB',
                                                                 'weight_pb_sum_weight': 'WEIGHT_PB_SUM_WEIGHT'},
                     append_to_in_id=True)
    gin, gout = _vsp['data_group_in'], _isp['data_group_out']
    iw = vis[gin.get('imaging_weight', gin.get('weight'))]
    wimg, sw = gcf_planes('weight', None, vis[gin['uvw']], iw, vis['FIELD_ID'], vis.coords['chan'].values,
                          gcf_dataset, _gp)
    pb = _lib.sqrt_abs(wimg)
    _img = _image_coords(_img, _gp, vis, _gp['chan_mode'])
    set_var(_img, gout['pb'], pb.cpu().numpy()[:, :, None], ('l', 'm', 'time', 'chan', 'pol'))
    set_var(_img, gout['weight_pb'], wimg.cpu().numpy()[:, :, None], ('l', 'm', 'time', 'chan', 'pol'))
    set_var(_img, gout['weight_pb_sum_weight'], sw[None], ('time', 'chan', 'pol'))
    _register_group(_img, gout)
    return _img
