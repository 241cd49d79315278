"""make_image_with_gcf / make_psf_with_gcf -- same signatures and outputs as
ngcasa/imaging/make_image_with_gcf.py:20-180 and make_psf_with_gcf.py:20-140:
mosaic gridding with the GCF table (ngg_grid_gcf), inverse FFT and crop
(ngg_fft_correct), and the forward normalisation of _normalize.py
(ngg_mosaic_normalize), on the GPU."""
import copy

import numpy as np

from .. import _lib
from ..xds import set_var
from ._imaging_utils._check_imaging_parms import _check_grid_parms, _check_norm_parms
from ._imaging_utils._mosaic import gcf_planes
from ._imaging_utils._sel import _check_sel_parms, _register_group
from .make_image import _image_coords


def _normalize(image, img_xds, gcf_xds, norm_parms, gin, centre=None):
    """_normalize.py:14-90, forward direction, in place on the device image."""
    nt = norm_parms['norm_type']
    pb = np.asarray(img_xds[gin['pb']].values)[:, :, 0]
    nimg = None
    if nt == 'flat_noise':
        nimg = pb
    elif nt == 'flat_sky':
        nimg = np.asarray(img_xds[gin['weight_pb']].values)[:, :, 0]
    ps = np.asarray(gcf_xds['PS_CORR_IMAGE'].values, dtype=np.float64)
    _lib.mosaic_normalize(image, ps_corr=ps, norm_image=nimg, pb=pb, pb_limit=float(norm_parms['pb_limit']),
                          oversampling=np.asarray(gcf_xds.attrs['oversampling']),
                          single_precision=bool(norm_parms['single_precision']), centre=centre)
    return image


def _make(mxds, gcf_dataset, img_dataset, grid_parms, norm_parms, vis_sel_parms, img_sel_parms, do_psf):
    _img = img_dataset.copy(deep=False)
    _vsp = copy.deepcopy(vis_sel_parms)
    _isp = copy.deepcopy(img_sel_parms)
    _gp = copy.deepcopy(grid_parms)
    _np = copy.deepcopy(norm_parms)
    assert 'xds' in _vsp, '######### ERROR: xds must be specified in sel_parms'
    vis = mxds.attrs[_vsp['xds']]
    assert _check_grid_parms(_gp), '######### ERROR: grid_parms checking failed'
    assert _check_norm_parms(_np), '######### ERROR: norm_parms checking failed'
    _check_sel_parms(vis, _vsp)
    new = {'sum_weight': 'PSF_SUM_WEIGHT', 'psf': 'PSF'} if do_psf else {'sum_weight': 'SUM_WEIGHT', 'image': 'IMAGE'}
    _check_sel_parms(_img, _isp, new_or_modified_data_variables=new,
                     required_data_variables={'pb': 'PB', 'weight_pb': 'WEIGHT_PB'}, append_to_in_id=False)
    gin, gout = _vsp['data_group_in'], _isp['data_group_out']
    iw = vis[gin.get('imaging_weight', gin.get('weight'))]
    img, sw = gcf_planes('psf' if do_psf else 'data', None if do_psf else vis[gin['data']], vis[gin['uvw']], iw,
                         vis['FIELD_ID'], vis.coords['chan'].values, gcf_dataset, _gp)
    centre = np.asarray(_gp['image_center']) if do_psf else None
    _normalize(img, img_dataset, gcf_dataset, _np, _isp['data_group_in'], centre)
    _img = _image_coords(_img, _gp, vis, _gp['chan_mode'])
    set_var(_img, gout['sum_weight'], sw[None], ('time', 'chan', 'pol'))
    set_var(_img, gout['psf' if do_psf else 'image'], img.cpu().numpy()[:, :, None],
            ('l', 'm', 'time', 'chan', 'pol'))
    _register_group(_img, gout)
    return _img


def make_image_with_gcf(mxds, gcf_dataset, img_dataset, grid_parms, norm_parms, vis_sel_parms, img_sel_parms):
    """Mosaic dirty image: IMAGE (l, m, time, chan, pol) and SUM_WEIGHT.

    norm_parms: norm_type 'flat_sky' (divide by WEIGHT_PB) | 'flat_noise'
    (divide by PB) | 'none', pb_limit 0.2 (zero where PB < pb_limit),
    single_precision True. img_dataset must hold PB and WEIGHT_PB
    (make_mosaic_pb).
    """
    return _make(mxds, gcf_dataset, img_dataset, grid_parms, norm_parms, vis_sel_parms, img_sel_parms, False)


def make_psf_with_gcf(mxds, gcf_dataset, img_dataset, grid_parms, norm_parms, vis_sel_parms, img_sel_parms):
    """Mosaic PSF, normalised as the image and divided by its value at the
    image centre; PSF (l, m, time, chan, pol) and PSF_SUM_WEIGHT. The
    reference's Gaussian beam fit (fit_gaussian) is not part of this
    library."""
    return _make(mxds, gcf_dataset, img_dataset, grid_parms, norm_parms, vis_sel_parms, img_sel_parms, True)
