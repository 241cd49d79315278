"""make_image / make_psf -- same signatures and semantics as
ngcasa/imaging/make_image.py:27-175 and make_psf.py:27-264 (GPU gridding,
cuFFT, fused crop and grid correction)."""
import copy

import numpy as np

from ..xds import set_var
from ._imaging_utils._check_imaging_parms import _check_grid_parms
from ._imaging_utils import _pipeline
from ._imaging_utils._beam_fit import LazyBeamFit
from ._imaging_utils._sel import _check_sel_parms, _register_group


def _image_coords(img_xds, grid_parms, vis, chan_mode):
    n = np.asarray(grid_parms['image_size'])
    cell = np.asarray(grid_parms['cell_size'])
    c = np.asarray(grid_parms['image_center'])
    l = (np.arange(n[0]) - c[0]) * cell[0]
    m = (np.arange(n[1]) - c[1]) * cell[1]
    freq = vis.coords['chan'].values
    chan = np.array([np.mean(freq)]) if chan_mode == 'continuum' else freq
    coords = {'l': ('l', l), 'm': ('m', m), 'chan': ('chan', chan), 'pol': ('pol', vis.coords['pol'].values),
              'time': ('time', np.array([np.mean(vis.coords['time'].values)]))}
    return img_xds.assign_coords(coords)


def _make(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, do_psf, cube_fn=None):
    _mxds = vis_mxds.copy(deep=False)
    _img = img_xds.copy(deep=False)
    _vsp = copy.deepcopy(vis_sel_parms)
    _isp = copy.deepcopy(img_sel_parms)
    _gp = copy.deepcopy(grid_parms)
    assert _check_grid_parms(_gp), '######### ERROR: grid_parms checking failed'
    assert 'xds' in _vsp, '######### ERROR: xds must be specified in sel_parms'
    _vis = _mxds.attrs[_vsp['xds']]
    _check_sel_parms(_vis, _vsp)
    new = ({'sum_weight': 'PSF_SUM_WEIGHT', 'psf': 'PSF', 'psf_fit': 'PSF_FIT'} if do_psf
           else {'sum_weight': 'SUM_WEIGHT', 'image': 'IMAGE'})
    _check_sel_parms(_img, _isp, new_or_modified_data_variables=new, append_to_in_id=True)
    gin, gout = _vsp['data_group_in'], _isp['data_group_out']
    iw_name = gin.get('imaging_weight', gin.get('weight'))
    vis = None if do_psf else _vis[gin['data']]
    cube_fn = cube_fn or _pipeline.image_cube
    image, sw = cube_fn(vis, _vis[gin['uvw']], _vis[iw_name], _vis.coords['chan'].values, _gp, do_psf)
    _img = _image_coords(_img, _gp, _vis, _gp['chan_mode'])
    set_var(_img, gout['sum_weight'], sw[None, :, :], ('time', 'chan', 'pol'))
    set_var(_img, gout['psf' if do_psf else 'image'], image[:, :, None, :, :], ('l', 'm', 'time', 'chan', 'pol'))
    if do_psf and min(image.shape[0], image.shape[1]) >= 9:
        # the Gaussian beam fit of the PSF main lobe (make_psf.py:159 calls
        # cngi.image.fit_gaussian), evaluated when PSF_FIT is first read
        delta = np.asarray(_gp['cell_size'], dtype=np.float64) * 3600.0 * 180.0 / np.pi
        set_var(_img, gout['psf_fit'], LazyBeamFit(image[:, :, None, :, :], delta),
                ('time', 'chan', 'pol', 'elps_index'))
    _register_group(_img, gout)
    return _img


def make_image(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms):
    """Cube or continuum dirty image with the prolate-spheroidal gridder.

    Adds IMAGE (l, m, time, chan, pol) = Re(FFT^-1 grid) * Nu*Nv cropped,
    divided by SUM_WEIGHT (time, chan, pol) and the grid-correction image.
    grid_parms: image_size, cell_size (arcsec), chan_mode, fft_padding.
    """
    return _make(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, False)


def make_psf(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms):
    """PSF (the image of the imaging weights), PSF_SUM_WEIGHT and PSF_FIT.

    PSF_FIT (time, chan, pol, 3): major / minor FWHM (arcsec) and position
    angle (degrees) of the elliptical Gaussian fitted to the PSF main lobe, as
    the reference's cngi.image.fit_gaussian computes it; like the reference's
    dask result it is evaluated on first access.
    """
    return _make(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, True)
