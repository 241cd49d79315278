"""synthesis_imaging_cube -- the reference's fused single-call imager
(ngcasa/imaging/synthesis_imaging_cube.py:30-325) on the GPU.

Per channel chunk the reference runs (_synthesis_imaging_cube_std_chunk,
:170-218): flags -> NaN in the visibilities, imaging weights
(_make_imaging_weight_chunk: weight density, Briggs factors, nearest-cell
lookup), the primary beam (_make_pb), the PSF and the dirty image with the
prolate-spheroidal gridder, the grid correction, and the Gaussian fit of the
PSF main lobe (casa_fit). Here the weight density and Briggs factors are one
pass each, and the nearest-cell lookup and the flags are folded into the
packing pass of the PSF and image gridding (ngg_grid_ps_weighted), so no
IMAGING_WEIGHT array is materialised; the primary beams come from
ngg_primary_beam.

Two departures, both documented:
* the reference computes the imaging weights and then grids the PSF and the
  image with the natural weights (:206, :211: `data_weight`), leaving its
  own Briggs/uniform weights unused; its documentation describes the
  function as applying them (docs/imaging/cube_imaging_example.ipynb), and
  with natural weighting (the documented example) both are the same. Here
  the imaging weights are applied.
* flags: as in the reference, only the visibilities are flagged (:180); the
  weights of flagged samples still enter the weight density and the PSF.
"""
import copy

import numpy as np

from .. import _lib
from ..xds import set_var
from ._imaging_utils._beam_fit import LazyBeamFit
from ._imaging_utils._check_imaging_parms import _check_grid_parms, _check_imaging_weights_parms, \
    _check_pb_parms
from ._imaging_utils._gridding_convolutional_kernels import _create_prolate_spheroidal_kernel, \
    _create_prolate_spheroidal_kernel_1D
from ._imaging_utils._pipeline import OVERSAMPLING, SUPPORT, _arr, chan_chunks, fft_precision
from ._imaging_utils._remove_padding import _remove_padding
from ._imaging_utils._sel import _check_sel_parms, _register_group
from .make_image import _image_coords


def synthesis_imaging_cube(vis_mxds, img_xds, grid_parms, imaging_weights_parms, pb_parms, vis_sel_parms,
                           img_sel_parms):
    """Flagging, imaging weights, primary beam, PSF, dirty image and PSF beam
    fit in one call (the reference's signature).

    Adds to a copy of img_xds: IMAGE and PSF (l, m, time, chan, pol),
    IMAGE_SUM_WEIGHT and PSF_SUM_WEIGHT (time, chan, pol), PB (l, m, time,
    chan, pol, dish_type) and RESTORE_PARMS (time, chan, pol, 3): major and
    minor FWHM (in the units of the cell size, radians) and position angle of
    the PSF main lobe. Full polarization is not supported (at most 2 pols).
    Inputs are not modified.
    """
    import torch
    _mxds = vis_mxds.copy(deep=False)
    _vsp = copy.deepcopy(vis_sel_parms)
    _isp = copy.deepcopy(img_sel_parms)
    _gp = copy.deepcopy(grid_parms)
    _iwp = copy.deepcopy(imaging_weights_parms)
    _pbp = copy.deepcopy(pb_parms)
    _img = img_xds.copy(deep=False)
    assert 'xds' in _vsp, '######### ERROR: xds must be specified in sel_parms'
    _vis = _mxds.attrs[_vsp['xds']]
    assert _vis.dims['pol'] <= 2, 'Full polarization is not supported.'
    assert _check_imaging_weights_parms(_iwp), '######### ERROR: imaging_weights_parms checking failed'
    assert _check_grid_parms(_gp), '######### ERROR: grid_parms checking failed'
    assert _check_pb_parms(_img, _pbp), '######### ERROR: pb_parms checking failed'
    _check_sel_parms(_vis, _vsp)
    _check_sel_parms(_img, _isp, new_or_modified_data_variables={
        'image_sum_weight': 'IMAGE_SUM_WEIGHT', 'image': 'IMAGE', 'psf_sum_weight': 'PSF_SUM_WEIGHT', 'psf': 'PSF',
        'pb': 'PB', 'restore_parms': 'RESTORE_PARMS'}, append_to_in_id=True)
    gin, gout = _vsp['data_group_in'], _isp['data_group_out']

    vis = _arr(_vis[gin['data']])
    uvw = _arr(_vis[gin['uvw']])
    weight = _arr(_vis[gin['weight']])
    flag = _arr(_vis[gin['flag']]) if 'flag' in gin else None
    freq = np.asarray(_vis.coords['chan'].values, dtype=np.float64)
    T, B, C, P = np.shape(weight)
    chan_mode = _gp['chan_mode']
    npad = np.asarray(_gp['image_size_padded'])
    image_size = np.asarray(_gp['image_size'])
    cell = np.asarray(_gp['cell_size'], dtype=np.float64)
    _, corr = _create_prolate_spheroidal_kernel(OVERSAMPLING, SUPPORT, npad)
    corr_d = _lib._dev(np.ascontiguousarray(_remove_padding(corr, image_size)), torch.float64, 'correction')
    cgk_d = _lib._dev(_create_prolate_spheroidal_kernel_1D(OVERSAMPLING, SUPPORT), torch.float64, 'cgk_1D')
    uvw_d = _lib._dev(uvw, torch.float64, 'uvw')
    n_img = 1 if chan_mode == 'continuum' else C
    precision = fft_precision(_gp, n_img, P, npad)
    image = np.empty((int(image_size[0]), int(image_size[1]), n_img, P))
    psf = np.empty_like(image)
    isw = np.empty((n_img, P))
    psw = np.empty((n_img, P))
    weighted = _iwp['weighting'] != 'natural'
    # The reference's chunks are channel chunks, and in continuum mode its
    # weight density is that of the chunk's channels alone
    # (_make_imaging_weight_chunk per chunk): a continuum image here is one
    # chunk, as a single-chunk reference call.
    for c0, c1 in chan_chunks(C, P, npad, chan_mode):
        sl = (slice(None), slice(None), slice(c0, c1))
        w_d = _lib._dev(np.asarray(weight)[sl] if not hasattr(weight, 'detach') else weight[sl], torch.float32,
                        'weight')
        v_d = _lib._dev(np.asarray(vis)[sl] if not hasattr(vis, 'detach') else vis[sl], torch.complex64, 'vis')
        f_d = _lib._dev(freq[c0:c1], torch.float64, 'freq')
        fl_d = None
        if flag is not None:
            fl_d = _lib._dev(np.asarray(flag)[sl] if not hasattr(flag, 'detach') else flag[sl], torch.uint8, 'flag')
        dens = fac = None
        if weighted:
            dens, dsw = _lib.grid_density(uvw_d, w_d, f_d, image_size, cell, chan_mode)
            fac = _lib.briggs_factors(dens, dsw, _iwp['weighting'], _iwp.get('robust', 0.5),
                                      _iwp.get('briggs_abs_noise', 1.0))
        out = slice(0, 1) if chan_mode == 'continuum' else slice(c0, c1)
        for do_psf in (True, False):
            g, sw = _lib.grid_ps(None if do_psf else v_d, uvw_d, w_d, f_d, cgk_d, npad, cell,
                                 mode='psf' if do_psf else 'data', chan_mode=chan_mode, layout='fft',
                                 support=SUPPORT, oversampling=OVERSAMPLING, density=dens, factors=fac,
                                 flag=None if do_psf else fl_d)
            img = _lib.fft_correct(g, sw, corr_d, image_size, precision=precision)
            del g
            (psf if do_psf else image)[:, :, out] = img.cpu().numpy()
            (psw if do_psf else isw)[out] = sw.cpu().numpy()
        del w_d, v_d, fl_d, dens, fac

    # primary beam of every dish type (the reference's pol axis repeats it)
    pb_freq = np.array([np.mean(freq)]) if chan_mode == 'continuum' else freq
    pb = _lib.primary_beam(_pbp['function'], _pbp['list_dish_diameters'], _pbp['list_blockage_diameters'],
                           pb_freq, image_size, cell, _gp['image_center'], ipower=2).cpu().numpy()
    pb = np.broadcast_to(pb[:, :, :, None, :], pb.shape[:3] + (P, pb.shape[3]))

    _img = _image_coords(_img, _gp, _vis, chan_mode)
    set_var(_img, gout['image'], image[:, :, None, :, :], ('l', 'm', 'time', 'chan', 'pol'))
    set_var(_img, gout['image_sum_weight'], isw[None, :, :], ('time', 'chan', 'pol'))
    set_var(_img, gout['psf'], psf[:, :, None, :, :], ('l', 'm', 'time', 'chan', 'pol'))
    set_var(_img, gout['psf_sum_weight'], psw[None, :, :], ('time', 'chan', 'pol'))
    set_var(_img, gout['pb'], np.ascontiguousarray(pb)[:, :, None], ('l', 'm', 'time', 'chan', 'pol', 'dish_type'))
    _img = _img.assign_coords({'dish_type': ('dish_type', np.arange(len(_pbp['list_dish_diameters'])))})
    if min(image.shape[0], image.shape[1]) >= 9:
        # casa_fit(psf, npix_window 9x9, sampling 9x9, cutoff 0.35, delta = cell_size) (:217)
        set_var(_img, gout['restore_parms'], LazyBeamFit(psf[:, :, None, :, :], cell),
                ('time', 'chan', 'pol', 'elps_index'))
    _register_group(_img, gout)
    return _img
