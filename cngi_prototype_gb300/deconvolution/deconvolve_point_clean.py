"""deconvolve_point_clean -- ngcasa/deconvolution/deconvolve_point_clean.py:
15-110 (a per-(time, chan) dask graph around _clean_wrap / _clean_jit), with
every plane's Hogbom minor cycle on the GPU (ngg_hogbom_clean).

deconvolve_parms: 'gain' (default 0.1), 'threshold' (relative to each
plane's first peak, default 0.0), 'n_iter' (default 1000), 'psf_scaling':
'peak' (default: Hogbom's algorithm, the PSF scaled by the peak is
subtracted) or 'none' (the reference's code as written, which subtracts
gain*psf, :216). sel_parms['data_group_in'] names 'image' and 'psf';
sel_parms['data_group_out'] names 'model' and 'residual' (defaults MODEL,
RESIDUAL). Adds MODEL and RESIDUAL (l, m, time, chan, pol); the input is not
modified.
"""
import copy

import numpy as np

from .. import _lib
from ..imaging._imaging_utils._pipeline import _arr
from ..xds import set_var


def deconvolve_point_clean(img_xds, deconvolve_parms, sel_parms):
    _img = img_xds.copy(deep=False)
    _dp = {'gain': 0.1, 'threshold': 0.0, 'n_iter': 1000, 'psf_scaling': 'peak', **copy.deepcopy(deconvolve_parms)}
    _sp = copy.deepcopy(sel_parms)
    if _dp['psf_scaling'] not in ('peak', 'none'):
        raise ValueError("deconvolve_parms['psf_scaling'] must be 'peak' or 'none'")
    if not (0.0 < float(_dp['gain']) <= 1.0) or int(_dp['n_iter']) < 0:
        raise ValueError('gain must be in (0, 1] and n_iter >= 0')
    gin = _sp.get('data_group_in', {'image': 'IMAGE', 'psf': 'PSF'})
    gout = {'model': 'MODEL', 'residual': 'RESIDUAL', **_sp.get('data_group_out', {})}
    dirty = np.asarray(_arr(_img[gin['image']]), dtype=np.float64)
    psf = np.asarray(_arr(_img[gin['psf']]), dtype=np.float64)
    model, residual, _ = _lib.hogbom_clean(dirty, psf, _dp['gain'], _dp['threshold'], _dp['n_iter'],
                                           _dp['psf_scaling'] == 'peak')
    dims = _img[gin['image']].dims
    set_var(_img, gout['residual'], residual.cpu().numpy(), dims)
    set_var(_img, gout['model'], model.cpu().numpy(), dims)
    return _img
