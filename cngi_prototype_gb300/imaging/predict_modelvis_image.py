"""predict_modelvis_image -- model visibilities from a model image cube.

The reference declares this function (ngcasa/imaging/predict_modelvis_image.py:20-39)
but leaves it unimplemented; its docstring and comments give the contract:
predict model visibilities from a model image (Jy/pixel) with the gridding
convolution function, save them under ``arr_name`` (default 'MODEL'),
optionally add to an existing model (``incremental``), and treat a one-channel
cube as a continuum image. Its listed steps are flat-sky normalisation,
stokes_to_corr, Fourier transform and degridding.

Here, for the standard prolate-spheroidal gridder (the one make_image uses):
the model is divided by the grid-correction image, embedded in the padded
grid and Fourier transformed (ngg_fft_correct_adjoint with unit sum_weight:
the exact adjoint of make_image's crop, correction and inverse FFT), then
every visibility reads back its 7x7 footprint, with the gridder's own cells,
oversampling offsets and edge rule, divided by its kernel sum
(ngg_predict_ps). The result is sum_pixels I(l, m) exp(-2 pi i (u l + v m)),
the sign under which make_image puts a source back at its pixel, up to the
kernel's aliasing and the 1/oversampling quantisation of the kernel offset
(a phase error of at most 2 pi |x| / (2 oversampling Npad) for a source x
pixels from the centre, as in the gridder). Visibilities whose footprint
crosses the grid edge, or whose uvw is NaN, are predicted as 0, as the
gridder drops them.

The model's pol axis is taken as correlations (the same basis the gridder
images); a one-pol model is broadcast to every correlation (Stokes I with
parallel-hand correlations, RR = LL = I). No primary-beam (flat-sky) step:
the standard gridder has none.
"""
import numpy as np

from .. import _lib
from ..xds import set_var
from ._imaging_utils._check_imaging_parms import _check_grid_parms
from ._imaging_utils._gridding_convolutional_kernels import _create_prolate_spheroidal_kernel, \
    _create_prolate_spheroidal_kernel_1D
from ._imaging_utils._remove_padding import _remove_padding

OVERSAMPLING = 100
SUPPORT = 7


def predict_modelvis_image(img_dataset, vis_dataset, grid_parms, storage_parms=None, model='MODEL', uvw='UVW'):
    """Return a copy of vis_dataset with model visibilities (time, baseline, chan, pol).

    img_dataset[model]: (l, m, time, chan, pol) model image in Jy/pixel, one
    time plane, chan = 1 (continuum) or the visibilities' channel count, pol =
    1 or the visibilities' pol count. grid_parms: image_size and cell_size
    (arcsec) of that model, fft_padding (default 1.2), as make_image.
    storage_parms: arr_name (default 'MODEL'), incremental (default False:
    replace; True: add to an existing arr_name). The inputs are not modified.
    """
    import torch
    sp = {'arr_name': 'MODEL', 'incremental': False, **(storage_parms or {})}
    gp = dict(grid_parms)
    assert _check_grid_parms(gp), '######### ERROR: grid_parms checking failed'
    if model not in img_dataset:
        raise KeyError('model image %r not in img_dataset' % (model,))
    img = np.asarray(img_dataset[model])
    if img.ndim != 5:
        raise ValueError('model image must be (l, m, time, chan, pol), got shape %s' % (img.shape,))
    size = np.asarray(gp['image_size'])
    if tuple(img.shape[:2]) != tuple(int(x) for x in size):
        raise ValueError('model image is %dx%d, grid_parms image_size is %s' % (img.shape[0], img.shape[1], size))
    if img.shape[2] != 1:
        raise ValueError('model image must have one time plane, got %d' % img.shape[2])
    T, B = vis_dataset[uvw].shape[:2]
    freq = np.asarray(vis_dataset.coords['chan'].values, dtype=np.float64)
    C = len(freq)
    P = len(vis_dataset.coords['pol'].values)
    C_img, P_img = img.shape[3], img.shape[4]
    if C_img not in (1, C):
        raise ValueError('model has %d channels; expected 1 (continuum) or %d' % (C_img, C))
    if P_img not in (1, P):
        raise ValueError('model has %d pols; expected 1 or %d' % (P_img, P))
    chan_mode = 'continuum' if (C_img == 1 and C > 1) else 'cube'

    npad = np.asarray(gp['image_size_padded'])
    m = torch.as_tensor(np.ascontiguousarray(img[:, :, 0, :, :], dtype=np.float64), device='cuda')
    if P_img != P:
        m = m.expand(-1, -1, -1, P).contiguous()
    corr = _remove_padding(_create_prolate_spheroidal_kernel(OVERSAMPLING, SUPPORT, npad)[1], size)
    ones = torch.ones((C_img, P), dtype=torch.float64, device='cuda')
    grid = _lib.fft_correct_adjoint(m, ones, np.ascontiguousarray(corr), npad)
    vis = _lib.degrid_ps(grid, np.asarray(vis_dataset[uvw], dtype=np.float64), None, freq,
                         _create_prolate_spheroidal_kernel_1D(OVERSAMPLING, SUPPORT), (T, B, C, P), gp['cell_size'],
                         chan_mode=chan_mode, layout='fft', support=SUPPORT, oversampling=OVERSAMPLING,
                         normalize=True)
    out = vis.cpu().numpy()
    name = sp['arr_name']
    ds = vis_dataset.copy(deep=False)
    if sp['incremental'] and name in vis_dataset:
        prev = np.asarray(vis_dataset[name])
        out = (prev + out).astype(prev.dtype)
    elif 'DATA' in vis_dataset and np.iscomplexobj(np.asarray(vis_dataset['DATA'])):
        out = out.astype(np.asarray(vis_dataset['DATA']).dtype)
    set_var(ds, name, out, ('time', 'baseline', 'chan', 'pol'))
    return ds
