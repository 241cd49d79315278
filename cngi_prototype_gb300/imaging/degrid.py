"""Differentiable degridding: model image -> model visibilities, with the
gridder as its exact adjoint.

The dirty-image operator of make_image (grid with the PS kernel, inverse FFT,
crop, divide by sum_weight and the grid-correction image) is linear in the
visibilities for fixed weights:

    D : vis (T,B,C,P) complex -> image (N0,N1,C,P) real.

``ImagingOperator.degrid`` applies its transpose D^T (ngg_fft_correct_adjoint
followed by ngg_degrid_ps) and ``ImagingOperator.image`` applies D
(ngg_grid_ps + ngg_fft_correct) with sum_weight frozen at the value the
weights give, so the pair is exactly adjoint:
    Re <D^T x, y> = <x, D y>.
``Degrid`` wraps D^T as a torch.autograd.Function whose backward is D; the
gradient of a chi-square in the visibilities is therefore twice the dirty
image of the residual visibilities (the reference gridder's residual image).
The reference has no visibility degridder (_standard_grid.py:429-430).
"""
import numpy as np

from .. import _lib
from ._imaging_utils._check_imaging_parms import _check_grid_parms
from ._imaging_utils._gridding_convolutional_kernels import _create_prolate_spheroidal_kernel, \
    _create_prolate_spheroidal_kernel_1D
from ._imaging_utils._remove_padding import _remove_padding

OVERSAMPLING = 100
SUPPORT = 7


class ImagingOperator:
    """Fixed geometry (uvw, weights, channels, grid) of the imaging operator D."""

    def __init__(self, uvw, weight, freq, grid_parms):
        import torch
        gp = dict(grid_parms)
        if 'image_size_padded' not in gp:
            assert _check_grid_parms(gp), 'grid_parms checking failed'
        self.grid_parms = gp
        self.npad = np.asarray(gp['image_size_padded'])
        self.image_size = np.asarray(gp['image_size'])
        self.cell = np.asarray(gp['cell_size'], dtype=np.float64)
        self.chan_mode = gp.get('chan_mode', 'cube')
        self.uvw = _lib._dev(uvw, torch.float64, 'uvw')
        self.weight = _lib._dev(weight, torch.float32, 'weight')
        self.freq = _lib._dev(np.asarray(freq, dtype=np.float64), torch.float64, 'freq')
        self.cgk = _lib._dev(_create_prolate_spheroidal_kernel_1D(OVERSAMPLING, SUPPORT), torch.float64, 'cgk')
        corr = _remove_padding(_create_prolate_spheroidal_kernel(OVERSAMPLING, SUPPORT, self.npad)[1],
                               self.image_size)
        self.correction = _lib._dev(np.ascontiguousarray(corr), torch.float64, 'correction')
        self.shape = tuple(self.weight.shape)
        # sum_weight of the weights alone (what every vis-independent D divides by)
        _, self.sum_weight = _lib.grid_ps(None, self.uvw, self.weight, self.freq, self.cgk, self.npad, self.cell,
                                          mode='psf', chan_mode=self.chan_mode, layout='fft',
                                          support=SUPPORT, oversampling=OVERSAMPLING)

    def image(self, vis):
        """D: visibilities -> dirty image (N0,N1,C_img,P) float64."""
        g, _ = _lib.grid_ps(vis, self.uvw, self.weight, self.freq, self.cgk, self.npad, self.cell, mode='data',
                            chan_mode=self.chan_mode, layout='fft', support=SUPPORT, oversampling=OVERSAMPLING)
        return _lib.fft_correct(g, self.sum_weight, self.correction, self.image_size)

    def degrid(self, image):
        """D^T: image (N0,N1,C_img,P) -> model visibilities (T,B,C,P) complex64."""
        g = _lib.fft_correct_adjoint(image, self.sum_weight, self.correction, self.npad)
        return _lib.degrid_ps(g, self.uvw, self.weight, self.freq, self.cgk, self.shape, self.cell,
                              chan_mode=self.chan_mode, layout='fft', support=SUPPORT, oversampling=OVERSAMPLING)


def _autograd():
    import torch

    class Degrid(torch.autograd.Function):
        """image -> model visibilities; backward = the gridder (the adjoint)."""

        @staticmethod
        def forward(ctx, image, op):
            ctx.op = op
            ctx.dtype = image.dtype
            return op.degrid(image.detach())

        @staticmethod
        def backward(ctx, grad_vis):
            # torch's gradient for a real loss of complex V is dL/dRe V + i dL/dIm V,
            # so the image gradient is Re<dV/dx, grad> = D(grad)
            g = ctx.op.image(grad_vis.contiguous().to(torch.complex64))
            return g.to(ctx.dtype), None

    return Degrid


_DEGRID = None


def degrid(image, op):
    """Differentiable D^T (see module docstring)."""
    global _DEGRID
    if _DEGRID is None:
        _DEGRID = _autograd()
    return _DEGRID.apply(image, op)
