"""Elliptical Gaussian fit of the PSF main lobe (the PSF_FIT that make_psf
attaches; cngi/image/fit_gaussian.py: fit_gaussian / casa_fit, host side).

Per (time, chan, pol) plane: the npix_window box at the image centre is
resampled on a sampling grid by scipy's bivariate spline (interpn,
'splinef2d'), values below cutoff are masked, and (sigma_x, sigma_y, angle)
of a unit-peak rotated Gaussian centred on the box minimise the squared
residual (scipy.optimize.minimize, default BFGS, from (2.5, 2.5, 0)). The
result is reported as (major FWHM, minor FWHM) in arcsec and a position
angle in degrees, with the reference's conventions (FWHM = 2.355 sigma,
angle = -(fitted angle - 90) folded into (-90, 90]).
"""
import numpy as np


def _rotated_gaussian(params, half):
    """Unit-peak Gaussian on the (2*half0+1, 2*half1+1) sampling grid."""
    sx, sy, rot = params
    theta = np.deg2rad(90.0 - rot)
    x = (np.arange(2 * half[0] + 1) - half[0])[:, None].astype(np.float64)
    y = (np.arange(2 * half[1] + 1) - half[1])[None, :].astype(np.float64)
    xr = x * np.cos(theta) - y * np.sin(theta)
    yr = x * np.sin(theta) + y * np.cos(theta)
    return np.exp(-((xr / sx) ** 2 + (yr / sy) ** 2) / 2.0)


def _chi2(params, samples, keep, half):
    g = _rotated_gaussian(params, half)
    return float(np.sum((g.ravel()[keep] - samples) ** 2))


def fit_beam(psf, delta_arcsec, npix_window=(9, 9), sampling=(9, 9), cutoff=0.35):
    """psf (l, m, time, chan, pol) -> (time, chan, pol, 3): major, minor FWHM
    (arcsec) and position angle (degrees)."""
    from scipy import optimize
    from scipy.interpolate import interpn
    psf = np.asarray(psf, dtype=np.float64)
    win = np.asarray(npix_window, dtype=int)
    smp = np.asarray(sampling, dtype=int)
    step = np.abs(np.asarray(delta_arcsec, dtype=np.float64))
    centre = np.array(psf.shape[:2]) // 2
    lo, hi = centre - win // 2, centre + win // 2 + 1
    box = psf[lo[0]:hi[0], lo[1]:hi[1]]
    ax0 = np.arange(win[0]) * step[0]
    ax1 = np.arange(win[1]) * step[1]
    s0 = np.linspace(0, win[0] - 1, smp[0]) * step[0]
    s1 = np.linspace(0, win[1] - 1, smp[1]) * step[1]
    # sample points in the order (s0 slow... as a (smp1, smp0) array transposed back)
    pts = np.stack([np.repeat(s0, len(s1)), np.tile(s1, len(s0))], axis=1)
    half = smp // 2
    out = np.zeros(psf.shape[2:] + (3,))
    for idx in np.ndindex(*psf.shape[2:]):
        plane = box[(slice(None), slice(None)) + idx]
        vals = interpn((ax0, ax1), plane, pts, method='splinef2d').reshape(smp[1], smp[0]).T
        vals = np.where(vals < cutoff, np.nan, vals).ravel()
        keep = ~np.isnan(vals)
        res = optimize.minimize(_chi2, [2.5, 2.5, 0.0], args=(vals[keep], keep, half))
        sx, sy, rot = res.x
        phi = rot - 90.0
        if phi < -90.0:
            phi += 180.0
        scale = np.array([smp[0] / win[0], smp[1] / win[1]])
        out[idx] = (max(abs(sx), abs(sy)) * step[0] * 2.355 / scale[0],
                    min(abs(sx), abs(sy)) * step[1] * 2.355 / scale[1], -phi)
    return out


class LazyBeamFit:
    """PSF_FIT as the reference returns it: a lazy array (its dask graph runs
    the fit only when the values are asked for). The fit runs on the first
    np.asarray / .compute() and is cached; shape (time, chan, pol, 3)."""

    def __init__(self, psf, delta_arcsec, npix_window=(9, 9), sampling=(9, 9), cutoff=0.35):
        self._psf = psf
        self._args = (delta_arcsec, npix_window, sampling, cutoff)
        self._value = None
        self.shape = tuple(psf.shape[2:]) + (3,)
        self.dtype = np.dtype(np.float64)
        self.ndim = len(self.shape)

    def compute(self):
        if self._value is None:
            self._value = fit_beam(self._psf, *self._args)
        return self._value

    def __array__(self, dtype=None, copy=None):
        v = self.compute()
        return v if dtype is None else v.astype(dtype)

    def __repr__(self):
        state = 'computed' if self._value is not None else 'not computed'
        return f'<LazyBeamFit {self.shape} ({state})>'
