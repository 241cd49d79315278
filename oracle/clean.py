"""Oracle (test infrastructure only): CPU restatement of the Hogbom CLEAN
minor cycle, ngcasa/deconvolution/deconvolve_point_clean.py _clean_jit
(:174-236) with _abs_image_peaks (:303-320).

scale_by_peak=False is the reference's code as written (it subtracts
gain*psf, :216); scale_by_peak=True is Hogbom's algorithm as documented
(subtract gain*peak*psf). The window subtraction is elementwise numpy (one
rounding for gain*psf, one for the difference), the arithmetic of the
reference's loops.
"""
import numpy as np


def _peak(plane):
    """First pixel (row-major) of largest |value| > 0, NaN never; None when none."""
    a = np.abs(plane)
    a = np.where(np.isnan(a), -1.0, a)
    i = int(np.argmax(a))
    if not a.flat[i] > 0.0:
        return None
    return np.unravel_index(i, plane.shape)


def clean_plane(residual, model, psf, gain, threshold, n_iter, scale_by_peak=True):
    """In place on one (nx, ny) plane; returns the number of subtractions."""
    pc = np.array(psf.shape) // 2
    nx, ny = residual.shape
    pos = _peak(residual)
    if pos is None:
        return 0
    peak = residual[pos]
    thr = threshold * abs(peak)
    i = 0
    while abs(peak) > thr and i < n_iter:
        model[pos] += gain * peak
        s = gain * peak if scale_by_peak else gain
        sx, ex = max(pos[0] - pc[0], 0), min(pos[0] + (psf.shape[0] - pc[0]), nx)
        sy, ey = max(pos[1] - pc[1], 0), min(pos[1] + (psf.shape[1] - pc[1]), ny)
        psx, psy = pc[0] + sx - pos[0], pc[1] + sy - pos[1]
        residual[sx:ex, sy:ey] -= s * psf[psx:psx + (ex - sx), psy:psy + (ey - sy)]
        i += 1
        pos = _peak(residual)
        if pos is None:
            break
        peak = residual[pos]
    return i


def clean(dirty, psf, gain, threshold, n_iter, scale_by_peak=True):
    """dirty (l, m, time, chan, pol), psf (l', m', time, chan, pol) -> (model, residual)."""
    residual = np.array(dirty, dtype=np.float64, copy=True)
    model = np.zeros_like(residual)
    for t in range(residual.shape[2]):
        for c in range(residual.shape[3]):
            for p in range(residual.shape[4]):
                r = np.ascontiguousarray(residual[:, :, t, c, p])
                m = np.zeros_like(r)
                clean_plane(r, m, np.asarray(psf[:, :, t, c, p], dtype=np.float64), gain, threshold, n_iter,
                            scale_by_peak)
                residual[:, :, t, c, p] = r
                model[:, :, t, c, p] = m
    return model, residual
