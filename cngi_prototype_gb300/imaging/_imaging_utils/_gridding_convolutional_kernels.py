"""Prolate-spheroidal gridding kernel and its grid-correction function.

Same role and signatures as the reference's
ngcasa/imaging/_imaging_utils/_gridding_convolutional_kernels.py
(_prolate_spheroidal_function :101-148, _create_prolate_spheroidal_kernel
:35-98, _create_prolate_spheroidal_kernel_1D :151-158). The function is
Schwab's rational approximation of the M=6, alpha=1 spheroidal function
(F. Schwab, "Optimal gridding of visibility data in radio interferometry",
1984): two pieces split at |nu| = 0.75, each a degree-4 numerator over a
degree-2 denominator in (nu^2 - nu_end^2). The published coefficient table is
necessarily identical to the reference's.
"""
import numpy as np

# Schwab's coefficients: rows = piece (|nu| < 0.75, 0.75 <= |nu| <= 1)
_NUM = ((8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1),
        (4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2))
_DEN = ((1.0000000e0, 8.212018e-1, 2.078043e-1),
        (1.0000000e0, 9.599102e-1, 2.918724e-1))
_NU_END = (0.75, 1.0)


def _prolate_spheroidal_function(u):
    """Return (grdsf(u), (1-u^2)*grdsf(u)); both 0 for |u| > 1."""
    nu = np.abs(np.asarray(u, dtype=np.float64))
    grdsf = np.zeros(nu.shape, dtype=np.float64)
    for piece, (lo, hi) in enumerate(((0.0, 0.75), (0.75, 1.0))):
        sel = (nu >= lo) & ((nu < hi) if piece == 0 else (nu <= hi))
        if not np.any(sel):
            continue
        d = nu[sel] ** 2 - _NU_END[piece] ** 2
        num = np.zeros(d.shape)
        for k, c in enumerate(_NUM[piece]):
            num = num + c * d ** k
        den = np.zeros(d.shape)
        for k, c in enumerate(_DEN[piece]):
            den = den + c * d ** k
        val = np.where(den > 0.0, num / np.where(den > 0.0, den, 1.0), 0.0)
        grdsf[sel] = val
    grdsf[nu > 1.0] = 0.0
    return grdsf, (1.0 - nu ** 2) * grdsf


def _create_prolate_spheroidal_kernel_1D(oversampling, support):
    """Oversampled half kernel, length oversampling*(support//2+1); the last
    `oversampling` entries (|nu| >= 1) are zero."""
    half = support // 2
    n = oversampling * half
    table = np.zeros(oversampling * (half + 1))
    table[:n] = _prolate_spheroidal_function(np.arange(n) / float(n))[1]
    return table


def _grid_correction_1d(n):
    x = np.abs(2.0 * (np.arange(n) - n // 2) / n)
    return _prolate_spheroidal_function(x)[0]


def _create_prolate_spheroidal_kernel(oversampling, support, n_uv):
    """Return (None, correction image over the padded grid).

    The reference also builds a 4-D oversampled kernel here that no caller
    uses (the gridders take the 1-D table); it is not built.
    """
    return None, np.outer(_grid_correction_1d(int(n_uv[0])), _grid_correction_1d(int(n_uv[1])))


def _create_prolate_spheroidal_image_2D(n_xy):
    return np.outer(_grid_correction_1d(int(n_xy[0])), _grid_correction_1d(int(n_xy[1])))
