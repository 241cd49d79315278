"""Hogbom minor cycle: the oracle against the reference's own _clean_jit
(tests/golden/clean.npz, made by make_golden.py clean), and the documented
algorithm on a clean point source."""
import numpy as np
import pytest

from conftest import load_golden


@pytest.mark.parametrize('gain,thr,niter', [(0.1, 0.05, 60), (0.3, 0.0, 25)])
def test_oracle_matches_reference_as_written(gain, thr, niter):
    from oracle import clean as O
    d = load_golden('clean')
    m, r = O.clean(d['dirty'], d['psf'], gain, thr, niter, scale_by_peak=False)
    assert np.array_equal(m, d[f'model_g{gain}_n{niter}'])
    assert np.array_equal(r, d[f'residual_g{gain}_n{niter}'])


def test_oracle_hogbom_recovers_a_point_source():
    from oracle import clean as O
    n = 32
    x = np.arange(2 * n)[:, None] - n
    y = np.arange(2 * n)[None, :] - n
    psf = np.exp(-(x ** 2 + y ** 2) / 6.0)
    dirty = 1.7 * psf[n - 10:2 * n - 10, n - 20:2 * n - 20]   # source at (10, 20), peak 1.7
    m, r = O.clean(dirty[:, :, None, None, None], psf[:, :, None, None, None], 0.2, 1e-4, 200, True)
    assert abs(m[10, 20, 0, 0, 0] - 1.7) < 1e-3 and np.count_nonzero(m) == 1
    assert np.abs(r).max() < 1e-3
