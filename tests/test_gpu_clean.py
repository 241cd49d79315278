"""Hogbom minor cycle on the GPU: bit-identical to the reference's _clean_jit
(as written) and to the oracle's Hogbom algorithm (FP64, one rounding per
operation as the reference's loops)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('gain,thr,niter', [(0.1, 0.05, 60), (0.3, 0.0, 25)])
def test_matches_reference_as_written(ngg, gain, thr, niter):
    d = load_golden('clean')
    m, r, its = ngg.hogbom_clean(d['dirty'], d['psf'], gain, thr, niter, scale_by_peak=False)
    assert np.array_equal(m.cpu().numpy(), d[f'model_g{gain}_n{niter}'])
    assert np.array_equal(r.cpu().numpy(), d[f'residual_g{gain}_n{niter}'])


def test_hogbom_matches_oracle_on_many_planes(ngg):
    from oracle import clean as O
    rng = np.random.default_rng(21)
    nx, ny, C, P = 96, 80, 3, 2
    x = np.arange(2 * nx)[:, None] - nx
    y = np.arange(2 * ny)[None, :] - ny
    base = np.exp(-(x ** 2 + y ** 2) / 10.0) * (1 + 0.1 * np.cos(0.5 * x))
    psf = np.repeat(np.repeat(base[:, :, None, None, None], C, axis=3), P, axis=4)
    dirty = 0.02 * rng.standard_normal((nx, ny, 1, C, P))
    for c in range(C):
        for p in range(P):
            for _ in range(6):
                sx, sy = rng.integers(0, nx), rng.integers(0, ny)
                dirty[:, :, 0, c, p] += rng.uniform(0.2, 3.0) * base[nx - sx:2 * nx - sx, ny - sy:2 * ny - sy]
    dirty[5, 7, 0, 1, 0] = np.nan   # NaN pixels are never a peak and are carried through
    for scale in (True, False):
        m_ref, r_ref = O.clean(dirty, psf, 0.15, 0.01, 400, scale)
        m, r, its = ngg.hogbom_clean(dirty, psf, 0.15, 0.01, 400, scale_by_peak=scale)
        assert np.array_equal(m.cpu().numpy(), m_ref)
        assert np.array_equal(r.cpu().numpy(), r_ref, equal_nan=True)
        assert int(its.max()) <= 400


def test_api_adds_model_and_residual(ngg):
    from cngi_prototype_gb300 import xds
    from cngi_prototype_gb300.deconvolution import deconvolve_point_clean
    d = load_golden('clean')
    img = xds.Dataset({'IMAGE': (('l', 'm', 'time', 'chan', 'pol'), d['dirty']),
                       'PSF': (('l2', 'm2', 'time', 'chan', 'pol'), d['psf'])})
    out = deconvolve_point_clean(img, {'gain': 0.1, 'threshold': 0.05, 'n_iter': 60, 'psf_scaling': 'none'},
                                 {'data_group_in': {'image': 'IMAGE', 'psf': 'PSF'}})
    assert 'MODEL' in out and 'RESIDUAL' in out and 'MODEL' not in img
    assert np.array_equal(out['RESIDUAL'].values, d['residual_g0.1_n60'])
    assert np.array_equal(out['MODEL'].values, d['model_g0.1_n60'])
