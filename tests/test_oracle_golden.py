"""The oracle is pinned to reference-generated golden vectors (bit-exact)."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import cbind
from oracle import imaging as O

CASES = ['std_cube', 'std_odd', 'std_onepol', 'std_continuum']


def _gp(d):
    gp = {'image_size': list(d['image_size']), 'cell_size': list(d['cell_arcsec']), 'chan_mode': str(d['chan_mode'])}
    O.check_grid_parms(gp)
    return gp


@pytest.mark.parametrize('name', CASES)
def test_numpy_oracle_matches_reference(name):
    d = load_golden(name)
    gp = _gp(d)
    cm = gp['chan_mode']
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    npad = gp['image_size_padded']
    assert np.array_equal(npad, d['image_size_padded'])
    assert np.array_equal(gp['cell_size'], d['cell_rad'])
    g, sw = O.standard_grid(d['vis'], d['uvw'], d['weight'], d['freq'], cgk, npad, gp['cell_size'], 7, 100,
                            False, False, True, cm)
    assert np.array_equal(g, d['grid']) and np.array_equal(sw, d['sum_weight'])
    pg, psw = O.standard_grid(None, d['uvw'], d['weight'], d['freq'], cgk, npad, gp['cell_size'], 7, 100,
                              True, False, False, cm)
    assert np.array_equal(pg, d['psf_grid']) and np.array_equal(psw, d['psf_sum_weight'])
    dg, dsw = O.grid_weight_density(d['uvw'], d['weight'], d['freq'], gp)
    assert np.array_equal(dg, d['density']) and np.array_equal(dsw, d['density_sum_weight'])
    if cm == 'cube':
        for tag in ['briggs_+0.5', 'uniform_+0.0', 'briggs_-1.3']:
            w, r = tag.split('_')
            dens = np.moveaxis(dg, (0, 1), (2, 3))
            bf = O.calculate_briggs_parms(dens, dsw, {'weighting': w, 'robust': float(r)})
            assert np.array_equal(bf, d['briggs_factors_' + tag])
            iw = O.standard_imaging_weight_degrid(dens, d['uvw'], d['weight'], bf, d['freq'], gp['image_size'],
                                                  gp['cell_size'])
            assert np.array_equal(iw, d['imaging_weight_' + tag])
        img, isw = O.make_image_arrays(d['vis'], d['uvw'], d['weight'], d['freq'], gp)
        assert np.array_equal(img, d['image']) and np.array_equal(isw, d['image_sum_weight'])
        psf, _ = O.make_image_arrays(None, d['uvw'], d['weight'], d['freq'], gp, do_psf=True)
        assert np.array_equal(psf, d['psf'])


@pytest.mark.parametrize('name', CASES)
def test_c_oracle_matches_reference(name):
    d = load_golden(name)
    gp = _gp(d)
    cm = gp['chan_mode']
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    npad = gp['image_size_padded']
    nt = 1 if cm == 'continuum' else 0   # one chunk: the reference's summation order
    g, sw = cbind.grid('data', d['vis'], d['uvw'], d['weight'], d['freq'], cgk, 7, 100, npad, gp['cell_size'], cm, nt)
    assert np.array_equal(g, d['grid']) and np.array_equal(sw, d['sum_weight'])
    pg, psw = cbind.grid('psf', None, d['uvw'], d['weight'], d['freq'], cgk, 7, 100, npad, gp['cell_size'], cm, nt)
    assert np.array_equal(pg, d['psf_grid']) and np.array_equal(psw, d['psf_sum_weight'])
    dg, dsw = cbind.grid('density', None, d['uvw'], d['weight'], d['freq'], np.ones(1), 1, 0, gp['image_size'],
                         gp['cell_size'], cm, nt)
    assert np.array_equal(dg, d['density']) and np.array_equal(dsw, d['density_sum_weight'])
    if cm == 'cube':
        bf = d['briggs_factors_briggs_+0.5']
        iw = cbind.weight_degrid(np.moveaxis(d['density'], (0, 1), (2, 3)), d['uvw'], d['weight'], bf, d['freq'],
                                 gp['image_size'], gp['cell_size'])
        assert np.array_equal(iw, d['imaging_weight_briggs_+0.5'])


def test_ps_kernel_known_answers():
    k = load_golden('ps_kernel')
    assert np.array_equal(O.create_prolate_spheroidal_kernel_1D(100, 7), k['cgk_1D'])
    assert np.array_equal(O.create_prolate_spheroidal_correction([128, 128]), k['corr128'])
    assert np.array_equal(O.create_prolate_spheroidal_correction([75, 77]), k['corr75x77'])
    assert abs(k['cgk_1D'][0] - 0.99999967) < 1e-8 and np.all(k['cgk_1D'][300:] == 0)
    assert abs(k['corr128'][64, 64] - 0.99999933) < 1e-8


def test_c_oracle_continuum_tree_sum_close_to_single_chunk():
    d = load_golden('std_continuum')
    gp = _gp(d)
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    g1, s1 = cbind.grid('data', d['vis'], d['uvw'], d['weight'], d['freq'], cgk, 7, 100, gp['image_size_padded'],
                        gp['cell_size'], 'continuum', 1)
    g4, s4 = cbind.grid('data', d['vis'], d['uvw'], d['weight'], d['freq'], cgk, 7, 100, gp['image_size_padded'],
                        gp['cell_size'], 'continuum', 4)
    assert np.abs(g1 - g4).max() <= 1e-12 * np.abs(g1).max()
    assert np.allclose(s1, s4, rtol=1e-13)


def test_empty_inputs():
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    g, sw = O.standard_grid(np.zeros((0, 3, 2, 2), np.complex64), np.zeros((0, 3, 3)), np.zeros((0, 3, 2, 2)),
                            np.array([1e9, 1.1e9]), cgk, np.array([40, 40]), [-1e-4, 1e-4], 7, 100, False)
    assert g.shape == (2, 2, 40, 40) and not g.any() and not sw.any()
    g2, sw2 = cbind.grid('data', np.zeros((0, 3, 2, 2), np.complex64), np.zeros((0, 3, 3)), np.zeros((0, 3, 2, 2)),
                         np.array([1e9, 1.1e9]), cgk, 7, 100, [40, 40], [-1e-4, 1e-4])
    assert not g2.any() and not sw2.any()


def test_beam_fit_matches_reference():
    """PSF beam fit (make_psf's PSF_FIT) against the reference's casa_fit
    (tests/golden/beam.npz): the same scipy spline and optimiser calls on the
    same objective, bit-identical."""
    from cngi_prototype_gb300.imaging._imaging_utils._beam_fit import LazyBeamFit, fit_beam
    d = load_golden('beam')
    assert np.array_equal(fit_beam(d['psf'], d['delta']), d['ellipse_parms'])
    lazy = LazyBeamFit(d['psf'], d['delta'])
    assert lazy.shape == d['ellipse_parms'].shape and 'not computed' in repr(lazy)
    assert np.array_equal(np.asarray(lazy), d['ellipse_parms'])
