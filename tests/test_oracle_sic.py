"""The oracle restates the path of synthesis_imaging_cube
(ngcasa/imaging/synthesis_imaging_cube.py:170-308) and reproduces the
reference's own outputs in tests/golden/sic.npz (made by make_golden.py sic):
flags to NaN, natural and Briggs 0.5 weights, PSF, image, sums of weights and
the primary beams of two dish types."""
import numpy as np

from conftest import load_golden
from oracle import imaging as O
from oracle import mosaic as M


def _gp(d):
    gp = {'image_size': [int(x) for x in d['image_size']], 'cell_size': [float(x) for x in d['cell_arcsec']],
          'chan_mode': 'cube'}
    O.check_grid_parms(gp)
    return gp


def _close(a, b, tol=1e-12):
    return np.abs(a - b).max() <= tol * np.abs(b).max()


def test_oracle_natural_chunk_matches_reference():
    d = load_golden('sic')
    gp = _gp(d)
    vis = d['vis'].copy()
    vis[d['flag'] == 1] = np.nan            # synthesis_imaging_cube.py:180 (weights stay)
    img, isw = O.make_image_arrays(vis, d['uvw'], d['weight'], d['freq'], gp)
    psf, psw = O.make_image_arrays(None, d['uvw'], d['weight'], d['freq'], gp, do_psf=True)
    assert _close(img, d['natural_image'])
    assert _close(psf, d['natural_psf'])
    assert np.allclose(isw, d['natural_image_sum_weight'], rtol=1e-13)
    assert np.allclose(psw, d['natural_psf_sum_weight'], rtol=1e-13)


def test_oracle_briggs_chunk_matches_reference():
    d = load_golden('sic')
    gp = _gp(d)
    iw = O.make_imaging_weight(d['uvw'], d['weight'], d['freq'], gp, {'weighting': 'briggs', 'robust': 0.5})
    ref = d['briggs_imaging_weight']
    assert np.array_equal(np.isnan(iw), np.isnan(ref))
    fin = ~np.isnan(ref)
    assert np.allclose(iw[fin], ref[fin], rtol=1e-13, atol=0)
    vis = d['vis'].copy()
    vis[d['flag'] == 1] = np.nan
    img, isw = O.make_image_arrays(vis, d['uvw'], iw, d['freq'], gp)
    psf, psw = O.make_image_arrays(None, d['uvw'], iw, d['freq'], gp, do_psf=True)
    assert _close(img, d['briggs_image'])
    assert _close(psf, d['briggs_psf'])
    assert np.allclose(isw, d['briggs_image_sum_weight'], rtol=1e-13)
    assert np.allclose(psw, d['briggs_psf_sum_weight'], rtol=1e-13)


def test_oracle_primary_beams_match_reference():
    d = load_golden('sic')
    gp = _gp(d)
    pb = M.airy_patterns('casa_airy', d['freq'], 2, d['dish'], d['blockage'], 2, gp['cell_size'], gp['image_size'],
                         np.asarray(gp['image_size']) // 2)
    pb = np.moveaxis(pb, (0, 1, 2), (4, 2, 3))          # (type, freq, pol, l, m) -> (l, m, freq, pol, type)
    assert pb.shape == d['natural_pb'].shape
    assert np.array_equal(pb, d['natural_pb'])


def test_beam_fit_of_the_psf_matches_reference():
    """RESTORE_PARMS: casa_fit of the PSF with delta = the cell size in radians."""
    from cngi_prototype_gb300.imaging._imaging_utils._beam_fit import fit_beam
    d = load_golden('sic')
    gp = _gp(d)
    got = fit_beam(d['natural_psf'][:, :, None, :, :], gp['cell_size'])[0]
    assert np.allclose(got, d['natural_restore_parms'], rtol=1e-9, atol=1e-12)
