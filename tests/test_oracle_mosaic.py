"""The mosaic oracle is pinned to reference-generated golden vectors
(bit-exact), and the product's host-side GCF logic agrees with it."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import imaging as O
from oracle import mosaic as M


def _gp(d):
    gp = {'image_size': [int(x) for x in d['image_size']], 'cell_size': [float(x) for x in d['cell_arcsec']],
          'chan_mode': 'cube', 'fft_padding': 1.2}
    O.check_grid_parms(gp)
    return gp


@pytest.fixture(scope='module')
def gold():
    return load_golden('mosaic')


def test_gcf_generation_matches_reference(gold):
    d = gold
    gp = _gp(d)
    cfb, pairs = M.create_cf_baseline_map(np.zeros(6, int), np.stack([d['antenna1'], d['antenna2']], 1), 1)
    cfc, pbf = M.create_cf_chan_map(d['freq'], 0.005)
    assert np.array_equal(cfb, d['cf_baseline_map']) and np.array_equal(cfc, d['cf_chan_map'])
    assert np.array_equal(pbf, d['pb_freq'])
    bp = M.baseline_patterns('casa_airy', pbf, pairs, [12.0], [0.75], 1, gp, d['oversampling'])
    bw = M.baseline_patterns('casa_airy', pbf, pairs, [12.0], [0.75], 2, gp, d['oversampling'])
    assert np.array_equal(bp, d['baseline_pb']) and np.array_equal(bw, d['weight_baseline_pb'])
    ck, wk, sup = M.resize_and_calc_support(M.pattern_to_kernel(bp), M.pattern_to_kernel(bw), d['oversampling'],
                                            d['max_support'], 0.025, gp['image_size_padded'])
    assert np.array_equal(ck, d['conv_kernel']) and np.array_equal(wk, d['weight_conv_kernel'])
    assert np.array_equal(sup, d['support'])


@pytest.mark.parametrize('tag', ['grid', 'psf_grid', 'weight_grid'])
def test_aperture_gridders_match_reference(gold, tag):
    d = gold
    gp = _gp(d)
    kern = d['weight_conv_kernel'] if tag == 'weight_grid' else d['conv_kernel']
    g, sw = M.aperture_grid(d['vis'], d['uvw'], d['imaging_weight'], d['field'], np.arange(2), d['cf_baseline_map'],
                            d['cf_chan_map'], d['cf_pol_map'], kern, d['support'], d['phase_gradient'], d['freq'],
                            gp['image_size_padded'], gp['cell_size'], d['oversampling'],
                            do_psf=tag == 'psf_grid', weight_grid=tag == 'weight_grid')
    swk = {'grid': 'sum_weight', 'psf_grid': 'psf_sum_weight', 'weight_grid': 'weight_sum_weight'}[tag]
    assert np.array_equal(g, d[tag]) and np.array_equal(sw, d[swk])


def test_phase_gradient_restatement(gold):
    """The golden phase gradient was made by the fixture script's own SIN
    restatement (astropy is not available), so this is a self-consistency
    check of the oracle's copy, plus the projection's known answers."""
    d = gold
    gp = _gp(d)
    sl = M.phase_slopes(d['field_phase_dir'], d['phase_center'], gp['image_size_padded'], gp['cell_size'],
                        d['oversampling'])
    assert np.array_equal(M.phase_gradient(sl, d['conv_kernel'].shape[-2:]), d['phase_gradient'])
    # the phase centre itself projects to pixel offset 0; a pure declination
    # offset dd projects to sin(dd) / cell along m
    pc = d['phase_center']
    off = M.sin_pixel_offsets(np.array([[pc[0], pc[1]], [pc[0], pc[1] + 1e-4]]), pc, gp['cell_size'])
    assert np.allclose(off[0], 0.0, atol=1e-12)
    assert np.isclose(off[1, 1], np.sin(1e-4) / gp['cell_size'][1], rtol=1e-12)


def test_sin_projection_known_answer():
    """The reference's recorded CASA toPixelWCS case
    (make_gridding_convolution_function.py:569-581): crpix 120, cdelt
    (-5e-5, 5e-5) deg, crval (180.4684619, -18.8638732472) deg."""
    pc = np.deg2rad([180.46846189999996568, -18.863873247222226581])
    world = np.deg2rad([[-179.5337374791666889, -18.863873258333338612]])
    off = M.sin_pixel_offsets(world, pc, np.deg2rad([-5e-05, 5e-05]))
    assert np.allclose(120 + off[0], [161.6249842951184803, 119.99951947142589859], rtol=0, atol=1e-9)


def test_product_host_logic_matches_oracle(gold):
    import importlib
    G = importlib.import_module('cngi_prototype_gb300.imaging.make_gridding_convolution_function')
    from cngi_prototype_gb300.imaging._imaging_utils import _mosaic
    from cngi_prototype_gb300 import xds
    d = gold
    gp = _gp(d)
    rng = np.random.default_rng(5)
    uai = rng.integers(0, 3, 10)
    ba = np.stack(np.triu_indices(10, 1), 1)
    for a, b in zip(G.create_cf_baseline_map(uai, ba, 3), M.create_cf_baseline_map(uai, ba, 3)):
        assert np.array_equal(a, b)
    for f in (d['freq'], np.linspace(1e9, 2e9, 64), np.array([1.4e9])):
        for a, b in zip(G.create_cf_chan_map(f, 0.005), M.create_cf_chan_map(f, 0.005)):
            assert np.array_equal(a, b)
    wk = M.pattern_to_kernel(d['weight_baseline_pb'])
    npad = gp['image_size_padded']
    for q in range(wk.shape[1]):
        k = wk[0, q, 0]
        got = G.calc_conv_size(k[:, npad[1] // 2], k[npad[0] // 2, :], np.abs(k).min(), np.abs(k).max(), npad,
                               0.025, d['oversampling'], d['max_support'])
        assert got == M.calc_conv_size(k, npad, 0.025, d['oversampling'], d['max_support'])
    assert np.array_equal(G.sin_pixel_offsets(d['field_phase_dir'], d['phase_center'], gp['cell_size']),
                          M.sin_pixel_offsets(d['field_phase_dir'], d['phase_center'], gp['cell_size']))
    # the gridder's separable slopes recovered from a PHASE_GRADIENT table
    sl = M.phase_slopes(d['field_phase_dir'], d['phase_center'], npad, gp['cell_size'], d['oversampling'])
    ds = xds.Dataset({'PHASE_GRADIENT': (('field_id', 'u', 'v'), d['phase_gradient'])})
    assert np.allclose(_mosaic.phase_slopes(ds), sl, rtol=1e-12, atol=1e-15)
    f = np.array([[3, 3, -1], [7, 3, 7]])
    assert np.array_equal(_mosaic.field_indices(f, [7, 3]), [[1, 1, -1], [0, 1, 0]])
    with pytest.raises(ValueError):
        _mosaic.field_indices(f, [3])


@pytest.mark.parametrize('tag', ['grid', 'psf_grid', 'weight_grid'])
def test_c_aperture_oracle_matches_reference(gold, tag):
    from oracle import cbind
    d = gold
    gp = _gp(d)
    kind = {'grid': 'data', 'psf_grid': 'psf', 'weight_grid': 'weight'}[tag]
    kern = d['weight_conv_kernel'] if tag == 'weight_grid' else d['conv_kernel']
    fidx = np.where(d['field'] >= 0, d['field'], -1)
    g, sw = cbind.aperture_grid(kind, d['vis'], d['uvw'], d['imaging_weight'], fidx, d['cf_baseline_map'],
                                d['cf_chan_map'], d['cf_pol_map'], kern, d['support'], d['phase_gradient'], d['freq'],
                                d['oversampling'], gp['image_size_padded'], gp['cell_size'])
    swk = {'grid': 'sum_weight', 'psf_grid': 'psf_sum_weight', 'weight_grid': 'weight_sum_weight'}[tag]
    assert np.array_equal(g, d[tag]) and np.array_equal(sw, d[swk])
    gc, swc = cbind.aperture_grid(kind, d['vis'], d['uvw'], d['imaging_weight'], fidx, d['cf_baseline_map'],
                                  d['cf_chan_map'], d['cf_pol_map'], kern, d['support'], d['phase_gradient'],
                                  d['freq'], d['oversampling'], gp['image_size_padded'], gp['cell_size'],
                                  chan_mode='continuum')
    gn, swn = M.aperture_grid(d['vis'], d['uvw'], d['imaging_weight'], d['field'], np.arange(2), d['cf_baseline_map'],
                              d['cf_chan_map'], d['cf_pol_map'], kern, d['support'], d['phase_gradient'], d['freq'],
                              gp['image_size_padded'], gp['cell_size'], d['oversampling'], 'continuum',
                              do_psf=kind == 'psf', weight_grid=kind == 'weight')
    assert np.array_equal(gc, gn) and np.array_equal(swc, swn)


def test_mlp_oracle_gradient_and_product_layout():
    """The network oracle's backward against central differences, and the
    product's initial parameters in the oracle's layout."""
    from oracle import mlp as OM
    from cngi_prototype_gb300.imaging.learned_gcf import init_params
    rng = np.random.default_rng(2)
    p = OM.init_params(1).astype(np.float64)
    z = rng.uniform(-1, 1, (64, 3))
    t = rng.standard_normal(64)
    L, g = OM.loss_grad(p, z, t)
    for i in rng.choice(OM.N_TRAINED, 40, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (OM.loss_grad(p + e, z, t)[0] - OM.loss_grad(p - e, z, t)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])
    q = init_params(0)
    assert q.size == OM.NPARAM and q.dtype == np.float32
    parts = OM.unpack(q)
    assert np.all(parts[1] == 0) and np.all(parts[9] == 0)
    assert np.all(parts[10][:30, 3] == 0) and np.all(parts[10][30:, :3] == 0)
