"""Mosaic (GCF-table) gridding, weight grid, GCF generation and the mosaic
imaging API on the GPU against the reference's golden outputs and the oracle."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import imaging as O
from oracle import mosaic as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def gold():
    return load_golden('mosaic')


def _gp(d, chan_mode='cube'):
    gp = {'image_size': [int(x) for x in d['image_size']], 'cell_size': [float(x) for x in d['cell_arcsec']],
          'chan_mode': chan_mode, 'fft_padding': 1.2}
    O.check_grid_parms(gp)
    return gp


def _peak_err(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _grid(ngg, d, kind, table, support, phase_slope, fidx, freq=None, chan_mode='cube', layout='natural', vis=None,
          uvw=None, iw=None, cfb=None, cfc=None):
    gp = _gp(d, chan_mode)
    args = (d['uvw'] if uvw is None else uvw, (d['imaging_weight'] if iw is None else iw).astype(np.float32),
            d['freq'] if freq is None else freq, fidx, d['cf_baseline_map'] if cfb is None else cfb,
            d['cf_chan_map'] if cfc is None else cfc, d['cf_pol_map'], table, support, phase_slope)
    if kind == 'weight':
        g, sw = ngg.grid_gcf_weight(*args, gp['image_size_padded'], gp['cell_size'], d['oversampling'],
                                    chan_mode=chan_mode, layout=layout)
    else:
        g, sw = ngg.grid_gcf(d['vis'] if vis is None else vis, *args, gp['image_size_padded'], gp['cell_size'],
                             d['oversampling'], mode=kind, chan_mode=chan_mode, layout=layout)
    return g.cpu().numpy(), sw.cpu().numpy()


def _slopes(d):
    gp = _gp(d)
    return M.phase_slopes(d['field_phase_dir'], d['phase_center'], gp['image_size_padded'], gp['cell_size'],
                          d['oversampling'])


@pytest.mark.parametrize('kind,tag,swk', [('data', 'grid', 'sum_weight'), ('psf', 'psf_grid', 'psf_sum_weight'),
                                          ('weight', 'weight_grid', 'weight_sum_weight')])
def test_gcf_gridders_match_reference(ngg, gold, kind, tag, swk):
    d = gold
    table = d['weight_conv_kernel'] if kind == 'weight' else d['conv_kernel']
    fidx = np.where(d['field'] >= 0, d['field'], -1)
    g, sw = _grid(ngg, d, kind, table, d['support'], _slopes(d), fidx)
    assert _peak_err(g, d[tag]) < 2e-6
    assert np.allclose(sw, d[swk], rtol=1e-6)
    # FFT-ordered planes are the ifftshift of the natural ones (up to the
    # order in which the atomic adds of different warps land)
    gf, swf = _grid(ngg, d, kind, table, d['support'], _slopes(d), fidx, layout='fft')
    assert _peak_err(gf, np.fft.ifftshift(g, axes=(2, 3))) < 1e-6
    assert np.allclose(swf, sw, rtol=1e-12)


def test_gcf_gridder_continuum_and_edge_rows(ngg, gold):
    """Continuum accumulation; rows without a field, NaN uvw, NaN / zero
    data and rows whose footprint leaves the grid are skipped."""
    d = gold
    rng = np.random.default_rng(3)
    uvw = d['uvw'].copy()
    vis = d['vis'].copy()
    iw = d['imaging_weight'].copy()
    field = d['field'].copy()
    uvw[1, 2] = np.nan
    uvw[2, 3, :2] *= 40.0                   # far outside the grid
    vis[4, 5, 1, 0] = np.nan
    vis[5, 6, 2, 1] = 0.0
    iw[6, 7, 0, 0] = 0.0
    field[7, :] = -1
    iw = iw.astype(np.float32).astype(np.float64)
    gp = _gp(d, 'continuum')
    for kind in ('data', 'psf'):
        ref, rsw = M.aperture_grid(vis, uvw, iw, field, np.arange(2), d['cf_baseline_map'], d['cf_chan_map'],
                                   d['cf_pol_map'], d['conv_kernel'], d['support'], d['phase_gradient'], d['freq'],
                                   gp['image_size_padded'], gp['cell_size'], d['oversampling'], 'continuum',
                                   do_psf=kind == 'psf')
        fidx = np.where(field >= 0, field, -1)
        g, sw = _grid(ngg, d, kind, d['conv_kernel'], d['support'], _slopes(d), fidx, chan_mode='continuum',
                      vis=vis, uvw=uvw, iw=iw)
        assert g.shape == ref.shape
        assert _peak_err(g, ref) < 2e-6
        assert np.allclose(sw, rsw, rtol=1e-9)
    del rng


def _random_mosaic(seed, n_ant=12, T=48, C=4, P=2, N=96, n_field=3, types=2):
    from cngi_prototype_gb300 import simulate
    rng = np.random.default_rng(seed)
    enu = simulate.disk_layout(n_ant, 60.0, rng)
    uvw = simulate.earth_rotation_uvw(enu, T, 90.0)
    a1, a2 = simulate.baseline_pairs(n_ant)
    B = uvw.shape[1]
    freq = 230e9 + np.arange(C) * 2e9
    vis = (rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P))).astype(np.complex64)
    iw = rng.uniform(0.5, 2.0, (T, B, C, P)).astype(np.float32).astype(np.float64)
    field = np.repeat(rng.integers(0, n_field, T)[:, None], B, axis=1)
    gp = {'image_size': [N, N + 6], 'cell_size': [0.5, 0.5], 'chan_mode': 'cube', 'fft_padding': 1.25}
    O.check_grid_parms(gp)
    pc = np.array([np.deg2rad(80.0), np.deg2rad(-45.0)])
    fpd = pc + np.deg2rad(np.array([[0, 0], [4.0, 1.0], [-3.0, 5.0]])[:n_field] / 3600)
    os_ = np.array([8, 8])
    maxs = np.array([13, 13])
    uai = rng.integers(0, types, n_ant)
    cfb, pairs = M.create_cf_baseline_map(uai, np.stack([a1, a2], 1), types)
    cfc, pbf = M.create_cf_chan_map(freq, 0.005)
    dish, block = [12.0, 7.0][:types], [0.75, 0.75][:types]
    bp = M.baseline_patterns('casa_airy', pbf, pairs, dish, block, 1, gp, os_)
    bw = M.baseline_patterns('casa_airy', pbf, pairs, dish, block, 2, gp, os_)
    ck, wk, sup = M.resize_and_calc_support(M.pattern_to_kernel(bp), M.pattern_to_kernel(bw), os_, maxs, 0.025,
                                            gp['image_size_padded'])
    sl = M.phase_slopes(fpd, pc, gp['image_size_padded'], gp['cell_size'], os_)
    pg = M.phase_gradient(sl, ck.shape[-2:])
    return dict(vis=vis, uvw=uvw, imaging_weight=iw, field=field, freq=freq, gp=gp, os=os_, cfb=cfb, cfc=cfc,
                cfp=np.zeros(P, int), ck=ck, wk=wk, sup=sup, slopes=sl, pg=pg, a1=a1, a2=a2, uai=uai, pc=pc,
                fpd=fpd, dish=dish, block=block, maxs=maxs)


@pytest.mark.parametrize('seed', [11, 12])
def test_gcf_gridder_random_mosaic(ngg, seed):
    """Heterogeneous array (two dish types -> three CF pairs), three fields,
    a rectangular grid, 8x oversampling."""
    r = _random_mosaic(seed)
    gp = r['gp']
    for kind in ('data', 'psf', 'weight'):
        table = r['wk'] if kind == 'weight' else r['ck']
        ref, rsw = M.aperture_grid(r['vis'], r['uvw'], r['imaging_weight'], r['field'], np.arange(3), r['cfb'],
                                   r['cfc'], r['cfp'], table, r['sup'], r['pg'], r['freq'], gp['image_size_padded'],
                                   gp['cell_size'], r['os'], do_psf=kind == 'psf', weight_grid=kind == 'weight')
        args = (r['uvw'], r['imaging_weight'].astype(np.float32), r['freq'], r['field'].astype(np.int32), r['cfb'],
                r['cfc'], r['cfp'], table, r['sup'], r['slopes'])
        if kind == 'weight':
            g, sw = ngg.grid_gcf_weight(*args, gp['image_size_padded'], gp['cell_size'], r['os'])
        else:
            g, sw = ngg.grid_gcf(r['vis'], *args, gp['image_size_padded'], gp['cell_size'], r['os'], mode=kind)
        g = g.cpu().numpy()
        assert _peak_err(g, ref) < 2e-6, kind
        assert np.allclose(sw.cpu().numpy(), rsw, rtol=1e-6), kind


def test_gcf_kernels_match_oracle(ngg, gold):
    d = gold
    gp = _gp(d)
    npad = gp['image_size_padded']
    _, pairs = M.create_cf_baseline_map(np.zeros(6, int), np.stack([d['antenna1'], d['antenna2']], 1), 1)
    ck, wk = ngg.gcf_kernels('casa_airy', [12.0], [0.75], pairs, d['pb_freq'], npad,
                             np.asarray(gp['cell_size']) * d['oversampling'], npad // 2)
    ref_k = M.pattern_to_kernel(d['baseline_pb'])[:, :, 0]
    ref_w = M.pattern_to_kernel(d['weight_baseline_pb'])[:, :, 0]
    assert _peak_err(ck.cpu().numpy(), ref_k) < 1e-12
    assert _peak_err(wk.cpu().numpy(), ref_w) < 1e-12
    # the textbook obscured-aperture form and an unobscured dish
    for fn, block in (('airy', [0.75]), ('airy', [0.0]), ('casa_airy', [0.0])):
        bp = M.baseline_patterns(fn, d['pb_freq'], pairs, [12.0], block, 1, gp, d['oversampling'])
        ck, _ = ngg.gcf_kernels(fn, [12.0], block, pairs, d['pb_freq'], npad,
                                np.asarray(gp['cell_size']) * d['oversampling'], npad // 2)
        assert _peak_err(ck.cpu().numpy(), M.pattern_to_kernel(bp)[:, :, 0]) < 1e-12


def _mxds(r_or_d, golden=False):
    from cngi_prototype_gb300 import xds
    if golden:
        d = r_or_d
        vis = xds.vis_dataset(d['uvw'], d['vis'], d['imaging_weight'].astype(np.float32), d['freq'],
                              field_id=d['field'], antenna1=d['antenna1'], antenna2=d['antenna2'])
        fpd, fid = d['field_phase_dir'], np.arange(len(d['field_phase_dir']))
    else:
        r = r_or_d
        vis = xds.vis_dataset(r['uvw'], r['vis'], r['imaging_weight'].astype(np.float32), r['freq'],
                              field_id=r['field'], antenna1=r['a1'], antenna2=r['a2'])
        fpd, fid = r['fpd'], np.arange(len(r['fpd']))
    vis.attrs['data_groups'][0]['0']['imaging_weight'] = 'DATA_WEIGHT'
    field = xds.Dataset({'PHASE_DIR': (('field_id', 'poly_id', 'pair'), fpd[:, None, :])},
                        coords={'field_id': ('field_id', fid)})
    return xds.mxds({'xds0': vis}, FIELD=field)


def test_make_gridding_convolution_function_matches_reference(ngg, gold):
    from cngi_prototype_gb300.imaging import make_gridding_convolution_function
    d = gold
    gcf = make_gridding_convolution_function(
        _mxds(d, golden=True),
        {'function': 'casa_airy', 'list_dish_diameters': [12.0], 'list_blockage_diameters': [0.75],
         'unique_ant_indx': [0] * 6, 'oversampling': [4, 4], 'max_support': [15, 15], 'phase_center': d['phase_center']},
        {'image_size': [int(x) for x in d['image_size']], 'cell_size': [float(x) for x in d['cell_arcsec']],
         'fft_padding': 1.2}, {'xds': 'xds0'})
    assert np.array_equal(gcf['SUPPORT'].values, d['support'])
    assert np.array_equal(gcf['CF_BASELINE_MAP'].values, d['cf_baseline_map'])
    assert np.array_equal(gcf['CF_CHAN_MAP'].values, d['cf_chan_map'])
    assert _peak_err(gcf['CONV_KERNEL'].values, d['conv_kernel']) < 1e-11
    assert _peak_err(gcf['WEIGHT_CONV_KERNEL'].values, d['weight_conv_kernel']) < 1e-11
    assert np.abs(gcf['PHASE_GRADIENT'].values - d['phase_gradient']).max() < 1e-12
    assert np.array_equal(gcf.attrs['oversampling'], [4, 4])


def test_mosaic_api_matches_oracle(ngg):
    """make_gridding_convolution_function -> make_mosaic_pb ->
    make_image_with_gcf / make_psf_with_gcf against the oracle's chain
    (FP64 gridders, numpy FFTs, _normalize)."""
    from cngi_prototype_gb300 import xds
    from cngi_prototype_gb300.imaging import (make_gridding_convolution_function, make_image_with_gcf,
                                              make_mosaic_pb, make_psf_with_gcf)
    r = _random_mosaic(21, n_ant=10, T=32, C=3)
    mx = _mxds(r)
    gp_user = {'image_size': list(r['gp']['image_size']), 'cell_size': [0.5, 0.5], 'fft_padding': 1.25}
    gcf = make_gridding_convolution_function(
        mx, {'function': 'casa_airy', 'list_dish_diameters': r['dish'], 'list_blockage_diameters': r['block'],
             'unique_ant_indx': list(r['uai']), 'oversampling': list(r['os']), 'max_support': list(r['maxs']),
             'phase_center': r['pc']}, gp_user, {'xds': 'xds0'})
    assert np.array_equal(gcf['SUPPORT'].values, r['sup'])
    img = make_mosaic_pb(mx, gcf, xds.Dataset(), {'xds': 'xds0'}, {}, gp_user)
    gp = r['gp']
    npad, isz = gp['image_size_padded'], gp['image_size']
    args = (r['uvw'], r['imaging_weight'], r['field'], np.arange(3), r['cfb'], r['cfc'], r['cfp'])
    wg, wsw = M.aperture_grid(None, *args, r['wk'], r['sup'], r['pg'], r['freq'], npad, gp['cell_size'], r['os'],
                              weight_grid=True)
    pb_ref, wpb_ref = M.mosaic_pb(wg, wsw, isz)
    assert _peak_err(img['WEIGHT_PB'].values[:, :, 0], wpb_ref) < 1e-5
    assert _peak_err(img['PB'].values[:, :, 0], pb_ref) < 1e-5
    assert np.allclose(img['WEIGHT_PB_SUM_WEIGHT'].values[0], wsw, rtol=1e-6)
    pb_gpu = img['PB'].values[:, :, 0]
    g, sw = M.aperture_grid(r['vis'], *args, r['ck'], r['sup'], r['pg'], r['freq'], npad, gp['cell_size'], r['os'])
    raw = M.grid_to_image(g, isz)
    for norm_type in ('flat_sky', 'flat_noise', 'none'):
        out = make_image_with_gcf(mx, gcf, img, gp_user, {'norm_type': norm_type}, {'xds': 'xds0'}, {})
        ref = M.normalize(raw, sw, pb_gpu, img['WEIGHT_PB'].values[:, :, 0], np.ones(tuple(isz)), r['os'],
                          norm_type, 0.2, True)
        got = out['IMAGE'].values[:, :, 0]
        keep = np.abs(pb_gpu - 0.2) > 1e-6          # pixels on the pb_limit edge may go either way
        assert _peak_err(np.where(keep, got, 0), np.where(keep, ref, 0)) < 1e-5, norm_type
        assert np.array_equal(got == 0, ref == 0) or (~keep).any()
        assert np.allclose(out['SUM_WEIGHT'].values[0], sw, rtol=1e-6)
    psf = make_psf_with_gcf(mx, gcf, img, gp_user, {'norm_type': 'flat_sky'}, {'xds': 'xds0'}, {})
    g, sw = M.aperture_grid(None, *args, r['ck'], r['sup'], r['pg'], r['freq'], npad, gp['cell_size'], r['os'],
                            do_psf=True)
    ref = M.normalize(M.grid_to_image(g, isz), sw, pb_gpu, img['WEIGHT_PB'].values[:, :, 0], np.ones(tuple(isz)),
                      r['os'], 'flat_sky', 0.2, True)
    c = gp['image_center']
    ref = ref / ref[c[0], c[1]]
    got = psf['PSF'].values[:, :, 0]
    assert np.allclose(got[c[0], c[1]], 1.0)
    assert _peak_err(got, ref) < 1e-5


def test_mosaic_normalize_kernel(ngg):
    """ngg_mosaic_normalize on identical inputs equals _normalize's arithmetic."""
    import torch
    rng = np.random.default_rng(8)
    img = rng.standard_normal((40, 34, 3, 2))
    pb = rng.uniform(0.0, 1.0, img.shape)
    wpb = pb ** 2 + 0.01
    ps = rng.uniform(0.5, 1.5, (40, 34))
    for nt, nimg in (('flat_sky', wpb), ('flat_noise', pb), ('none', None)):
        ref = M.normalize(img, np.ones((3, 2)), pb, wpb, ps, (10, 10), nt, 0.2, True)
        t = torch.as_tensor(img, device='cuda').contiguous()
        ngg.mosaic_normalize(t, ps, nimg, pb, 0.2, (10, 10), True)
        got = t.cpu().numpy()
        assert np.array_equal(got == 0, ref == 0)
        assert np.allclose(got, ref, rtol=2e-7, atol=0)
        t = torch.as_tensor(img, device='cuda').contiguous()
        ngg.mosaic_normalize(t, ps, nimg, pb, 0.0, (10, 10), False, centre=(20, 17))
        ref = M.normalize(img, np.ones((3, 2)), pb, wpb, ps, (10, 10), nt, 0.0, False)
        assert np.allclose(t.cpu().numpy(), ref / ref[20, 17], rtol=1e-13)


def test_gcf_rejects_bad_tables(ngg, gold):
    d = gold
    fidx = np.where(d['field'] >= 0, d['field'], -1)
    with pytest.raises(ngg.NggError, match='table'):
        _grid(ngg, d, 'data', np.ascontiguousarray(d['conv_kernel'][..., 12:-12, 12:-12]), d['support'], _slopes(d), fidx)
    with pytest.raises(ngg.NggError, match='support'):
        _grid(ngg, d, 'data', d['conv_kernel'], np.full_like(d['support'], 33), _slopes(d), fidx)


def test_aperture_seam_functions_match_reference(ngg, gold):
    """The per-chunk seam (reference names and arguments, numpy in and out)."""
    from cngi_prototype_gb300.imaging._imaging_utils import _aperture_grid as A
    d = gold
    gp = _gp(d)
    gp.update({'oversampling': d['oversampling'], 'field_id': np.arange(2), 'complex_grid': True})
    common = (d['uvw'], d['imaging_weight'], d['field'], d['cf_baseline_map'], d['cf_chan_map'], d['cf_pol_map'])
    g, sw = A._aperture_grid_numpy_wrap(d['vis'], *common, d['conv_kernel'], d['support'], d['phase_gradient'],
                                        d['freq'], gp)
    assert g.dtype == np.complex128 and _peak_err(g, d['grid']) < 2e-6 and np.allclose(sw, d['sum_weight'], rtol=1e-6)
    g, sw = A._aperture_psf_grid_numpy_wrap(*common, d['conv_kernel'], d['support'], d['phase_gradient'], d['freq'],
                                            gp)
    assert _peak_err(g, d['psf_grid']) < 2e-6 and np.allclose(sw, d['psf_sum_weight'], rtol=1e-6)
    g, sw = A._aperture_weight_grid_numpy_wrap(*common, d['weight_conv_kernel'], d['support'], d['phase_gradient'],
                                               d['freq'], gp)
    assert _peak_err(g, d['weight_grid']) < 2e-6 and np.allclose(sw, d['weight_sum_weight'], rtol=1e-6)


def test_graph_aperture_grid_matches_reference(ngg, gold):
    """_graph_aperture_grid (reference name and arguments): datasets in,
    [grid (u, v, C, P), sum_weight] out, equal to the golden grids."""
    from cngi_prototype_gb300 import xds
    from cngi_prototype_gb300.imaging._imaging_utils._aperture_grid import _graph_aperture_grid
    d = gold
    gp = _gp(d)
    gp.update({'oversampling': d['oversampling'], 'field_id': np.arange(2), 'complex_grid': True})
    vds = xds.vis_dataset(d['uvw'], d['vis'], d['imaging_weight'], d['freq'], field_id=d['field'])
    vds['IMAGING_WEIGHT'] = (('time', 'baseline', 'chan', 'pol'), d['imaging_weight'])
    gcf = xds.Dataset({'CF_BASELINE_MAP': (('baseline',), d['cf_baseline_map']),
                       'CF_CHAN_MAP': (('chan',), d['cf_chan_map']), 'CF_POL_MAP': (('pol',), d['cf_pol_map']),
                       'CONV_KERNEL': (('a', 'b', 'c', 'x', 'y'), d['conv_kernel']),
                       'WEIGHT_CONV_KERNEL': (('a', 'b', 'c', 'x', 'y'), d['weight_conv_kernel']),
                       'SUPPORT': (('a', 'b', 'c', 'i'), d['support']),
                       'PHASE_GRADIENT': (('f', 'x', 'y'), d['phase_gradient'])},
                      coords={'field_id': ('field', np.arange(2))})
    sel = {'data_group_in': {'data': 'DATA', 'uvw': 'UVW', 'imaging_weight': 'IMAGING_WEIGHT'}}
    for flags, key in (({}, 'grid'), ({'do_psf': True}, 'psf_grid'), ({'grid_weights': True}, 'weight_grid')):
        g, sw = _graph_aperture_grid(vds, gcf, {**gp, **flags}, sel)
        assert g.shape == np.moveaxis(d[key], [0, 1], [-2, -1]).shape
        assert _peak_err(np.moveaxis(g, [-2, -1], [0, 1]), d[key]) < 2e-6
