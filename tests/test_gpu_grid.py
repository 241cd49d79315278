"""GPU parity of the standard-gridder path against the oracle (through the C ABI).

Tolerances: cell/offset indices bit-exact; grids, sums of weights, imaging
weights and images within 1e-5 of the peak (FP32 taps and accumulation against
an FP64 oracle evaluated on the same float32-rounded weights).
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import cbind
from oracle import imaging as O

pytestmark = pytest.mark.gpu

CASES = ['std_cube', 'std_odd', 'std_onepol', 'std_continuum']
TOL = 1e-5


def _gp(d):
    gp = {'image_size': list(d['image_size']), 'cell_size': list(d['cell_arcsec']), 'chan_mode': str(d['chan_mode'])}
    O.check_grid_parms(gp)
    return gp


def _w32(d):
    return d['weight'].astype(np.float32)


def _peak_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_cell_indices_bit_exact_random(ngg):
    rng = np.random.default_rng(5)
    n = 200000
    freq = np.linspace(1.0e9, 1.5e9, 7)
    for npad, cell_as in [(614, 2.0), (4915, 1.0), (2457, 0.2), (75, 40.0)]:
        dl = np.array([-cell_as, cell_as]) * O.ARCSEC_TO_RAD
        s = O.uv_scale(freq, dl, np.array([npad, npad]))
        umax = 0.55 * npad / np.abs(s).max()
        uvw = rng.uniform(-umax, umax, (n, 3))
        for mirror in (False, True):
            idx, nfb = ngg.cell_indices(uvw, freq, [npad, npad], dl, 100, mirror)
            idx = idx.cpu().numpy()
            u = uvw[:, None, 0] * s[0][None, :]
            v = uvw[:, None, 1] * s[1][None, :]
            if mirror:
                u, v = -u, -v
            up, vp = u + npad // 2, v + npad // 2
            cu, cv = np.trunc(up + 0.5), np.trunc(vp + 0.5)
            ou = np.floor((cu - up) * 100 + 0.5)
            ov = np.floor((cv - vp) * 100 + 0.5)
            ok = (cu > 1) & (cv > 1)   # interior cells (offsets of edge cells are irrelevant)
            assert np.array_equal(idx[..., 0], cu.astype(np.int32))
            assert np.array_equal(idx[..., 1], cv.astype(np.int32))
            assert np.array_equal(idx[..., 2][ok], ou[ok].astype(np.int32))
            assert np.array_equal(idx[..., 3][ok], ov[ok].astype(np.int32))


def test_cell_indices_bit_exact_at_rounding_boundaries(ngg):
    """uvw placed within a few ulps of every rounding boundary must still give
    the FP64 answer (these take the FP64 fallback path)."""
    rng = np.random.default_rng(9)
    npad = 4915
    freq = np.array([1.0e9, 1.2345e9])
    dl = np.array([-1.0, 1.0]) * O.ARCSEC_TO_RAD
    s = O.uv_scale(freq, dl, np.array([npad, npad]))
    k = rng.integers(-600, 600, 5000).astype(np.float64)
    frac = rng.choice([0.0, 0.5, 0.005, 0.995, 0.125], 5000)
    target = k + frac        # pixel offsets at cell and oversampling boundaries
    u = target / s[0][0]
    v = target / s[1][0]
    rows = []
    for dd in range(-4, 5):
        rows.append(np.stack([np.nextafter(u, u + dd) if dd else u, np.nextafter(v, v - dd) if dd else v,
                              np.zeros_like(u)], axis=1))
    uvw = np.concatenate(rows)
    idx, nfb = ngg.cell_indices(uvw, freq, [npad, npad], dl, 100, False)
    idx = idx.cpu().numpy()
    uu = uvw[:, None, 0] * s[0][None, :]
    vv = uvw[:, None, 1] * s[1][None, :]
    up, vp = uu + npad // 2, vv + npad // 2
    cu, cv = np.trunc(up + 0.5), np.trunc(vp + 0.5)
    ou = np.floor((cu - up) * 100 + 0.5)
    ov = np.floor((cv - vp) * 100 + 0.5)
    assert np.array_equal(idx[..., 0], cu.astype(np.int32))
    assert np.array_equal(idx[..., 1], cv.astype(np.int32))
    assert np.array_equal(idx[..., 2], ou.astype(np.int32))
    assert np.array_equal(idx[..., 3], ov.astype(np.int32))
    assert nfb > 0


@pytest.mark.parametrize('name', CASES)
def test_grid_data_and_psf_match_oracle(ngg, name):
    d = load_golden(name)
    gp = _gp(d)
    cm = gp['chan_mode']
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    npad = gp['image_size_padded']
    w32 = _w32(d)
    for mode in ('data', 'psf'):
        g, sw = ngg.grid_ps(d['vis'], d['uvw'], w32, d['freq'], cgk, npad, gp['cell_size'], mode=mode, chan_mode=cm)
        g, sw = g.cpu().numpy(), sw.cpu().numpy()
        go, swo = cbind.grid(mode, d['vis'], d['uvw'], w32.astype(np.float64), d['freq'], cgk, 7, 100, npad,
                             gp['cell_size'], cm)
        assert g.shape == go.shape
        assert _peak_err(g, go) < TOL, (mode, _peak_err(g, go))
        assert np.allclose(sw, swo, rtol=1e-6, atol=0), (mode, sw, swo)
        # and against the reference's own output (float64 weights)
        ref = d['grid'] if mode == 'data' else d['psf_grid']
        assert _peak_err(g, ref) < TOL
        # the footprint is exactly the reference's: same set of touched cells
        assert np.array_equal(np.abs(g) > 0, np.abs(go) > 0)


@pytest.mark.parametrize('name', CASES)
def test_grid_fft_layout_is_shifted_natural(ngg, name):
    d = load_golden(name)
    gp = _gp(d)
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    npad = gp['image_size_padded']
    g, _ = ngg.grid_ps(d['vis'], d['uvw'], _w32(d), d['freq'], cgk, npad, gp['cell_size'], chan_mode=gp['chan_mode'])
    gf, _ = ngg.grid_ps(d['vis'], d['uvw'], _w32(d), d['freq'], cgk, npad, gp['cell_size'], chan_mode=gp['chan_mode'],
                        layout='fft')
    g, gf = g.cpu().numpy(), gf.cpu().numpy()
    assert _peak_err(gf, np.fft.ifftshift(g, axes=(2, 3))) < 1e-6


@pytest.mark.parametrize('name', ['std_cube', 'std_odd', 'std_onepol', 'std_continuum'])
def test_density_briggs_lookup_match_reference(ngg, name):
    d = load_golden(name)
    gp = _gp(d)
    cm = gp['chan_mode']
    w32 = _w32(d)
    dens, dsw = ngg.grid_density(d['uvw'], w32, d['freq'], gp['image_size'], gp['cell_size'], cm)
    dens_np, dsw_np = dens.cpu().numpy(), dsw.cpu().numpy()
    do, dswo = cbind.grid('density', None, d['uvw'], w32.astype(np.float64), d['freq'], np.ones(1), 1, 0,
                          gp['image_size'], gp['cell_size'], cm)
    for p in range(do.shape[1]):   # every pol plane of the reference equals the single plane
        assert _peak_err(dens_np, do[:, p]) < 1e-6
        assert np.allclose(dsw_np, dswo[:, p], rtol=1e-6)
    assert np.array_equal(dens_np > 0, do[:, 0] > 0)
    if cm != 'cube':
        return
    for tag in ['briggs_+0.5', 'uniform_+0.0', 'briggs_-1.3']:
        w, r = tag.split('_')
        f = ngg.briggs_factors(dens, dsw, w, float(r))
        ref_f = d['briggs_factors_' + tag]
        assert np.allclose(f.cpu().numpy(), ref_f[:, :, 0], rtol=1e-5)
        iw = ngg.weight_lookup(d['uvw'], w32, d['freq'], dens, f, gp['cell_size'], cm).cpu().numpy()
        ref = d['imaging_weight_' + tag]
        assert np.allclose(iw, ref, rtol=2e-6, atol=1e-7 * np.abs(ref).max())
        assert np.array_equal(iw == 0, ref == 0)


@pytest.mark.parametrize('name', ['std_cube', 'std_odd', 'std_onepol'])
def test_image_and_psf_match_reference(ngg, name):
    """Grid -> inverse FFT -> crop -> correction against the reference's
    image and PSF. With the complex128 transform (what make_image's default
    'auto' precision runs at this size) the error is the gridder's alone and
    stays within 1e-5 of the peak. The complex64 transform adds its own
    rounding, which the reference's correction image (1.3e-3 in the image
    corners) amplifies ~770x; its bound is the measured floor of that
    transform on these grids (scipy's FP32 FFT of the same FP64 grid gives
    6e-6 alone), 2e-5."""
    d = load_golden(name)
    gp = _gp(d)
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    npad = gp['image_size_padded']
    corr = O.remove_padding(O.create_prolate_spheroidal_correction(npad), gp['image_size'])
    for mode, key in (('data', 'image'), ('psf', 'psf')):
        for precision, tol in (('double', TOL), ('single', 2 * TOL)):
            g, sw = ngg.grid_ps(d['vis'], d['uvw'], _w32(d), d['freq'], cgk, npad, gp['cell_size'], mode=mode,
                                layout='fft')
            img = ngg.fft_correct(g, sw, corr, gp['image_size'], precision=precision).cpu().numpy()
            ref = d[key]
            assert img.shape == ref.shape
            assert _peak_err(img, ref) < tol, (mode, precision, _peak_err(img, ref))


def test_edge_cases(ngg):
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    freq = np.array([1.0e9, 1.1e9])
    dl = np.array([-1e-4, 1e-4])
    # empty time axis
    g, sw = ngg.grid_ps(np.zeros((0, 3, 2, 2), np.complex64), np.zeros((0, 3, 3)), np.zeros((0, 3, 2, 2), np.float32),
                        freq, cgk, [40, 40], dl)
    assert not g.cpu().numpy().any() and not sw.cpu().numpy().any()
    # all NaN visibilities / NaN uvw / zero weights -> empty grid
    vis = np.full((4, 3, 2, 2), np.nan, np.complex64)
    g, sw = ngg.grid_ps(vis, np.zeros((4, 3, 3)), np.ones((4, 3, 2, 2), np.float32), freq, cgk, [40, 40], dl)
    assert not g.cpu().numpy().any() and not sw.cpu().numpy().any()
    g, sw = ngg.grid_ps(np.ones((4, 3, 2, 2), np.complex64), np.full((4, 3, 3), np.nan),
                        np.ones((4, 3, 2, 2), np.float32), freq, cgk, [40, 40], dl)
    assert not g.cpu().numpy().any()
    # four polarizations (two kernel launches) agree with the oracle
    rng = np.random.default_rng(3)
    uvw = rng.uniform(-1500, 1500, (10, 6, 3))
    vis = (rng.standard_normal((10, 6, 2, 4)) + 1j * rng.standard_normal((10, 6, 2, 4))).astype(np.complex64)
    w = rng.uniform(0.5, 1.5, (10, 6, 2, 4)).astype(np.float32)
    g, sw = ngg.grid_ps(vis, uvw, w, freq, cgk, [64, 70], dl)
    go, swo = cbind.grid('data', vis, uvw, w.astype(np.float64), freq, cgk, 7, 100, [64, 70], dl)
    assert _peak_err(g.cpu().numpy(), go) < TOL and np.allclose(sw.cpu().numpy(), swo, rtol=1e-6)
    # bad arguments raise
    with pytest.raises(ngg.NggError):
        ngg.grid_ps(vis, uvw, w, freq, cgk, [64, 70], dl, support=5)


def test_graph_standard_grid_matches_reference(ngg):
    """_graph_standard_grid (reference name and arguments): dataset in,
    [grid (u, v, C, P), sum_weight (C, P)] out, equal to the golden grids."""
    from cngi_prototype_gb300 import xds
    from cngi_prototype_gb300.imaging._imaging_utils import _gridding_convolutional_kernels as G
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    from cngi_prototype_gb300.imaging._imaging_utils._standard_grid import _graph_standard_grid
    d = load_golden('std_cube')
    gp = {'image_size': [int(x) for x in d['image_size']], 'cell_size': [float(x) for x in d['cell_arcsec']]}
    _check_grid_parms(gp)
    gp.update({'oversampling': 100, 'support': 7, 'complex_grid': True})
    vds = xds.vis_dataset(d['uvw'], d['vis'], d['weight'], d['freq'])
    vds['IMAGING_WEIGHT'] = (('time', 'baseline', 'chan', 'pol'), d['weight'])
    sel = {'data_group_in': {'data': 'DATA', 'uvw': 'UVW', 'imaging_weight': 'IMAGING_WEIGHT'}}
    cgk = G._create_prolate_spheroidal_kernel_1D(100, 7)
    for flags, key, swkey in (({'do_psf': False}, 'grid', 'sum_weight'), ({'do_psf': True}, 'psf_grid', 'psf_sum_weight')):
        g, sw = _graph_standard_grid(vds, cgk, {**gp, **flags}, sel)
        ref = np.moveaxis(d[key], [0, 1], [-2, -1])
        assert g.shape == ref.shape
        assert np.abs(g - ref).max() <= 1e-5 * np.abs(ref).max()
        assert np.allclose(sw, d[swkey], rtol=1e-6)
