"""predict_modelvis_image on the GPU: the oracle's prediction (FP64), the
storage options, and a major cycle that closes (image -> CLEAN -> predict ->
residual visibilities)."""
import numpy as np
import pytest

from oracle import imaging as O

pytestmark = pytest.mark.gpu


def _vis_ds(seed, T, C, P, n_ant=12):
    from cngi_prototype_gb300 import simulate, xds
    rng = np.random.default_rng(seed)
    enu = simulate.disk_layout(n_ant, 400.0, rng)
    uvw = simulate.earth_rotation_uvw(enu, T, 120.0)
    B = uvw.shape[1]
    freq = 1.0e9 + 2e7 * np.arange(C)
    vis = np.zeros((T, B, C, P), dtype=np.complex128)
    return xds.vis_dataset(uvw, vis, np.ones((T, B, C, P)), freq), uvw, freq, rng


def _img(model):
    from cngi_prototype_gb300 import xds
    return xds.Dataset({'MODEL': (('l', 'm', 'time', 'chan', 'pol'), model)})


@pytest.mark.parametrize('C,C_img,P,P_img,N0,N1', [(2, 2, 2, 2, 80, 72), (3, 1, 2, 1, 80, 72), (1, 1, 1, 1, 80, 72),
                                                   (2, 2, 1, 1, 81, 73)])
def test_predict_matches_oracle(ngg, C, C_img, P, P_img, N0, N1):
    from cngi_prototype_gb300.imaging import predict_modelvis_image
    ds, uvw, freq, rng = _vis_ds(7 + C + N0, 24, C, P)
    gp = {'image_size': [N0, N1], 'cell_size': [9.0, 9.0]}
    model = rng.standard_normal((N0, N1, 1, C_img, P_img))
    out = predict_modelvis_image(_img(model), ds, gp)
    got = out['MODEL'].values
    O.check_grid_parms(gp)
    m = model[:, :, 0]
    if P_img != P:
        m = np.repeat(m, P, axis=3)
    ref = O.predict_vis(m, uvw, freq, gp)
    assert got.shape == ref.shape and got.dtype == np.complex128   # DATA's dtype
    # complex64 model grid: ~3e-6 of the peak on this white-noise model (its
    # edge pixels amplified up to ~10x by 1/grdsf); the FP32 path's bound is 1e-5
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def test_storage_parms_and_inputs_unchanged(ngg):
    from cngi_prototype_gb300.imaging import predict_modelvis_image
    ds, uvw, freq, rng = _vis_ds(11, 12, 2, 2)
    gp = {'image_size': [64, 64], 'cell_size': [9.0, 9.0]}
    a = rng.standard_normal((64, 64, 1, 2, 2))
    b = rng.standard_normal((64, 64, 1, 2, 2))
    first = predict_modelvis_image(_img(a), ds, gp, {'arr_name': 'MODEL_DATA'})
    assert 'MODEL_DATA' in first and 'MODEL_DATA' not in ds and 'MODEL' not in first
    both = predict_modelvis_image(_img(b), first, gp, {'arr_name': 'MODEL_DATA', 'incremental': True})
    alone = predict_modelvis_image(_img(a + b), ds, gp, {'arr_name': 'MODEL_DATA'})
    v = alone['MODEL_DATA'].values
    assert np.abs(both['MODEL_DATA'].values - v).max() <= 1e-5 * np.abs(v).max()
    with pytest.raises(ValueError):
        predict_modelvis_image(_img(a[:32]), ds, gp)


def test_major_cycle_closes(ngg):
    """Point sources on pixel centres, 40 antennas over 5.3 h: make_image, a
    PSF twice the image size, CLEAN to 0.2% of the peak, predict the CLEAN
    model. The residual visibilities DATA - MODEL are < 1% of DATA, the CLEAN
    model holds each source's flux, and the dirty image of the residual
    visibilities stays at the CLEAN residual's level (0.2% of the peak, plus
    the shifted-PSF and prediction approximations, both ~0.2%)."""
    from cngi_prototype_gb300 import simulate, xds
    from cngi_prototype_gb300.deconvolution import deconvolve_point_clean
    from cngi_prototype_gb300.imaging import make_image, make_psf, predict_modelvis_image
    rng = np.random.default_rng(5)
    enu = simulate.disk_layout(40, 600.0, rng)
    uvw = simulate.earth_rotation_uvw(enu, 160, 120.0)
    freq = np.array([1.0e9])
    N = 96
    gp = {'image_size': [N, N], 'cell_size': [6.0, 6.0], 'chan_mode': 'cube', 'phase_center': [0.0, 0.0]}
    gp2 = dict(gp, image_size=[2 * N, 2 * N])
    cell = np.deg2rad(np.array([6.0, 6.0]) / 3600)
    px = np.array([48, 30, 60, 70]); py = np.array([48, 55, 35, 62])
    flux = np.array([1.0, 0.6, 0.4, 0.25])
    l, m = simulate.pixel_to_lm(px, py, [N, N], cell)
    vis = simulate.point_source_vis(uvw, freq, l, m, flux, n_pol=1, dtype=np.complex128)
    ds = xds.vis_dataset(uvw, vis, np.ones(vis.shape), freq, pol=(1,))
    mx = xds.mxds({'xds0': ds})
    dirty = make_image(mx, xds.Dataset(), gp, {'xds': 'xds0'}, {})['IMAGE'].values
    psf = make_psf(mx, xds.Dataset(), gp2, {'xds': 'xds0'}, {})['PSF'].values
    psf_peak = float(psf[N, N, 0, 0, 0])   # ~ 1/grdsf(0): model components in Jy/pixel after dividing
    img = xds.Dataset({'IMAGE': (('l', 'm', 'time', 'chan', 'pol'), dirty),
                       'PSF': (('l2', 'm2', 'time', 'chan', 'pol'), psf)})
    cl = deconvolve_point_clean(img, {'gain': 0.2, 'threshold': 0.002, 'n_iter': 3000}, {})
    model = cl['MODEL'].values / psf_peak
    for k in range(len(flux)):
        assert abs(model[px[k] - 2:px[k] + 3, py[k] - 2:py[k] + 3, 0, 0, 0].sum() - flux[k]) < 0.005
    pred = predict_modelvis_image(cl, ds, gp, model='MODEL')['MODEL'].values / psf_peak
    res = vis - pred
    assert np.sqrt(np.mean(np.abs(res) ** 2)) < 0.01 * np.sqrt(np.mean(np.abs(vis) ** 2))
    ds_res = xds.vis_dataset(uvw, res, np.ones(vis.shape), freq, pol=(1,))
    rimg = make_image(xds.mxds({'xds0': ds_res}), xds.Dataset(), gp, {'xds': 'xds0'}, {})['IMAGE'].values
    assert np.abs(rimg).max() < 0.005 * flux.max()
    assert np.abs(cl['RESIDUAL'].values).max() < 0.0025 * flux.max()
