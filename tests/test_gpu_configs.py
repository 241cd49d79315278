"""GPU parity at the workload sizes the benchmark quotes, against the oracle.

* Small cube (27 antennas, 600 x 10 s, 32 channels, RR/LL, 512^2 at 2",
  natural weighting): make_imaging_weight + make_psf + make_image through the
  public API, image and PSF against the FP64 C oracle grid + numpy FFT.
* Large cube, three channels of its band (bottom, middle, top, where the uv
  extent is widest): the full 4915^2 grid and all 1024 x 2016 rows, Briggs
  0.5 with 5% flags; density grid, imaging weights, grid and sum_weight
  against the oracle.
* Mosaic, reduced (7 pointings, 4 channels, 12 m dishes at 100 GHz, 2048^2 at
  0.2", support 29): GCF tables and the aperture gridder against the oracle.
* Degrid/grid pair at 2048^2 (C3's image and grid, a few thousand rows):
  adjoint identity, FP64 adjoint and central differences at 256 pixels.

Tolerances: 1e-5 of the peak for grids and images (FP32 taps and sums against
FP64), sums of weights 1e-6 relative, imaging weights 2e-6 relative.
"""
import numpy as np
import pytest

from oracle import cbind
from oracle import imaging as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _peak_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _ref_image(go, swo, npad, image_size):
    """Oracle image: FP64 grid -> numpy FFT -> crop -> / sum_weight / correction."""
    corr = O.remove_padding(O.create_prolate_spheroidal_correction(np.asarray(npad)), image_size)
    return O.correct_image(O.uncorrected_image(go, image_size), swo, corr)


def test_small_cube_whole_pipeline_matches_oracle(ngg):
    from cngi_prototype_gb300 import simulate, xds
    from cngi_prototype_gb300.imaging import make_image, make_imaging_weight, make_psf
    obs = simulate.config_standard_small(seed=1)
    T, B, C, P = obs.vis.shape
    assert (T, B, C, P) == (600, 351, 32, 2)
    gp = {'image_size': [512, 512], 'cell_size': [2.0, 2.0], 'chan_mode': 'cube', 'phase_center': [0.0, 0.0]}
    mx = xds.mxds({'xds0': xds.vis_dataset(obs.uvw, obs.vis, obs.weight, obs.freq)})
    m2 = make_imaging_weight(mx, {'weighting': 'natural'}, gp, {'xds': 'xds0'})
    im = make_psf(m2, xds.Dataset(), gp, {'xds': 'xds0'}, {})
    im = make_image(m2, im, gp, {'xds': 'xds0'}, {})
    gpc = dict(gp)
    O.check_grid_parms(gpc)
    npad, cell = gpc['image_size_padded'], gpc['cell_size']
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    w64 = obs.weight.astype(np.float64)
    go, swo = cbind.grid('data', obs.vis, obs.uvw, w64, obs.freq, cgk, 7, 100, npad, cell)
    ref = _ref_image(go, swo, npad, gp['image_size'])
    img = im['IMAGE'].values[:, :, 0]
    assert img.shape == ref.shape
    e = _peak_err(img, ref)
    assert e < TOL, e
    assert np.allclose(im['SUM_WEIGHT'].values[0], swo, rtol=1e-6)
    gp_, swp = cbind.grid('psf', None, obs.uvw, w64, obs.freq, cgk, 7, 100, npad, cell)
    pref = _ref_image(gp_, swp, npad, gp['image_size'])
    e = _peak_err(im['PSF'].values[:, :, 0], pref)
    assert e < TOL, e
    assert np.allclose(im['PSF_SUM_WEIGHT'].values[0], swp, rtol=1e-6)


@pytest.fixture(scope='module')
def large_cube_slice():
    """Channels 0, 127 and 255 of the 256-channel large cube: all rows, 5%
    flags, vis on the GPU (cube-mode channels are independent, so a channel
    subset images exactly as in the whole cube)."""
    import torch
    from cngi_prototype_gb300 import simulate
    parts = [simulate.config_large_cube(seed=2, vis_device='cuda', chan_range=(c, c + 1)) for c in (0, 127, 255)]
    vis = torch.cat([p.vis for p in parts], dim=2).contiguous()
    w = torch.cat([p.weight for p in parts], dim=2).contiguous()
    freq = np.concatenate([p.freq for p in parts])
    return parts[0].uvw, vis, w, freq


def test_large_cube_channels_briggs_grid_match_oracle(ngg, large_cube_slice):
    import torch
    uvw, vis_d, w_d, freq = large_cube_slice
    T, B, C, P = vis_d.shape
    assert (T, B, C, P) == (1024, 2016, 3, 2)
    gp = {'image_size': [4096, 4096], 'cell_size': [1.0, 1.0], 'chan_mode': 'cube'}
    O.check_grid_parms(gp)
    npad, cell = gp['image_size_padded'], gp['cell_size']
    assert list(npad) == [4915, 4915]
    uvw_d = torch.as_tensor(uvw, device='cuda')
    f_d = torch.as_tensor(freq, device='cuda')
    # Briggs 0.5 weights on the GPU
    dens, dsw = ngg.grid_density(uvw_d, w_d, f_d, gp['image_size'], cell)
    fac = ngg.briggs_factors(dens, dsw, 'briggs', 0.5)
    iw_d = ngg.weight_lookup(uvw_d, w_d, f_d, dens, fac, cell)
    # the same through the oracle, from the same float32 natural weights
    w_h = w_d.cpu().numpy().astype(np.float64)
    do, dswo = cbind.grid('density', None, uvw, w_h, freq, np.ones(1), 1, 0, gp['image_size'], cell)
    assert _peak_err(dens.cpu().numpy(), do[:, 0]) < 1e-6
    assert np.allclose(dsw.cpu().numpy(), dswo[:, 0], rtol=1e-6)
    fo = O.calculate_briggs_parms(np.moveaxis(do, (0, 1), (2, 3)), dswo,
                                  {'weighting': 'briggs', 'robust': 0.5})
    assert np.allclose(fac.cpu().numpy(), fo[:, :, 0], rtol=1e-5)
    iwo = cbind.weight_degrid(np.moveaxis(do, (0, 1), (2, 3)), uvw, w_h, fo, freq, gp['image_size'], cell)
    iw = iw_d.cpu().numpy()
    fin = np.isfinite(iwo)
    assert np.array_equal(fin, np.isfinite(iw))
    assert np.allclose(iw[fin], iwo[fin], rtol=2e-6, atol=1e-7 * np.abs(iwo[fin]).max())
    # grid and sum_weight with those imaging weights (float32 on both sides)
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    g, sw = ngg.grid_ps(vis_d, uvw_d, iw_d, f_d, torch.as_tensor(cgk, device='cuda'), npad, cell)
    iw64 = iw.astype(np.float64)
    vis_h = vis_d.cpu().numpy()
    go, swo = cbind.grid('data', vis_h, uvw, iw64, freq, cgk, 7, 100, npad, cell)
    gh = g.cpu().numpy()
    del g
    for c in range(C):
        e = _peak_err(gh[c], go[c])
        assert e < TOL, (c, e)
        assert np.array_equal(np.abs(gh[c]) > 0, np.abs(go[c]) > 0)
    assert np.allclose(sw.cpu().numpy(), swo, rtol=1e-6)
    # images of the three channels (FFT, crop, correction on the GPU)
    corr = O.remove_padding(O.create_prolate_spheroidal_correction(np.asarray(npad)), gp['image_size'])
    gf = torch.fft.ifftshift(torch.as_tensor(gh, device='cuda'), dim=(2, 3)).contiguous()
    del gh
    img = ngg.fft_correct(gf, sw, corr, gp['image_size']).cpu().numpy()
    del gf
    ref = _ref_image(go, swo, npad, gp['image_size'])
    for c in range(C):
        e = _peak_err(img[:, :, c], ref[:, :, c])
        assert e < TOL, (c, e)


def test_reduced_mosaic_matches_oracle(ngg):
    """7 pointings, 4 channels of the mosaic workload (support 29)."""
    import torch
    from cngi_prototype_gb300 import simulate, xds
    from cngi_prototype_gb300.imaging import make_gridding_convolution_function
    from cngi_prototype_gb300.imaging._imaging_utils import _mosaic
    obs = simulate.config_mosaic(seed=4, n_chan=4, n_pointing=7, vis_device='cuda')
    vis_d, w_d = obs.vis, obs.weight
    T, B, C, P = vis_d.shape
    gp = {'image_size': [2048, 2048], 'cell_size': [0.2, 0.2], 'fft_padding': 1.2}
    gcf_parms = {'function': 'casa_airy', 'list_dish_diameters': [obs.dish],
                 'list_blockage_diameters': [obs.blockage],
                 'unique_ant_indx': [0] * (int(max(obs.antenna1.max(), obs.antenna2.max())) + 1),
                 'oversampling': list(obs.oversampling), 'max_support': list(obs.max_support),
                 'phase_center': obs.phase_center, 'chan_tolerance_factor': 0.005}
    fds = xds.Dataset({'PHASE_DIR': (('field_id', 'poly_id', 'pair'), obs.field_phase_dir[:, None, :])},
                      coords={'field_id': ('field_id', np.arange(len(obs.field_phase_dir)))})
    vds = xds.vis_dataset(obs.uvw, None, np.broadcast_to(np.float32(1), (T, B, C, P)), obs.freq, field_id=obs.field,
                          antenna1=obs.antenna1, antenna2=obs.antenna2)
    mx = xds.mxds({'xds0': vds}, FIELD=fds)
    gcf = make_gridding_convolution_function(mx, gcf_parms, gp, {'xds': 'xds0'})
    sup = np.asarray(gcf['SUPPORT'].values)
    assert int(sup.max()) == 29
    gpc = dict(gp)
    O.check_grid_parms(gpc)
    npad, cell = gpc['image_size_padded'], gpc['cell_size']
    os_ = np.asarray(gcf.attrs['oversampling'])
    fidx = _mosaic.field_indices(obs.field, gcf['field_id'].values)
    maps = [gcf[k].values for k in ('CF_BASELINE_MAP', 'CF_CHAN_MAP', 'CF_POL_MAP')]
    ck = gcf['CONV_KERNEL'].values
    slopes = _mosaic.phase_slopes(gcf)
    g, sw = ngg.grid_gcf(vis_d, obs.uvw, w_d, obs.freq, fidx, *maps, ck, sup, slopes, npad, cell, os_)
    vis_h = vis_d.cpu().numpy()
    w_h = w_d.cpu().numpy().astype(np.float64)
    go, swo = cbind.aperture_grid('data', vis_h, obs.uvw, w_h, fidx, *maps, ck, sup, gcf['PHASE_GRADIENT'].values,
                                  obs.freq, os_, npad, cell)
    gh = g.cpu().numpy()
    for c in range(C):
        e = _peak_err(gh[c], go[c])
        assert e < 2e-6, (c, e)
    assert np.allclose(sw.cpu().numpy(), swo, rtol=1e-6)
    del torch


def _c3_geometry(n_time=2, C=2, P=1):
    from cngi_prototype_gb300 import simulate
    rng = np.random.default_rng(3)
    enu = simulate.log_spiral_layout(64, 2500.0, rng)
    uvw = simulate.earth_rotation_uvw(enu, n_time, 8.0 * 496)
    T, B = uvw.shape[:2]
    freq = 1.0e9 + (np.arange(C) + 0.5) * (0.5e9 / C)
    w = rng.uniform(0.5, 2.0, (T, B, C, P)).astype(np.float32)
    gp = {'image_size': [2048, 2048], 'cell_size': [1.0, 1.0], 'chan_mode': 'cube'}
    O.check_grid_parms(gp)
    return uvw, w, freq, gp, rng


def test_degrid_pair_at_2048_adjoint_and_fp64(ngg):
    import torch
    from cngi_prototype_gb300.imaging.degrid import ImagingOperator
    from test_gpu_degrid import _numpy_degrid
    uvw, w, freq, gp, rng = _c3_geometry()
    op = ImagingOperator(uvw, w, freq, gp)
    T, B, C, P = w.shape
    assert T * B == 4032 and list(op.npad) == [2457, 2457]
    N = 2048
    for _ in range(2):
        x = torch.as_tensor(rng.standard_normal((N, N, C, P)), device='cuda')
        y = torch.as_tensor((rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P)))
                            .astype(np.complex64), device='cuda')
        ax = op.degrid(x).to(torch.complex128)
        dy = op.image(y)
        lhs = float(torch.sum(torch.conj(ax) * y.to(torch.complex128)).real)
        rhs = float(torch.sum(x * dy))
        scale = float(torch.linalg.vector_norm(ax) * torch.linalg.vector_norm(y.to(torch.complex128)) +
                      torch.linalg.vector_norm(x) * torch.linalg.vector_norm(dy))
        assert abs(lhs - rhs) <= 1e-6 * scale, (lhs, rhs, scale)
    x = rng.standard_normal((N, N, C, P))
    got = op.degrid(torch.as_tensor(x, device='cuda')).cpu().numpy()
    corr = O.remove_padding(O.create_prolate_spheroidal_correction(op.npad), gp['image_size'])
    ref = _numpy_degrid(x, uvw, w.astype(np.float64), freq, gp, op.sum_weight.cpu().numpy(), corr)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def test_degrid_pair_at_2048_finite_differences(ngg):
    import torch
    from cngi_prototype_gb300.imaging.degrid import ImagingOperator, degrid
    uvw, w, freq, gp, rng = _c3_geometry()
    op = ImagingOperator(uvw, w, freq, gp)
    T, B, C, P = w.shape
    N = 2048
    # model: Gaussian blobs (FWHM 2-20 px), data = model visibilities + noise 0.1
    yy, xx = np.meshgrid(np.arange(N), np.arange(N), indexing='ij')
    model = np.zeros((N, N))
    for k in range(20):
        px, py = rng.uniform(200, N - 200, 2)
        s2 = (rng.uniform(2, 20) / 2.3548) ** 2
        model += rng.uniform(0, 1) * np.exp(-((xx - px) ** 2 + (yy - py) ** 2) / (2 * s2))
    x_true = torch.as_tensor(np.repeat(model[:, :, None, None], C, axis=2), device='cuda')
    v_data = (op.degrid(x_true).to(torch.complex128) +
              torch.as_tensor(0.1 * (rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P))),
                              device='cuda')).to(torch.complex64)
    # The map is linear, so its backward does not depend on x. At 2048^2 one
    # pixel moves a visibility by ~1e-7 of the visibility of a full-image
    # model, so a model of even 1e-3 per pixel would make the FP32 rounding of
    # A(x +- eps delta) as large as the difference itself: x is kept at 1e-9.
    x = torch.as_tensor(rng.uniform(0, 1e-9, (N, N, C, P)), device='cuda').requires_grad_(True)

    def loss(img):
        r = degrid(img, op).to(torch.complex128) - v_data.to(torch.complex128)
        return torch.sum(r.real ** 2 + r.imag ** 2)

    loss(x).backward()
    grad = x.grad.detach().cpu().numpy()
    eps = 1e-3
    idx = rng.integers(0, N, (256, 2))
    ch = rng.integers(0, C, 256)
    fd = np.empty(256)
    with torch.no_grad():
        for k in range(256):
            d = torch.zeros_like(x)
            d[idx[k, 0], idx[k, 1], ch[k], 0] = eps
            fd[k] = (float(loss(x + d)) - float(loss(x - d))) / (2 * eps)
    an = grad[idx[:, 0], idx[:, 1], ch, 0]
    rel = np.abs(fd - an) / np.abs(an).max()
    assert np.median(rel) < 1e-4 and rel.max() < 1e-3, (np.median(rel), rel.max())
    # and the gradient is twice the FP64 reference gridder's residual image
    vm = op.degrid(x.detach())
    resid = (vm - v_data).cpu().numpy()
    ref, _ = O.make_image_arrays(resid, uvw, w.astype(np.float64), freq, gp)
    assert np.abs(grad - 2 * ref).max() <= 5e-5 * np.abs(2 * ref).max()
