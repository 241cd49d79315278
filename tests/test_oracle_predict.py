"""The oracle's model-visibility prediction against the direct Fourier sum.

The reference's predict_modelvis_image is a stub (no outputs to pin), so the
oracle is pinned to the definition it states: the model visibilities of a
model image in Jy/pixel, V(u, v) = sum_pixels I exp(-2 pi i (u l + v m)),
with (l, m) the pixel's direction under make_image's geometry (a source at
(l, m) images at that pixel). The oracle reads the gridder's 7x7 footprint
with its oversampling-100 offsets, so its error is the kernel's aliasing
(< 2e-3 of the flux over the inner 80% of the field) plus the offset's
quantisation: a phase of at most 2 pi |x| (0.5 / 100) / Npad for a source x
pixels from the centre.
"""
import numpy as np

from oracle import imaging as O


def _obs(seed=3, n_ant=12, T=30):
    from cngi_prototype_gb300 import simulate
    rng = np.random.default_rng(seed)
    enu = simulate.disk_layout(n_ant, 400.0, rng)
    return simulate.earth_rotation_uvw(enu, T, 120.0), rng


def test_predict_matches_direct_fourier_sum():
    from cngi_prototype_gb300 import simulate
    uvw, rng = _obs()
    freq = np.array([1.0e9, 1.05e9])
    N = 128
    gp = {'image_size': [N, N], 'cell_size': [8.0, 8.0]}
    O.check_grid_parms(gp)
    npad = np.asarray(gp['image_size_padded'])
    cell = np.deg2rad(np.array([8.0, 8.0]) / 3600)
    px = rng.integers(N // 2 - 48, N // 2 + 48, 6)
    py = rng.integers(N // 2 - 48, N // 2 + 48, 6)
    flux = rng.uniform(0.2, 1.0, 6)
    model = np.zeros((N, N, 1, 2))
    np.add.at(model, (px, py, 0, 0), flux)
    model[:, :, 0, 1] = model[:, :, 0, 0]
    got = O.predict_vis(model, uvw, freq, gp)
    l, m = simulate.pixel_to_lm(px, py, [N, N], cell)
    ref = simulate.point_source_vis(uvw, freq, l, m, flux, n_pol=2, dtype=np.complex128)
    assert np.all(got != 0)   # every footprint is inside this grid
    quant = np.pi * (np.abs(px - N // 2) / npad[0] + np.abs(py - N // 2) / npad[1]) / 100.0
    bound = np.sum(flux * (quant + 2e-3))
    assert np.abs(got - ref).max() <= bound


def test_predict_is_linear_and_continuum_maps_to_plane_zero():
    uvw, rng = _obs(seed=4, T=10)
    freq = np.array([1.0e9, 1.02e9, 1.04e9])
    gp = {'image_size': [48, 40], 'cell_size': [10.0, 10.0]}
    O.check_grid_parms(gp)
    a = rng.standard_normal((48, 40, 1, 1))
    b = rng.standard_normal((48, 40, 1, 1))
    va, vb, vab = (O.predict_vis(x, uvw, freq, gp) for x in (a, b, 2 * a - b))
    assert np.abs(vab - (2 * va - vb)).max() <= 1e-12 * np.abs(vab).max()
    cube = O.predict_vis(np.repeat(a, 3, axis=2), uvw, freq, gp)
    assert np.array_equal(cube, va)
