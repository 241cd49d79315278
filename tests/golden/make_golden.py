"""Generate the golden fixtures for the standard-gridder path.

Run where a checkout of the reference exists, naming its root:

    CNGI_REFERENCE_ROOT=<checkout> python tests/golden/make_golden.py

It runs the reference's own per-chunk functions -- _standard_grid_numpy_wrap,
_standard_grid_psf_numpy_wrap, _standard_imaging_weight_degrid_numpy_wrap,
synthesis_imaging_cube's per-chunk function and numpy imaging helpers, the prolate-spheroidal
kernel builders, the GCF helpers and direction_rotate's rotation and phasor
functions, the Hogbom minor cycle and the PSF beam fit -- through ``refshim`` on small seeded
synthetic inputs, and stores inputs and outputs as compressed .npz files next
to this script. The tests read only the .npz files.
"""
import copy
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.abspath(os.path.join(HERE, '..', '..')))

import refshim  # noqa: E402
from cngi_prototype_gb300 import simulate  # noqa: E402


def small_obs(seed, n_ant=8, radius=300.0, n_time=24, dt=120.0, n_chan=3, n_pol=2,
              image=64, cell=45.0, flag_frac=0.05):
    rng = np.random.default_rng(seed)
    enu = simulate.disk_layout(n_ant, radius, rng)
    uvw = simulate.earth_rotation_uvw(enu, n_time, dt)
    freq = 1.0e9 + np.arange(n_chan) * 5.0e7
    T, B = uvw.shape[:2]
    l = np.deg2rad(np.array([0.02, -0.05, 0.1]))
    m = np.deg2rad(np.array([0.03, 0.01, -0.07]))
    vis = simulate.point_source_vis(uvw, freq, l, m, [1.0, 0.5, 0.25], n_pol, 0.1, rng)
    weight = rng.uniform(0.5, 2.0, (T, B, n_chan, n_pol))
    flags = rng.random((T, B, n_chan, n_pol)) < flag_frac
    vis[flags] = np.nan
    weight[rng.random(weight.shape) < 0.02] = 0.0            # zero weights are skipped
    uvw[3, 2, :] = np.nan                                      # a NaN uvw row
    return dict(vis=vis.astype(np.complex64), uvw=uvw, weight=weight, freq=freq,
                image_size=np.array([image, image]), cell_arcsec=np.array([cell, cell]))


def main():
    R = refshim.modules()
    out = {}

    # --- prolate spheroidal kernel tables ------------------------------
    cgk = R.gck._create_prolate_spheroidal_kernel_1D(100, 7)
    _, corr128 = R.gck._create_prolate_spheroidal_kernel(100, 7, np.array([128, 128]))
    _, corr75 = R.gck._create_prolate_spheroidal_kernel(100, 7, np.array([75, 77]))
    u = np.linspace(0, 1.2, 241)
    g0, g1 = R.gck._prolate_spheroidal_function(u)
    np.savez_compressed(os.path.join(HERE, 'ps_kernel.npz'), cgk_1D=cgk, corr128=corr128,
                        corr75x77=corr75, u=u, grdsf=g0, kernel=g1)

    cases = {
        'std_cube': dict(seed=11),
        'std_odd': dict(seed=12, image=63, cell=40.0),
        'std_onepol': dict(seed=13, n_pol=1),
        'std_continuum': dict(seed=14, chan_mode='continuum'),
    }
    for name, kw in cases.items():
        chan_mode = kw.pop('chan_mode', 'cube')
        o = small_obs(**kw)
        gp = {'image_size': [int(x) for x in o['image_size']], 'cell_size': [float(x) for x in o['cell_arcsec']],
              'chan_mode': chan_mode, 'fft_padding': 1.2}
        assert R.cp._check_grid_parms(gp)
        gp['oversampling'] = 100
        gp['support'] = 7
        cgk = R.gck._create_prolate_spheroidal_kernel_1D(100, 7)
        # data grid
        g = copy.deepcopy(gp)
        g['complex_grid'] = True
        g['do_psf'] = False
        grid, sw = R.sg._standard_grid_numpy_wrap(o['vis'], o['uvw'], o['weight'], o['freq'], cgk, g)
        # psf grid
        g = copy.deepcopy(gp)
        g['complex_grid'] = False
        g['do_psf'] = True
        g['do_imaging_weight'] = False
        pgrid, psw = R.sg._standard_grid_psf_numpy_wrap(o['uvw'], o['weight'], o['freq'], cgk, g)
        # weight density grid (unpadded), briggs factors and lookup
        g = copy.deepcopy(gp)
        g['image_size_padded'] = g['image_size']
        g['oversampling'] = 0
        g['support'] = 1
        g['do_psf'] = True
        g['complex_grid'] = False
        g['do_imaging_weight'] = True
        dgrid, dsw = R.sg._standard_grid_psf_numpy_wrap(o['uvw'], o['weight'], o['freq'], np.ones(1), g)
        res = dict(grid=grid, sum_weight=sw, psf_grid=pgrid, psf_sum_weight=psw,
                   density=dgrid, density_sum_weight=dsw,
                   image_size_padded=gp['image_size_padded'], cell_rad=gp['cell_size'],
                   chan_mode=np.array(chan_mode))
        for weighting, robust in [('briggs', 0.5), ('uniform', 0.0), ('briggs', -1.3)]:
            iwp = {'weighting': weighting, 'robust': robust}
            if chan_mode == 'cube':
                bf = R.sic._calculate_briggs_parms(dgrid, dsw, iwp)
                if weighting == 'uniform':
                    # synthesis_imaging_cube's uniform branch returns a
                    # (2,1,1,C,P) array the degridder cannot index;
                    # make_imaging_weight (make_imaging_weight.py:210-216)
                    # slices it to (2,C,P) = [[1...],[0...]].
                    bf = bf[:, 0, 0]
                iw = R.sg._standard_imaging_weight_degrid_numpy_wrap(
                    np.moveaxis(dgrid, (0, 1), (2, 3)), o['uvw'], o['weight'], bf, o['freq'], g)
                tag = f'{weighting}_{robust:+.1f}'
                res['briggs_factors_' + tag] = bf
                res['imaging_weight_' + tag] = iw
        # full image / psf pipeline (numpy helpers of synthesis_imaging_cube)
        if chan_mode == 'cube':
            g = copy.deepcopy(gp)
            _, corr = R.gck._create_prolate_spheroidal_kernel(100, 7, g['image_size_padded'])
            corr = R.rp._remove_padding(corr, g['image_size'])
            img, isw = R.sic._make_image(o['vis'].copy(), o['uvw'], o['weight'], o['freq'], cgk, g)
            img = R.sic.correct_image(img, isw[None, None, :, :], corr[:, :, None, None])
            g = copy.deepcopy(gp)
            psf, psw2 = R.sic._make_psf(o['uvw'], o['weight'], o['freq'], cgk, g)
            psf = R.sic.correct_image(psf, psw2[None, None, :, :], corr[:, :, None, None])
            res.update(image=img, image_sum_weight=isw, psf=psf, psf_sum_weight2=psw2)
        np.savez_compressed(os.path.join(HERE, f'{name}.npz'), vis=o['vis'], uvw=o['uvw'],
                            weight=o['weight'], freq=o['freq'], image_size=o['image_size'],
                            cell_arcsec=o['cell_arcsec'], **res)
        out[name] = {k: getattr(v, 'shape', None) for k, v in res.items()}
    for k, v in out.items():
        print(k, v)


def sin_pixel_offsets(field_phase_dir, phase_center, npad, cell_rad):
    """Pixel offsets of field centres in the SIN projection of the padded grid
    (the reference evaluates this with astropy's all_world2pix,
    make_gridding_convolution_function.py:331-347; restated here)."""
    a0, d0 = phase_center
    a, d = field_phase_dir[:, 0], field_phase_dir[:, 1]
    l = np.cos(d) * np.sin(a - a0)
    m = np.sin(d) * np.cos(d0) - np.cos(d) * np.sin(d0) * np.cos(a - a0)
    rad_to_deg = 180 / np.pi
    cdelt = np.asarray(cell_rad) * rad_to_deg
    return np.stack([np.rad2deg(l) / cdelt[0], np.rad2deg(m) / cdelt[1]], axis=1)


def phase_gradient(field_phase_dir, phase_center, npad, cell_rad, oversampling, resize_conv_size):
    pix_dist = sin_pixel_offsets(field_phase_dir, phase_center, npad, cell_rad)
    pix = -pix_dist * 2 * np.pi / (np.asarray(npad) * np.asarray(oversampling))
    c = np.asarray(resize_conv_size) // 2
    x = np.arange(-c[0], resize_conv_size[0] - c[0])
    y = np.arange(-c[1], resize_conv_size[1] - c[1])
    xg, yg = np.meshgrid(x, y, indexing='ij')
    return np.moveaxis(np.exp(1j * (xg[:, :, None] * pix[:, 0] + yg[:, :, None] * pix[:, 1])), 2, 0)


def mosaic_case(R):
    rng = np.random.default_rng(31)
    n_ant = 6
    enu = simulate.disk_layout(n_ant, 40.0, rng)
    T_per = 10
    n_field = 2
    T = T_per * n_field
    uvw = simulate.earth_rotation_uvw(enu, T, 60.0)
    a1, a2 = simulate.baseline_pairs(n_ant)
    B = uvw.shape[1]
    freq = np.array([100.0e9, 100.6e9, 101.2e9])
    C, P = len(freq), 2
    vis = (rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P))).astype(np.complex64)
    iw = rng.uniform(0.5, 2.0, (T, B, C, P))
    field = np.repeat(np.arange(n_field), T_per)[:, None].repeat(B, axis=1).astype(np.int64)
    field[3, 4] = -1                        # a row without a field is skipped
    dec0 = np.deg2rad(-30.0)
    phase_center = np.array([np.deg2rad(150.0), dec0])
    off = np.deg2rad(20.0 / 3600)
    field_phase_dir = np.array([[phase_center[0] - off / np.cos(dec0) / 2, dec0],
                                [phase_center[0] + off / np.cos(dec0) / 2, dec0]])
    gp = {'image_size': [64, 64], 'cell_size': [2.0, 2.0], 'chan_mode': 'cube', 'fft_padding': 1.2}
    assert R.cp._check_grid_parms(gp)
    gcf = {'function': 'casa_airy', 'list_dish_diameters': [12.0], 'list_blockage_diameters': [0.75],
           'unique_ant_indx': [0] * n_ant, 'oversampling': [4, 4], 'max_support': [15, 15],
           'freq_chan': list(freq), 'pol': [0, 1], 'chan_tolerance_factor': 0.005}
    assert R.cp._check_gcf_parms(gcf)
    gcf['basline_ant'] = np.stack([a1, a2], axis=1)
    gcf['resize_conv_size'] = (gcf['max_support'] + 1) * gcf['oversampling']
    cfb_map, pb_pairs = R.gcf.create_cf_baseline_map(gcf['unique_ant_indx'], gcf['basline_ant'], 1)
    cfc_map, pb_freq = R.gcf.create_cf_chan_map(freq, gcf['chan_tolerance_factor'])
    cfp_map = np.zeros(P, dtype=int)
    gcf['ipower'] = 1
    bp = R.gcf.make_baseline_patterns(pb_freq, np.array([0]), pb_pairs, R.pb._casa_airy_disk_rorder, gcf, gp)
    gcf['ipower'] = 2
    bw = R.gcf.make_baseline_patterns(pb_freq, np.array([0]), pb_pairs, R.pb._casa_airy_disk_rorder, gcf, gp)
    ck_full = np.real(np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(bp, axes=(3, 4)), axes=(3, 4)), axes=(3, 4)))
    wk_full = np.real(np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(bw, axes=(3, 4)), axes=(3, 4)), axes=(3, 4)))
    ck, wk, support = R.gcf.resize_and_calc_support(ck_full, wk_full, gcf, gp)
    pg = phase_gradient(field_phase_dir, phase_center, gp['image_size_padded'], gp['cell_size'],
                        gcf['oversampling'], gcf['resize_conv_size'])
    g = copy.deepcopy(gp)
    g.update({'oversampling': gcf['oversampling'], 'complex_grid': True, 'do_psf': False,
              'field_id': np.arange(n_field)})
    grid, sw = R.ag._aperture_grid_numpy_wrap(vis, uvw, iw, field, cfb_map, cfc_map, cfp_map, ck, support, pg, freq, g)
    g['do_psf'] = True
    pgrid, psw = R.ag._aperture_psf_grid_numpy_wrap(uvw, iw, field, cfb_map, cfc_map, cfp_map, ck, support, pg, freq, g)
    wgrid, wsw = R.ag._aperture_weight_grid_numpy_wrap(uvw, iw, field, cfb_map, cfc_map, cfp_map, wk, support, pg,
                                                       freq, g)
    np.savez_compressed(os.path.join(HERE, 'mosaic.npz'), vis=vis, uvw=uvw, imaging_weight=iw, field=field,
                        freq=freq, antenna1=a1, antenna2=a2, field_phase_dir=field_phase_dir,
                        phase_center=phase_center, image_size=np.array(gp['image_size']),
                        cell_arcsec=np.array([2.0, 2.0]), oversampling=gcf['oversampling'],
                        max_support=gcf['max_support'], cf_baseline_map=cfb_map, cf_chan_map=cfc_map,
                        cf_pol_map=cfp_map, pb_freq=pb_freq, baseline_pb=bp, weight_baseline_pb=bw,
                        conv_kernel=ck, weight_conv_kernel=wk, support=support, phase_gradient=pg,
                        grid=grid, sum_weight=sw, psf_grid=pgrid, psf_sum_weight=psw,
                        weight_grid=wgrid, weight_sum_weight=wsw)
    print('mosaic', 'support', support.ravel(), 'pb_freq', pb_freq, 'ck', ck.shape, 'grid', grid.shape,
          'sw', sw.ravel()[:4])


def rotate_case():
    """direction_rotate: the reference's calc_rotation_mats, apply_rotation_matrix
    and apply_phasor (direction_rotate.py:127-248) on a 3-field case, for both
    common_tangent_reprojection and both single_precision settings."""
    refshim.install()
    import importlib
    dr = importlib.import_module('ngcasa.imaging.direction_rotate')
    rng = np.random.default_rng(11)
    T, B, C, P = 10, 6, 3, 2
    field_of_row = np.array([5, 5, 5, 5, 2, 2, 2, 9, 9, 9])
    field_id = np.repeat(field_of_row[:, None], B, axis=1)
    uvw = rng.uniform(-2000.0, 2000.0, (T, B, 3))
    uvw[:, :, 2] *= 0.1
    vis = (rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P))).astype(np.complex64)
    freq = 100.0e9 + np.arange(C) * 0.8e9
    new_pc = [1.2, -0.4]
    all_ids = np.array([2, 5, 7, 9])
    phase_dir = np.array([[1.2 + 3e-4, -0.4 - 2e-4], [1.2 - 5e-4, -0.4 + 1e-4], [0.3, 0.2], [1.2 + 1e-4, -0.4 + 6e-4]])

    class Sel:
        def __init__(self, a):
            self.values = a

        def __getitem__(self, k):
            return Sel(self.values[k])

    class PhaseDir:
        def sel(self, field_id, d1):
            idx = [int(np.where(all_ids == f)[0][0]) for f in field_id]
            return Sel(phase_dir[idx])

    class Obj:
        pass

    vds = Obj()
    vds.FIELD_ID = field_id
    fds = Obj()
    fds.PHASE_DIR = PhaseDir()
    out = dict(uvw=uvw, vis=vis, freq=freq, field_id=field_id, new_phase_center=np.array(new_pc),
               field_ids=all_ids, phase_dir=phase_dir)
    for ctr in (True, False):
        parms = {'new_phase_center': new_pc, 'common_tangent_reprojection': ctr, 'single_precision': True}
        rotmat, phase_rot, rot_ids = dr.calc_rotation_mats(vds, fds, parms)
        uvw_rot = dr.apply_rotation_matrix(uvw, field_id[:, :, None], rotmat, rot_ids)
        tag = 'ctr' if ctr else 'noctr'
        out[f'rotmat_{tag}'] = rotmat
        out[f'phase_rotation_{tag}'] = phase_rot
        out[f'rot_field_id_{tag}'] = rot_ids
        out[f'uvw_rot_{tag}'] = uvw_rot
        for single in (True, False):
            v = dr.apply_phasor(vis, uvw_rot[:, :, :, None], field_id[:, :, None, None], freq[None, None, :, None],
                                phase_rot, rot_ids, ctr, single)
            out[f'vis_rot_{tag}_{"single" if single else "double"}'] = v
    np.savez_compressed(os.path.join(HERE, 'rotate.npz'), **out)


def clean_case():
    """Hogbom minor cycle: the reference's _clean_jit (deconvolve_point_clean.py
    :174-236, as written) on dirty images and PSFs of a few point sources."""
    refshim.install()
    import importlib
    import sys as _sys
    import types as _types
    for name in ('ngcasa.deconvolution',):
        if name not in _sys.modules:
            m = _types.ModuleType(name)
            m.__path__ = [os.path.join(refshim._reference_root(), 'ngcasa/deconvolution')]
            _sys.modules[name] = m
    nb = _sys.modules['numba']
    nb.u4 = np.uint32
    dc = importlib.import_module('ngcasa.deconvolution.deconvolve_point_clean')
    rng = np.random.default_rng(13)
    nx, ny, P = 40, 36, 2
    x = np.arange(2 * nx)[:, None] - nx
    y = np.arange(2 * ny)[None, :] - ny
    psf1 = np.exp(-(x ** 2 + y ** 2) / 8.0) * np.cos(0.3 * x) + 0.02 * np.cos(0.9 * y)
    psf = np.stack([psf1, psf1 * 0.9 + 0.1 * np.exp(-(x ** 2 + y ** 2) / 3.0)], axis=-1)[:, :, None, None, :]
    dirty = np.zeros((nx, ny, 1, 1, P))
    for p in range(P):
        for _ in range(4):
            px, py, a = rng.integers(3, nx - 3), rng.integers(3, ny - 3), rng.uniform(0.5, 2.0)
            dirty[:, :, 0, 0, p] += a * psf[nx - px:2 * nx - px, ny - py:2 * ny - py, 0, 0, p]
    dirty += 0.01 * rng.standard_normal(dirty.shape)
    out = dict(dirty=dirty, psf=psf)
    for gain, thr, niter in ((0.1, 0.05, 60), (0.3, 0.0, 25)):
        res = dirty.copy()
        mdl = np.zeros(res.shape)
        dc._clean_jit(res, mdl, psf, gain, thr, niter)
        out[f'model_g{gain}_n{niter}'] = mdl
        out[f'residual_g{gain}_n{niter}'] = res
    np.savez_compressed(os.path.join(HERE, 'clean.npz'), **out)


def beam_case():
    """PSF beam fit: the reference's casa_fit (cngi/image/fit_gaussian.py) on the
    std_cube PSF planes (the fit make_psf attaches as PSF_FIT)."""
    refshim.install()
    import importlib
    fg = importlib.import_module('cngi.image.fit_gaussian')
    d = dict(np.load(os.path.join(HERE, 'std_cube.npz')))
    psf = d['psf'][:, :, None, :, :]                 # (l, m, time, chan, pol)
    delta = np.array([-45.0, 45.0])                   # arcsec; l's step is negative
    parms = fg.casa_fit(psf, np.array([9, 9]), np.array([9, 9]), 0.35, delta)
    np.savez_compressed(os.path.join(HERE, 'beam.npz'), psf=psf, delta=delta, ellipse_parms=parms)


def sic_case():
    """synthesis_imaging_cube: the reference's per-chunk function
    (_synthesis_imaging_cube_std_chunk) on a flagged small cube with natural
    weighting (its images, sums of weights, primary beams and PSF fit), and,
    for Briggs 0.5, its helpers composed as the function documents it (the
    imaging weights of _make_imaging_weight_chunk applied to the PSF and the
    image; the reference's chunk function grids with the natural weights)."""
    R = refshim.modules()
    rng = np.random.default_rng(31)
    enu = simulate.disk_layout(8, 300.0, rng)
    uvw = simulate.earth_rotation_uvw(enu, 24, 120.0)
    freq = 1.0e9 + np.arange(3) * 5.0e7
    T, B = uvw.shape[:2]
    vis = simulate.point_source_vis(uvw, freq, np.deg2rad(np.array([0.02, -0.05, 0.1])),
                                    np.deg2rad(np.array([0.03, 0.01, -0.07])), [1.0, 0.5, 0.25], 2, 0.1,
                                    rng).astype(np.complex64)
    weight = rng.uniform(0.5, 2.0, (T, B, 3, 2))
    weight[rng.random(weight.shape) < 0.02] = 0.0
    flag = (rng.random((T, B, 3, 2)) < 0.08).astype(np.int8)
    uvw[3, 2, :] = np.nan
    gp = {'image_size': [64, 64], 'cell_size': [45.0, 45.0], 'chan_mode': 'cube', 'fft_padding': 1.2}
    assert R.cp._check_grid_parms(gp)
    pbp = {'function': 'casa_airy', 'list_dish_diameters': [12.0, 7.0], 'list_blockage_diameters': [0.75, 0.75]}
    out = dict(vis=vis, uvw=uvw, weight=weight, flag=flag, freq=freq, image_size=np.array([64, 64]),
               cell_arcsec=np.array([45.0, 45.0]), dish=np.array(pbp['list_dish_diameters']),
               blockage=np.array(pbp['list_blockage_diameters']))
    parms = {'grid_parms': copy.deepcopy(gp), 'imaging_weights_parms': {'weighting': 'natural'},
             'pb_parms': copy.deepcopy(pbp)}
    img, isw, psf, psw, pb, elp = R.sic._synthesis_imaging_cube_std_chunk(vis.copy(), uvw, weight, flag, freq, parms)
    out.update(natural_image=img, natural_image_sum_weight=isw, natural_psf=psf, natural_psf_sum_weight=psw,
               natural_pb=pb, natural_restore_parms=elp)
    # Briggs 0.5: the helpers as documented (weights applied)
    g = copy.deepcopy(gp)
    g['oversampling'], g['support'] = 100, 7
    cgk = R.gck._create_prolate_spheroidal_kernel_1D(100, 7)
    _, corr = R.gck._create_prolate_spheroidal_kernel(100, 7, g['image_size_padded'])
    corr = R.rp._remove_padding(corr, g['image_size'])
    iw = R.sic._make_imaging_weight_chunk(uvw, weight, freq, copy.deepcopy(g), {'weighting': 'briggs', 'robust': 0.5})
    vf = vis.copy()
    vf[flag == 1] = np.nan
    bimg, bisw = R.sic._make_image(vf, uvw, iw, freq, cgk, copy.deepcopy(g))
    bimg = R.sic.correct_image(bimg, bisw[None, None, :, :], corr[:, :, None, None])
    bpsf, bpsw = R.sic._make_psf(uvw, iw, freq, cgk, copy.deepcopy(g))
    bpsf = R.sic.correct_image(bpsf, bpsw[None, None, :, :], corr[:, :, None, None])
    out.update(briggs_imaging_weight=iw, briggs_image=bimg, briggs_image_sum_weight=bisw, briggs_psf=bpsf,
               briggs_psf_sum_weight=bpsw)
    np.savez_compressed(os.path.join(HERE, 'sic.npz'), **out)
    print({k: getattr(v, 'shape', None) for k, v in out.items()})


def time_reference(n_time=20, n_chan=4):
    """Time the reference's own _standard_grid_numpy_wrap (pure Python under
    refshim's identity numba.jit) on a subsample of the small standard cube
    (27 antennas, 351 baselines, 2 pols): the supplementary CPU figure beside
    the C restatement. Prints microseconds per visibility (time, baseline,
    chan, pol sample). Writes no fixture."""
    import time
    R = refshim.modules()
    obs = simulate.config_standard_small(seed=1)
    vis = np.ascontiguousarray(obs.vis[:n_time, :, :n_chan])
    w = np.ascontiguousarray(obs.weight[:n_time, :, :n_chan]).astype(np.float64)
    uvw = np.ascontiguousarray(obs.uvw[:n_time])
    freq = np.asarray(obs.freq[:n_chan])
    gp = {'image_size': [int(x) for x in obs.image_size], 'cell_size': [float(x) for x in obs.cell_arcsec],
          'chan_mode': 'cube', 'fft_padding': 1.2}
    assert R.cp._check_grid_parms(gp)
    gp.update({'oversampling': 100, 'support': 7, 'complex_grid': True, 'do_psf': False})
    cgk = R.gck._create_prolate_spheroidal_kernel_1D(100, 7)
    t0 = time.perf_counter()
    R.sg._standard_grid_numpy_wrap(vis, uvw, w, freq, cgk, gp)
    dt = time.perf_counter() - t0
    n = vis.size
    print(f'reference _standard_grid_numpy_wrap (pure Python, identity numba.jit): {n} vis '
          f'({n_time} times x {vis.shape[1]} baselines x {n_chan} chan x {vis.shape[3]} pols) in {dt:.2f} s = '
          f'{dt / n * 1e6:.1f} us/vis = {n / dt / 1e6:.4f} Mvis/s, one core')


if __name__ == '__main__':
    if len(sys.argv) > 1 and sys.argv[1] == 'time_reference':
        time_reference()
        sys.exit(0)
    if len(sys.argv) == 1 or sys.argv[1] == 'standard':
        main()
    if len(sys.argv) == 1 or sys.argv[1] == 'mosaic':
        mosaic_case(refshim.modules())
    if len(sys.argv) == 1 or sys.argv[1] == 'rotate':
        rotate_case()
    if len(sys.argv) == 1 or sys.argv[1] == 'clean':
        clean_case()
    if len(sys.argv) == 1 or sys.argv[1] == 'beam':
        beam_case()
    if len(sys.argv) == 1 or sys.argv[1] == 'sic':
        sic_case()
