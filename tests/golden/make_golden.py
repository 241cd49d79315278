"""Generate the golden fixtures for the standard-gridder path.

Run in a container that has the reference checkout (default
/root/reference, override with CNGI_REFERENCE_ROOT):

    python tests/golden/make_golden.py

It runs the reference's own per-chunk functions -- _standard_grid_numpy_wrap,
_standard_grid_psf_numpy_wrap, _standard_imaging_weight_degrid_numpy_wrap,
synthesis_imaging_cube's numpy imaging helpers, the prolate-spheroidal
kernel builders and the GCF helpers -- through ``refshim`` on small seeded
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


if __name__ == '__main__':
    main()
