"""One rank of the multi-process imaging tests (launched by test_distributed.py).

argv: rank world port out_dir scenario core
  scenario: 'continuum' | 'cube' | 'fail_mark' | 'fail_exit'
  core: 'oracle' -- the per-rank gridding/FFT core is replaced by the oracle
        (CPU, test infrastructure: the host-side sharding, sums and
        normalisation are what is under test); 'gpu' -- the CUDA path.
Each rank writes out_dir/rank<r>.npz with its results, or rank<r>.err with
the type and text of the exception it raised.
"""
import datetime
import os
import sys
import traceback

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import numpy as np  # noqa: E402

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def _np(x):
    x = x.values if hasattr(x, 'values') and not isinstance(x, np.ndarray) else x
    return np.asarray(x.detach().cpu().numpy() if hasattr(x, 'detach') else x)


def use_oracle_core():
    """Route the per-rank imaging core through the oracle (CPU)."""
    import torch
    from oracle import imaging as O
    from cngi_prototype_gb300.imaging._imaging_utils import _pipeline

    def image_cube(vis, uvw, iw, freq, gp, do_psf, normalize=True):
        npad = np.asarray(gp['image_size_padded'])
        corr = O.remove_padding(O.create_prolate_spheroidal_correction(npad), gp['image_size'])
        cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
        grid, sw = O.standard_grid(None if do_psf else _np(vis), _np(uvw), _np(iw).astype(np.float64),
                                   np.asarray(freq), cgk, npad, gp['cell_size'], 7, 100, do_psf, False,
                                   not do_psf, gp.get('chan_mode', 'cube'))
        img = O.uncorrected_image(grid, gp['image_size'])
        return O.correct_image(img, sw if normalize else np.ones_like(sw), corr), sw

    def imaging_weights(uvw, weight, freq, gp, iwp, density_reduce=None):
        dens, sw = O.grid_weight_density(_np(uvw), _np(weight).astype(np.float64), np.asarray(freq), gp)
        if density_reduce is not None:
            d, s = density_reduce(torch.from_numpy(dens), torch.from_numpy(sw))
            dens, sw = d.numpy(), s.numpy()
        f = O.calculate_briggs_parms(np.moveaxis(dens, (0, 1), (2, 3)), sw, iwp)
        iw = O.standard_imaging_weight_degrid(np.moveaxis(dens, (0, 1), (2, 3)), _np(uvw), _np(weight), f,
                                              np.asarray(freq), np.asarray(gp['image_size']), gp['cell_size'],
                                              gp.get('chan_mode', 'cube'))
        return torch.from_numpy(iw)

    _pipeline.image_cube = image_cube
    _pipeline.imaging_weights = imaging_weights


def observation():
    from cngi_prototype_gb300 import xds
    d = dict(np.load(os.path.join(GOLDEN, 'std_cube.npz')))
    ds = xds.vis_dataset(d['uvw'], d['vis'], d['weight'], d['freq'], time=np.arange(d['uvw'].shape[0]) * 10.0)
    gp = {'image_size': [int(x) for x in d['image_size']], 'cell_size': [float(x) for x in d['cell_arcsec']],
          'phase_center': [0.0, 0.0]}
    return xds.mxds({'xds0': ds}), gp


def run(mx, gp, chan_mode, fn_weight, fn_psf, fn_image, group=None):
    """Briggs weights, PSF and image of mx; returns a dict of arrays."""
    from cngi_prototype_gb300 import xds
    g = dict(gp, chan_mode=chan_mode)
    kw = {} if group is None else {'group': group}
    m2 = fn_weight(mx, {'weighting': 'briggs', 'robust': 0.3}, g, {'xds': 'xds0'}, **kw)
    psf = fn_psf(m2, xds.Dataset(), g, {'xds': 'xds0'}, {}, **kw)
    img = fn_image(m2, xds.Dataset(), g, {'xds': 'xds0'}, {}, **kw)
    return {'imaging_weight': m2.attrs['xds0']['IMAGING_WEIGHT'].values, 'psf': psf['PSF'].values,
            'psf_sum_weight': psf['PSF_SUM_WEIGHT'].values, 'image': img['IMAGE'].values,
            'sum_weight': img['SUM_WEIGHT'].values, 'time': img.coords['time'].values}


def main():
    rank, world, port = int(sys.argv[1]), int(sys.argv[2]), int(sys.argv[3])
    out_dir, scenario, core = sys.argv[4], sys.argv[5], sys.argv[6]
    import torch.distributed as dist
    from cngi_prototype_gb300.imaging import distributed as D
    timeout = datetime.timedelta(seconds=6 if scenario.startswith('fail') else 60)
    try:
        if core == 'oracle':
            use_oracle_core()
        dist.init_process_group('gloo', init_method=f'tcp://127.0.0.1:{port}', rank=rank, world_size=world,
                                timeout=timeout)
        store = dist.FileStore(os.path.join(out_dir, 'store'), world)
        group = D.ShardGroup(store=store, timeout_s=timeout.total_seconds())
        mx, gp = observation()
        chan_mode = 'cube' if scenario == 'cube' else 'continuum'
        shard = D.shard_vis(mx, {'xds': 'xds0'}, chan_mode, rank, world)
        if scenario == 'fail_mark' and rank == 1:
            group.fail('input file missing')
            os._exit(0)
        if scenario == 'fail_exit' and rank == 1:
            os._exit(0)
        res = run(shard, gp, chan_mode, D.make_imaging_weight_sharded, D.make_psf_sharded, D.make_image_sharded,
                  group)
        np.savez(os.path.join(out_dir, f'rank{rank}.npz'), **res)
    except Exception as e:  # reported to the test through the file
        with open(os.path.join(out_dir, f'rank{rank}.err'), 'w') as f:
            f.write(type(e).__name__ + '\n' + str(e) + '\n' + traceback.format_exc())
    finally:
        if dist.is_initialized() and not scenario.startswith('fail'):
            dist.destroy_process_group()
    os._exit(0)


if __name__ == '__main__':
    main()
