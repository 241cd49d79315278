#!/usr/bin/env python
"""Gridding throughput of the large-cube imaging workload on GB300.

Workload (one step): DATA-mode convolutional gridding of the whole large
cube through ngg_grid_ps -- 64 antennas in a 3-arm log spiral of 2.5 km
radius (2016 baselines), 1024 x 8 s integrations, 256 channels over
1.0-1.5 GHz, RR/LL (1.057e9 visibilities, 5% flagged), Briggs robust 0.5
imaging weights (computed on the GPU before timing), 4096^2 image at 1 arcsec
(4915^2 padded grid), prolate-spheroidal support 7, oversampling 100.
Synthetic seeded data stand in for an observation (no dataset offline).

Prints one JSON line. `value` = Mvis/s with inputs resident in HBM; `e2e` =
the same call fed from pinned host buffers (H2D of the step's inputs and D2H
of the resulting grid inside the timed region). The inputs (12.7 GB) exceed
L2, so no flush is needed between steps. `roofline` is the tile-accumulation
kernel against the measured HBM copy bandwidth; `cpu_baseline` is the C FP64
restatement of the reference gridder on all host cores on a channel sample.

--impl reference times the CPU restatement of the reference's gridder alone.
Multi-GPU (torchrun): the large cube is channel-partitioned, each rank grids
its channel shard (weak scaling, no collective on the data path); the other
workloads run one replica per rank. Rank 0 prints the line.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'Mvis/s gridded & err vs FP64; learned vs table GCF mosaic time at 1e-3 error'
WORKLOAD = 'large_cube_briggs_grid'


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=5)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='ngg', choices=['ngg', 'reference'])
    p.add_argument('--n-time', type=int, default=1024)
    p.add_argument('--n-chan', type=int, default=256)
    p.add_argument('--image-size', type=int, default=4096,
                   help='large_cube: image side in pixels, cell 4096/N arcsec (the same field); smaller sizes are '
                        'profiling cases of the same kernels, not the headline workload')
    p.add_argument('--cpu-chans', type=int, default=16, help='channels in the CPU-baseline sample')
    p.add_argument('--no-e2e', action='store_true')
    p.add_argument('--no-cpu', action='store_true')
    p.add_argument('--no-err', action='store_true')
    p.add_argument('--workload', default='large_cube',
                   choices=['large_cube', 'mosaic', 'standard_small', 'degrid', 'cycle'],
                   help='large_cube (default, the headline), mosaic (aperture-projection imaging, table and '
                        'learned GCF), standard_small (the small cube through the whole API), degrid (the '
                        'differentiable degrid/grid pair), cycle (direction_rotate, Hogbom CLEAN and '
                        'predict_modelvis_image)')
    p.add_argument('--mosaic-chans', type=int, default=16)
    p.add_argument('--mosaic-pointings', type=int, default=49)
    p.add_argument('--no-learned', action='store_true')
    p.add_argument('--no-mosaic', action='store_true', help='large_cube: skip the mosaic (table vs learned GCF) record')
    p.add_argument('--no-others', action='store_true',
                   help='large_cube: skip the small-cube and degrid/grid records')
    p.add_argument('--learned-steps', type=int, default=30000)
    p.add_argument('--learned-freqs', type=int, default=64)
    return p.parse_args()


def dist_env():
    return int(os.environ.get('RANK', 0)), int(os.environ.get('WORLD_SIZE', 1)), int(os.environ.get('LOCAL_RANK', 0))


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


class Clocks:
    """nvidia-smi sampler for the timed region (SM clock, throttle reasons)."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index):
        self.path = os.path.join(tempfile.gettempdir(), f'ngg_clocks_{os.getpid()}.csv')
        self.idx = gpu_index
        self.p = None

    def start(self):
        try:
            self.f = open(self.path, 'w')
            self.p = subprocess.Popen(['nvidia-smi', '-i', str(self.idx), '--query-gpu=' + self.Q,
                                       '--format=csv,noheader,nounits', '-lms', '200'], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], 0.0, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in open(self.path):
            parts = [x.strip() for x in line.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == 'active':
                    reasons.add(n)
        if not sm:
            return None
        return {'sm_mhz': float(np.median(sm)), 'sm_max_mhz': smax, 'reasons': sorted(reasons), 'samples': len(sm)}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def oracle_sample(uvw, vis_s, w_s, freq_s, cgk, npad, cell, threads):
    """Time the C FP64 restatement of the reference gridder on a channel sample."""
    from oracle import cbind
    cbind.build()
    t0 = time.perf_counter()
    g, sw = cbind.grid('data', vis_s, uvw, w_s, freq_s, cgk, 7, 100, npad, cell, 'cube', threads)
    dt = time.perf_counter() - t0
    return g, sw, dt


def large_cube_config(T, B, C, P, world, image_size=4096):
    """The `config` of the large-cube line (both arms)."""
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    gp = {'image_size': [image_size, image_size], 'cell_size': [4096.0 / image_size] * 2}
    _check_grid_parms(gp)
    return {'workload': WORKLOAD, 'n_time': T, 'n_baseline': B, 'n_chan': C, 'n_pol': P, 'n_vis': T * B * C * P,
            'image_size': image_size, 'grid': int(gp['image_size_padded'][0]), 'cell_arcsec': 4096.0 / image_size,
            'weighting': 'briggs 0.5', 'support': 7,
            'oversampling': 100, 'flags': 0.05,
            'l2': f'inputs ({T * B * C * P * 12 / 1e9:.1f} GB) larger than L2; no flush',
            'parallelism': f'channel shard x{world} (no exchange)'}


def large_cube_obs(args, rank, world, device):
    """The synthetic large cube of this rank (seed 2; rank r holds channels
    [r*n_chan, (r+1)*n_chan) of one N*n_chan-channel cube)."""
    from cngi_prototype_gb300 import simulate
    return simulate.config_large_cube(seed=2, n_time=args.n_time, n_chan=args.n_chan * world, vis_device=device,
                                      image_size=args.image_size,
                                      chan_range=(rank * args.n_chan, (rank + 1) * args.n_chan))


def reference_arm(args, rank):
    """The reference's gridder, restated in C (FP64, OpenMP over channels),
    on all host threads: the same large cube as the GPU arm (same seed, same
    5% flags) with the same Briggs 0.5 imaging weights, computed from the
    natural weights by the oracle's restatement of make_imaging_weight
    (cube mode: per-channel density, so a channel sample's weights are the
    whole cube's). Each step grids a bounded channel sample."""
    if rank != 0:
        return
    import torch
    from oracle import cbind
    from oracle import imaging as O
    from cngi_prototype_gb300.imaging._imaging_utils import _gridding_convolutional_kernels as G
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    device = 'cuda' if torch.cuda.is_available() else 'cpu'   # synthesis only (torch); the gridding is on the CPU
    obs = large_cube_obs(args, 0, 1, device)
    gp = {'image_size': list(obs.image_size), 'cell_size': list(obs.cell_arcsec)}
    _check_grid_parms(gp)
    cgk = G._create_prolate_spheroidal_kernel_1D(100, 7)
    T, B, C, P = obs.vis.shape
    nc = min(args.cpu_chans, C)
    vis = obs.vis[:, :, :nc].cpu().numpy()
    w_nat = obs.weight[:, :, :nc].cpu().numpy().astype(np.float64)
    del obs['vis'], obs['weight']
    if device == 'cuda':
        torch.cuda.empty_cache()
    freq = obs.freq[:nc]
    threads = cpu_threads()
    # Briggs 0.5 imaging weights (untimed: make_image takes them as input)
    dens, dsw = cbind.grid('density', None, obs.uvw, w_nat, freq, np.ones(1), 1, 0, gp['image_size'],
                           gp['cell_size'], 'cube', threads)
    dens_uvcp = np.moveaxis(dens, (0, 1), (2, 3))
    fac = O.calculate_briggs_parms(dens_uvcp, dsw, {'weighting': 'briggs', 'robust': 0.5})
    iw = cbind.weight_degrid(dens_uvcp, obs.uvw, w_nat, fac, freq, gp['image_size'], gp['cell_size'], 'cube',
                             threads)
    del dens, dens_uvcp
    times = []
    for k in range(args.warmup + args.steps):
        _, _, dt = oracle_sample(obs.uvw, vis, iw, freq, cgk, gp['image_size_padded'], gp['cell_size'], threads)
        if k >= args.warmup:
            times.append(dt)
    nvis = T * B * nc * P
    v = nvis / float(np.mean(times)) / 1e6
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'Mvis/s', 'n_gpus': args.gpus,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': float(np.mean(times)) * 1e3,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
        'config': large_cube_config(T, B, C, P, 1, args.image_size),
        'cpu_baseline': {'value': v, 'unit': 'Mvis/s', 'cores': threads, 'kind': 'port',
                         'sample': f'channels 0-{nc - 1} of the {C}-channel cube (same seed, flags and Briggs 0.5 '
                                   f'weights as the GPU arm): all {T}x{B} rows x {P} pols ({nvis} vis) per step, C '
                                   f'FP64 restatement of _standard_grid_jit, OpenMP over channels, complex128 grid'},
        'e2e': {'value': v, 'unit': 'Mvis/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line), flush=True)


MOSAIC_WORKLOAD = 'mosaic_table_gcf'


def _mosaic_inputs(args, seed, vis_device):
    from cngi_prototype_gb300 import simulate, xds
    obs = simulate.config_mosaic(seed=seed, n_chan=args.mosaic_chans, n_pointing=args.mosaic_pointings,
                                 vis_device=vis_device)
    gp_user = {'image_size': list(obs.image_size), 'cell_size': list(obs.cell_arcsec), 'fft_padding': 1.2}
    gcf_parms = {'function': 'casa_airy', 'list_dish_diameters': [obs.dish], 'list_blockage_diameters': [obs.blockage],
                 'unique_ant_indx': [0] * (int(max(obs.antenna1.max(), obs.antenna2.max())) + 1),
                 'oversampling': list(obs.oversampling),
                 'max_support': list(obs.max_support), 'phase_center': obs.phase_center,
                 'chan_tolerance_factor': 0.005}
    field_ds = xds.Dataset({'PHASE_DIR': (('field_id', 'poly_id', 'pair'), obs.field_phase_dir[:, None, :])},
                           coords={'field_id': ('field_id', np.arange(len(obs.field_phase_dir)))})
    return obs, gp_user, gcf_parms, field_ds


def _mosaic_mxds(obs, vis, weight, field_ds):
    from cngi_prototype_gb300 import xds
    vds = xds.vis_dataset(obs.uvw, vis, weight, obs.freq, field_id=obs.field, antenna1=obs.antenna1,
                          antenna2=obs.antenna2)
    vds.attrs['data_groups'][0]['0']['imaging_weight'] = 'DATA_WEIGHT'
    return xds.mxds({'xds0': vds}, FIELD=field_ds)


def _dirty(grid_fft, sw, chans):
    """Re(FFT^-1) of FFT-layout planes / sum_weight for a few channels (numpy FP64)."""
    out = []
    for c in chans:
        g = grid_fft[c].cpu().numpy().astype(np.complex128)
        im = np.fft.fftshift(np.fft.ifft2(g), axes=(1, 2)).real
        s = sw[c].cpu().numpy()
        out.append(im / np.where(s == 0, 1.0, s)[:, None, None])
    return np.stack(out)


def learned_leg(args, obs, gcf, gp, vis_d, uvw_d, w_d, f_d, fidx_d, sl_d, g_tab, sw_tab, ms_tab, t_gcf, steps):
    """Learned GCF against the table GCF on the mosaic workload: train on the
    GCFs the method generates (GPU), grid with per-channel tables synthesised
    on the tensor cores, compare images with the table path (reference PB
    channels) and with a table built at every channel's exact frequency."""
    import torch
    from cngi_prototype_gb300 import _lib
    from cngi_prototype_gb300.imaging.learned_gcf import LearnedGCF
    from cngi_prototype_gb300.imaging.make_gridding_convolution_function import gcf_tables
    T, B, C, P = vis_d.shape
    npad, cell = gp['image_size_padded'], gp['cell_size']
    os_ = np.asarray(obs.oversampling)
    bw = float(obs.freq.max() - obs.freq.min())
    band = (float(obs.freq.min()) - 0.1 * bw, float(obs.freq.max()) + 0.1 * bw)   # channels inside, not at the edge
    lg = LearnedGCF.fit('casa_airy', obs.dish, obs.blockage, band, gp, os_, obs.max_support,
                        n_freq=args.learned_freqs, steps=args.learned_steps, batch=65536)

    def step_learned():
        return lg.grid(vis_d, uvw_d, w_d, f_d, fidx_d, sl_d, npad, cell, layout='fft')

    for _ in range(2):
        gl, swl = step_learned()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        gl, swl = step_learned()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_l = e0.elapsed_time(e1) / steps
    # the tensor-core synthesis alone: every (channel, offset, tap) of the tables
    S = int(lg.support_for(obs.freq).max()) | 1
    n_eval = C * (int(os_[0]) + 1) * (int(os_[1]) + 1) * S * S
    zz = torch.zeros((n_eval, 3), dtype=torch.float32, device='cuda')
    _lib.mlp_forward(lg.params, zz[:1024], tensor_cores=True)
    torch.cuda.synchronize()
    e0.record(stream)
    _lib.mlp_forward(lg.params, zz, tensor_cores=True)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_tc = e0.elapsed_time(e1)
    flop = 2.0 * 3 * 4 * 64 * 64 * n_eval       # 4 layers, split-BF16 = 3 MMAs per product
    del zz
    # exact-frequency table path (one CF per channel)
    ck_x, _, sup_x = gcf_tables('casa_airy', [obs.dish], [obs.blockage], np.array([[0, 0]]), obs.freq, gp, os_,
                                obs.max_support, 0.025)
    cfc = torch.arange(C, dtype=torch.int32, device='cuda')
    zb = torch.zeros(B, dtype=torch.int32, device='cuda')
    zp = torch.zeros(P, dtype=torch.int32, device='cuda')
    gx, swx = _lib.grid_gcf(vis_d, uvw_d, w_d, f_d, fidx_d, zb, cfc, zp, ck_x, torch.as_tensor(sup_x.reshape(1, C, 1, 2),
                            dtype=torch.int32, device='cuda'), sl_d, npad, cell, os_, layout='fft')
    chans = sorted(set([0, C // 2, C - 1]))
    i_tab, i_x, i_l = _dirty(g_tab, sw_tab, chans), _dirty(gx, swx, chans), _dirty(gl, swl, chans)
    pk = np.abs(i_x).max()
    rel = lambda a, b: float(np.abs(a - b).max() / pk)
    return {
        'train': {'n_samples': lg.info['n_samples'], 'n_freq': lg.info['n_freq'], 'steps': lg.info['steps'],
                  'batch': lg.info['batch'], 'data_s': lg.info['data_s'], 'train_s': lg.info['train_s'],
                  'final_loss': lg.info['final_loss'], 'kernels': 'ngg_mlp_train (own FP32 fwd/bwd/Adam)'},
        'ms_learned_grid': ms_l, 'ms_table_grid': ms_tab, 'gcf_generation_s': t_gcf,
        'speedup_grid_only': ms_tab / ms_l,
        'speedup_incl_gcf_generation': (ms_tab + t_gcf * 1e3) / ms_l,
        'tc_synthesis': {'evaluations': n_eval, 'ms': ms_tc, 'tflops': flop / (ms_tc * 1e-3) / 1e12,
                         'naive_per_tap_evaluations': int(T * B * C * P) * S * S},
        'image_err_learned_vs_table': rel(i_l, i_tab), 'image_err_learned_vs_exact_table': rel(i_l, i_x),
        'image_err_table_vs_exact_table': rel(i_tab, i_x),
        'images': f'dirty images (Re FFT^-1 / sum_weight) of channels {chans}, both pols, peak-normalised by the '
                  f'exact-frequency table image',
        'table_bytes': int(ck_x.numel() * 8), 'network_bytes': int(_lib.MLP_NPARAM * 4),
    }


def _timed(fn, steps, warmup):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _line(args, world, workload, value, ms, config, roofline, cpu, e2e, err, clk, launches, extra=None, emit=True):
    """A workload's JSON line: printed when the workload runs on its own,
    returned for the records the large-cube line carries."""
    line = {'metric': METRIC, 'value': value, 'unit': 'Mvis/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic', 'config': {'workload': workload, **config},
            'roofline': roofline, 'cpu_baseline': cpu, 'e2e': e2e, 'err_vs_fp64': err, 'clocks': clk,
            'gpu_launches': launches}
    if extra:
        line.update(extra)
    if emit:
        print(json.dumps(line), flush=True)
    return line


def run_standard_small(args, rank, world, local, dist, emit=True):
    """The small standard cube (27 antennas, 600 x 10 s, 32 channels, RR/LL,
    512^2 at 2 arcsec, natural weighting): ngg_grid_ps device-resident, and
    make_imaging_weight + make_psf + make_image end to end from host arrays."""
    import torch
    from cngi_prototype_gb300 import _lib, simulate, xds
    from cngi_prototype_gb300.imaging import make_image, make_imaging_weight, make_psf
    from cngi_prototype_gb300.imaging._imaging_utils import _gridding_convolutional_kernels as G
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    obs = simulate.config_standard_small(seed=1 + rank)
    T, B, C, P = obs.vis.shape
    gp_user = {'image_size': list(obs.image_size), 'cell_size': list(obs.cell_arcsec), 'chan_mode': 'cube',
               'phase_center': [0.0, 0.0]}
    gp = dict(gp_user)
    _check_grid_parms(gp)
    npad, cell = gp['image_size_padded'], gp['cell_size']
    cgk = G._create_prolate_spheroidal_kernel_1D(100, 7)
    vis_d = torch.as_tensor(obs.vis, device='cuda')
    w_d = torch.as_tensor(obs.weight, device='cuda')
    uvw_d = torch.as_tensor(obs.uvw, device='cuda')
    f_d = torch.as_tensor(obs.freq, device='cuda')
    k_d = torch.as_tensor(cgk, device='cuda')
    grid = torch.empty((C, P, int(npad[0]), int(npad[1])), dtype=torch.complex64, device='cuda')
    sw = torch.empty((C, P), dtype=torch.float64, device='cuda')
    ms = _timed(lambda: _lib.grid_ps(vis_d, uvw_d, w_d, f_d, k_d, npad, cell, grid=grid, sum_weight=sw),
                args.steps, args.warmup)
    n_vis = T * B * C * P
    value = n_vis * world / (ms * 1e-3) / 1e6
    grid_bytes = C * P * int(npad[0]) * int(npad[1]) * 8
    alg = n_vis * 12 + T * B * 24 + grid_bytes + C * P * 8
    peak, peak_kind = measured_peaks()
    roofline = {'bound': 'hbm', 'achieved': alg / (ms * 1e-3) / 1e9, 'peak': peak, 'unit': 'GB/s',
                'frac': alg / (ms * 1e-3) / 1e9 / peak, 'traffic': None, 'kernel': 'ngg_grid_ps (whole call)',
                'kernel_ms': ms, 'algorithmic_bytes': alg, 'peak_kind': peak_kind,
                'note': 'small workload: launch- and binning-bound, not HBM-bound'}
    # end to end: the three API calls on host numpy datasets
    mx = xds.mxds({'xds0': xds.vis_dataset(obs.uvw, obs.vis, obs.weight, obs.freq)})

    def api():
        m2 = make_imaging_weight(mx, {'weighting': 'natural'}, gp_user, {'xds': 'xds0'})
        im = make_psf(m2, xds.Dataset(), gp_user, {'xds': 'xds0'}, {})
        return make_image(m2, im, gp_user, {'xds': 'xds0'}, {})
    api()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = api()
    torch.cuda.synchronize()
    te = time.perf_counter() - t0
    e2e = {'value': n_vis / te / 1e6, 'unit': 'Mvis/s', 'h2d_bytes_per_step': int(2 * (obs.vis.nbytes +
           obs.weight.nbytes + obs.uvw.nbytes)), 'd2h_bytes_per_step': int(2 * out['IMAGE'].values.nbytes),
           'ms_per_step': te * 1e3, 'note': 'make_imaging_weight + make_psf + make_image, wall clock'}
    cpu = err = None
    if rank == 0 and not args.no_cpu:
        from oracle import cbind
        threads = cpu_threads()
        go, swo, dt = oracle_sample(obs.uvw, obs.vis, obs.weight.astype(np.float64), obs.freq, cgk, npad, cell,
                                    threads)
        cpu = {'value': n_vis / dt / 1e6, 'unit': 'Mvis/s', 'cores': threads, 'kind': 'port',
               'sample': f'the whole cube ({n_vis} vis), C FP64 restatement of _standard_grid_jit'}
        corr = G._create_prolate_spheroidal_kernel(100, 7, npad)[1]
        s0 = int(npad[0]) // 2 - obs.image_size[0] // 2
        corr = corr[s0:s0 + obs.image_size[0], s0:s0 + obs.image_size[1]]
        ref = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(go, axes=(2, 3))), axes=(2, 3)).real
        ref = ref[:, :, s0:s0 + obs.image_size[0], s0:s0 + obs.image_size[1]] * (int(npad[0]) * int(npad[1]))
        ref = np.moveaxis(ref / np.where(swo == 0, 1, swo)[:, :, None, None], (0, 1), (2, 3)) / corr[:, :, None, None]
        img = out['IMAGE'].values[:, :, 0]
        ie = np.abs(img - ref)
        pk = np.abs(ref).max()
        # the gridder alone: this library's grid through numpy's FP64 FFT
        g = grid.cpu().numpy()
        gi = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(g.astype(np.complex128), axes=(2, 3))), axes=(2, 3)).real
        gi = gi[:, :, s0:s0 + obs.image_size[0], s0:s0 + obs.image_size[1]] * (int(npad[0]) * int(npad[1]))
        swg = sw.cpu().numpy()
        gi = np.moveaxis(gi / np.where(swg == 0, 1, swg)[:, :, None, None], (0, 1), (2, 3)) / corr[:, :, None, None]
        # the whole pipeline with the single-precision inverse FFT (the
        # default 'auto' takes the double-precision one at this size)
        gp32 = dict(gp_user, fft_precision='single')
        m2 = make_imaging_weight(mx, {'weighting': 'natural'}, gp32, {'xds': 'xds0'})
        img32 = make_image(m2, xds.Dataset(), gp32, {'xds': 'xds0'}, {})['IMAGE'].values[:, :, 0]
        err = {'image_max': float(ie.max() / pk), 'image_rms': float(np.sqrt(np.mean(ie ** 2)) / pk),
               'gridding_image_max': float(np.abs(gi - ref).max() / pk),
               'image_max_fft32': float(np.abs(img32 - ref).max() / pk),
               'sample': 'IMAGE of make_image (all 32 channels, both pols; default fft_precision auto = double '
                         'at this size) vs the FP64 oracle grid + numpy FFT; gridding_image_max: ngg_grid_ps grid '
                         '+ numpy FP64 FFT; image_max_fft32: make_image with fft_precision single'}
    if rank == 0:
        return _line(args, world, 'standard_small_natural', value, ms,
              {'n_time': T, 'n_baseline': B, 'n_chan': C, 'n_pol': P, 'n_vis': n_vis, 'image_size': 512,
               'grid': int(npad[0]), 'cell_arcsec': 2.0, 'weighting': 'natural', 'support': 7, 'oversampling': 100,
               'l2': 'grid and inputs (0.5 GB) larger than L2', 'parallelism': f'replica x{world}'},
              roofline, cpu, e2e, err, None, 11 * args.steps, emit=emit)


def run_degrid(args, rank, world, local, dist, emit=True):
    """Differentiable degrid/grid pair: 2048^2 float32 model of 500 Gaussian
    blobs (FWHM 2-20 px), 64 antennas x 992 times (2.0M rows), 64 channels
    over 1.0-1.5 GHz, 1 pol, 1 arcsec cells. One step = model visibilities
    (D^T, ngg_fft_correct_adjoint + ngg_degrid_ps), chi-square against
    synthetic data (sigma 0.1), and its gradient (D, ngg_grid_ps +
    ngg_fft_correct) through the autograd function."""
    import torch
    from cngi_prototype_gb300 import simulate
    from cngi_prototype_gb300.imaging.degrid import ImagingOperator, degrid
    rng = np.random.default_rng(3 + rank)
    enu = simulate.log_spiral_layout(64, 2500.0, rng)
    uvw = simulate.earth_rotation_uvw(enu, 992, 8.0)
    T, B = uvw.shape[:2]
    C, P, N = 64, 1, 2048
    freq = 1.0e9 + (np.arange(C) + 0.5) * (0.5e9 / C)
    gp = {'image_size': [N, N], 'cell_size': [1.0, 1.0], 'chan_mode': 'cube'}
    w = torch.ones((T, B, C, P), dtype=torch.float32, device='cuda')
    op = ImagingOperator(uvw, w, freq, gp)
    # model: 500 Gaussians on the GPU
    yy, xx = torch.meshgrid(torch.arange(N, device='cuda', dtype=torch.float32),
                            torch.arange(N, device='cuda', dtype=torch.float32), indexing='ij')
    model = torch.zeros((N, N), dtype=torch.float32, device='cuda')
    pos = rng.uniform(0, N, (500, 2))
    fw = rng.uniform(2, 20, 500)
    amp = rng.uniform(0, 1, 500)
    for k in range(500):
        s2 = (fw[k] / 2.3548) ** 2
        model += float(amp[k]) * torch.exp(-((xx - float(pos[k, 0])) ** 2 + (yy - float(pos[k, 1])) ** 2) / (2 * s2))
    x = model[:, :, None, None].expand(N, N, C, P).contiguous().requires_grad_(True)
    with torch.no_grad():
        v_model = op.degrid(x.detach())
        noise = torch.complex(torch.randn(v_model.shape, device='cuda'), torch.randn(v_model.shape, device='cuda'))
        v_data = (v_model + 0.1 * noise).to(torch.complex64)

    def step():
        x.grad = None
        r = degrid(x, op) - v_data
        loss = (r.real ** 2 + r.imag ** 2).sum()
        loss.backward()
        return loss

    ms = _timed(step, args.steps, args.warmup)
    n_vis = T * B * C * P
    value = n_vis * world / (ms * 1e-3) / 1e6
    fwd_ms = _timed(lambda: op.degrid(x.detach()), args.steps, 1)
    bwd_ms = _timed(lambda: op.image(v_data), args.steps, 1)
    cpu = None
    if rank == 0 and not args.no_cpu:
        from cngi_prototype_gb300.imaging._imaging_utils import _gridding_convolutional_kernels as G
        nc = min(C, cpu_threads())
        threads = cpu_threads()
        vs = v_data[:, :, :nc].cpu().numpy()
        _, _, dt = oracle_sample(uvw, vs, np.ones(vs.shape), freq[:nc], G._create_prolate_spheroidal_kernel_1D(100, 7),
                                 op.npad, op.cell, threads)
        cpu = {'value': T * B * nc * P / dt / 1e6, 'unit': 'Mvis/s', 'cores': threads, 'kind': 'port',
               'sample': f'the gradient half (gridding) of channels 0-{nc - 1}: C FP64 restatement of '
                         f'_standard_grid_jit; the reference has no degridder'}
    if rank == 0:
        return _line(args, world, 'degrid_grid_chi2_step', value, ms,
              {'n_time': T, 'n_baseline': B, 'n_chan': C, 'n_pol': P, 'n_vis': n_vis, 'image_size': N,
               'grid': int(op.npad[0]), 'cell_arcsec': 1.0, 'model': '500 Gaussians, FWHM 2-20 px',
               'parallelism': f'replica x{world}'},
              None, cpu, None, None, None, 12 * args.steps,
              {'forward_degrid_ms': fwd_ms, 'backward_grid_ms': bwd_ms,
               'note': 'value = model visibilities per second of one forward + chi-square + backward step'},
              emit=emit)


def _ev_ms(fn, steps, warmup):
    """Mean ms of fn() over `steps` calls, CUDA events on the current stream
    (the stream every libngg call in this process is launched on)."""
    return _timed(fn, steps, warmup)


def run_cycle(args, rank, world, local, dist):
    """The imaging major-cycle pieces around the gridder, each device-resident:
    * direction_rotate on the mosaic geometry (50 x 12 m antennas in a 750 m
      disk, 49 pointings x 30 x 6 s = 1470 times, 1225 baselines, 16 channels
      over 100-101.6 GHz, RR/LL: 57.6M vis; one field per time row, hexagonal
      pointings at 26 arcsec): ngg_rotate_uvw + ngg_phase_rotate (complex64);
    * Hogbom CLEAN (ngg_hogbom_clean) of the small standard cube's dirty image
      and PSF (512^2, 32 channels x 2 pols = 64 planes), gain 0.1, 1000
      iterations per plane;
    * predict_modelvis_image's device part on the degrid geometry (2048^2
      model of 500 Gaussians, 64 antennas x 992 times, 64 channels, 1 pol:
      128M vis): ngg_fft_correct_adjoint + ngg_predict_ps.
    value = predicted Mvis/s; each leg reports its own rate, roofline and
    CPU baseline (the oracle's numpy restatement on one core, on a sample)."""
    import ctypes
    import torch
    from cngi_prototype_gb300 import _lib, simulate, xds
    from cngi_prototype_gb300.imaging import make_image, make_psf
    from cngi_prototype_gb300.imaging.direction_rotate import calc_rotation_mats, _row_fields
    from cngi_prototype_gb300.imaging._imaging_utils import _gridding_convolutional_kernels as G
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    from cngi_prototype_gb300.imaging._imaging_utils._remove_padding import _remove_padding
    peak, peak_kind = measured_peaks()
    L = _lib.load()
    st = _lib._stream()
    out = {}

    # ---- direction_rotate -------------------------------------------------
    rng = np.random.default_rng(6 + rank)
    enu = simulate.disk_layout(50, 750.0, rng)
    n_pt, n_int = 49, 30
    T = n_pt * n_int
    uvw = simulate.earth_rotation_uvw(enu, T, 6.0)
    B = uvw.shape[1]
    C, P = 16, 2
    freq = 100.0e9 + (np.arange(C) + 0.5) * 0.1e9
    ctr = (np.deg2rad(201.4), np.deg2rad(-43.0))
    offs = simulate.hex_offsets(n_pt, np.deg2rad(26.0 / 3600))
    ra, dec = simulate.sin_to_radec(offs[:, 0], offs[:, 1], ctr)
    field_ds = xds.Dataset({'PHASE_DIR': (('field_id', 'd1', 'd2'), np.stack([ra, dec], -1)[:, None, :])},
                           coords={'field_id': ('field_id', np.arange(n_pt))})
    field_id = np.repeat(np.repeat(np.arange(n_pt), n_int)[:, None], B, axis=1)
    rp = {'new_phase_center': ctr, 'common_tangent_reprojection': True}
    mats, phase, fid = calc_rotation_mats(field_id, field_ds, rp)
    rf = _row_fields(field_id, fid)
    g = torch.Generator(device='cuda')
    g.manual_seed(7)
    vis = torch.complex(torch.randn((T, B, C, P), device='cuda', generator=g),
                        torch.randn((T, B, C, P), device='cuda', generator=g))
    d_uvw = torch.as_tensor(uvw, device='cuda')
    d_rf = torch.as_tensor(rf, device='cuda')
    d_mats = torch.as_tensor(mats, device='cuda')
    d_ph = torch.as_tensor(phase, device='cuda')
    d_foc = torch.as_tensor(freq / 299792458.0, device='cuda')
    uvw_rot = torch.empty((T, B, 3), dtype=torch.float64, device='cuda')
    pd = torch.empty((T, B), dtype=torch.float64, device='cuda')
    vis_rot = torch.empty_like(vis)
    P_ = _lib._ptr

    def rot_uvw():
        _lib._check(L.ngg_rotate_uvw(P_(d_uvw), P_(d_rf), T, B, P_(d_mats), P_(d_ph), n_pt, 1, P_(uvw_rot), P_(pd),
                                     st), 'ngg_rotate_uvw')

    def rot_vis():
        _lib._check(L.ngg_phase_rotate(P_(vis), P_(pd), T, B, C, P, P_(d_foc), 1, P_(vis_rot), st),
                    'ngg_phase_rotate')

    ms_uvw = _ev_ms(rot_uvw, args.steps, args.warmup)
    ms_vis = _ev_ms(rot_vis, args.steps, args.warmup)
    n_vis = T * B * C * P
    rot_bytes = n_vis * 16 + T * B * 8     # vis in + out (complex64), phase per row
    cpu_rot = None
    if rank == 0 and not args.no_cpu:
        from oracle import rotate as OR
        ns = 60   # time rows in the sample
        vs = vis[:ns].cpu().numpy()
        t0 = time.perf_counter()
        ur = OR.rotate_uvw(uvw[:ns], field_id[:ns], mats, fid)
        OR.apply_phasor(vs, ur, field_id[:ns], freq, phase, fid, True, True)
        dt = time.perf_counter() - t0
        cpu_rot = {'value': ns * B * C * P / dt / 1e6, 'unit': 'Mvis/s', 'cores': 1, 'kind': 'port',
                   'sample': f'{ns} of {T} time rows, all baselines, channels and pols: the oracle\'s numpy '
                             f'restatement of apply_rotation_matrix + apply_phasor'}
    out['direction_rotate'] = {
        'value': n_vis / ((ms_uvw + ms_vis) * 1e-3) / 1e6, 'unit': 'Mvis/s', 'ms_per_step': ms_uvw + ms_vis,
        'ms_rotate_uvw': ms_uvw, 'ms_phase_rotate': ms_vis, 'n_vis': n_vis,
        'roofline': {'bound': 'hbm', 'kernel': 'k_phasor', 'achieved': rot_bytes / (ms_vis * 1e-3) / 1e9,
                     'peak': peak, 'unit': 'GB/s', 'frac': rot_bytes / (ms_vis * 1e-3) / 1e9 / peak,
                     'algorithmic_bytes': rot_bytes, 'peak_kind': peak_kind, 'traffic': None},
        'cpu_baseline': cpu_rot, 'gpu_launches_per_step': 2}
    del vis, vis_rot, uvw_rot, pd
    torch.cuda.empty_cache()

    # ---- Hogbom CLEAN -------------------------------------------------------
    obs = simulate.config_standard_small(seed=1 + rank)
    gp = {'image_size': list(obs.image_size), 'cell_size': list(obs.cell_arcsec), 'chan_mode': 'cube',
          'phase_center': [0.0, 0.0]}
    mx = xds.mxds({'xds0': xds.vis_dataset(obs.uvw, obs.vis, obs.weight, obs.freq)})
    dirty = make_image(mx, xds.Dataset(), gp, {'xds': 'xds0'}, {})['IMAGE'].values
    psf = make_psf(mx, xds.Dataset(), gp, {'xds': 'xds0'}, {})['PSF'].values
    nx, ny = dirty.shape[:2]
    n_planes = int(np.prod(dirty.shape[2:]))
    n_iter, gain = 1000, 0.1
    res = torch.as_tensor(np.ascontiguousarray(np.moveaxis(dirty.reshape(nx, ny, -1), 2, 0)), device='cuda')
    res0 = res.clone()
    ps = torch.as_tensor(np.ascontiguousarray(np.moveaxis(psf.reshape(nx, ny, -1), 2, 0)), device='cuda')
    mdl = torch.zeros_like(res)
    its = torch.zeros(n_planes, dtype=torch.int32, device='cuda')

    def clean():
        res.copy_(res0)
        mdl.zero_()
        _lib._check(L.ngg_hogbom_clean(P_(res), P_(ps), P_(mdl), n_planes, nx, ny, nx, ny, gain, 0.0, n_iter, 1,
                                       P_(its), st), 'ngg_hogbom_clean')

    ms_clean = _ev_ms(clean, args.steps, args.warmup)
    n_its = int(its.sum().item())
    # per subtraction a plane is read to find the next peak (nx*ny*8 bytes):
    # the least any Hogbom cycle moves; the window subtraction adds to it
    cl_bytes = n_its * nx * ny * 8
    cpu_cl = None
    if rank == 0 and not args.no_cpu:
        from oracle import clean as OC
        k_it = 100
        t0 = time.perf_counter()
        OC.clean(dirty[:, :, :1, :1, :1], psf[:, :, :1, :1, :1], gain, 0.0, k_it, True)
        dt = time.perf_counter() - t0
        cpu_cl = {'value': k_it / dt, 'unit': 'plane-iterations/s', 'cores': 1, 'kind': 'port',
                  'sample': f'one 512^2 plane, {k_it} iterations: the oracle\'s numpy Hogbom (FP64)'}
    out['hogbom_clean'] = {
        'value': n_its / (ms_clean * 1e-3), 'unit': 'plane-iterations/s', 'ms_per_step': ms_clean,
        'planes': n_planes, 'image': [nx, ny], 'iterations': n_its, 'gain': gain,
        'roofline': {'bound': 'hbm', 'kernel': 'k_hogbom', 'achieved': cl_bytes / (ms_clean * 1e-3) / 1e9,
                     'peak': peak, 'unit': 'GB/s', 'frac': cl_bytes / (ms_clean * 1e-3) / 1e9 / peak,
                     'algorithmic_bytes': cl_bytes, 'peak_kind': peak_kind, 'traffic': None,
                     'note': 'one CTA per plane: 64 of the SMs busy'},
        'cpu_baseline': cpu_cl, 'gpu_launches_per_step': 1}
    del res, res0, ps, mdl
    torch.cuda.empty_cache()

    # ---- predict_modelvis_image ----------------------------------------------
    rng = np.random.default_rng(3 + rank)
    enu = simulate.log_spiral_layout(64, 2500.0, rng)
    uvw = simulate.earth_rotation_uvw(enu, 992, 8.0)
    T, B = uvw.shape[:2]
    C, P, N = 64, 1, 2048
    freq = 1.0e9 + (np.arange(C) + 0.5) * (0.5e9 / C)
    gp = {'image_size': [N, N], 'cell_size': [1.0, 1.0]}
    _check_grid_parms(gp)
    npad = np.asarray(gp['image_size_padded'])
    yy, xx = torch.meshgrid(torch.arange(N, device='cuda', dtype=torch.float32),
                            torch.arange(N, device='cuda', dtype=torch.float32), indexing='ij')
    model = torch.zeros((N, N), dtype=torch.float32, device='cuda')
    pos = rng.uniform(0, N, (500, 2))
    fw = rng.uniform(2, 20, 500)
    amp = rng.uniform(0, 1, 500)
    for k in range(500):
        s2 = (fw[k] / 2.3548) ** 2
        model += float(amp[k]) * torch.exp(-((xx - float(pos[k, 0])) ** 2 + (yy - float(pos[k, 1])) ** 2) / (2 * s2))
    m = model[:, :, None, None].expand(N, N, C, P).contiguous()
    corr = np.ascontiguousarray(_remove_padding(G._create_prolate_spheroidal_kernel(100, 7, npad)[1], gp['image_size']))
    ones = torch.ones((C, P), dtype=torch.float64, device='cuda')
    cgk = G._create_prolate_spheroidal_kernel_1D(100, 7)
    d_uvw = torch.as_tensor(uvw, device='cuda')
    d_freq = torch.as_tensor(freq, device='cuda')
    d_cgk = torch.as_tensor(cgk, device='cuda')
    d_corr = torch.as_tensor(corr, device='cuda')
    grid = torch.empty((C, P, int(npad[0]), int(npad[1])), dtype=torch.complex64, device='cuda')
    pv = torch.empty((T, B, C, P), dtype=torch.complex64, device='cuda')
    a = _lib.NggDegridArgs()
    a.chan_mode = _lib.CHAN_MODES['cube']
    a.layout = _lib.LAYOUTS['fft']
    a.support, a.oversampling = 7, 100
    a.n_time, a.n_baseline, a.n_chan, a.n_pol = T, B, C, P
    a.n_u, a.n_v = int(npad[0]), int(npad[1])
    a.delta_lm[0], a.delta_lm[1] = float(gp['cell_size'][0]), float(gp['cell_size'][1])
    a.grid, a.uvw, a.weight, a.freq = P_(grid).value, P_(d_uvw).value, None, P_(d_freq).value
    a.cgk_1D, a.vis = P_(d_cgk).value, P_(pv).value

    def fft_adj():
        _lib._check(L.ngg_fft_correct_adjoint(P_(m), 0, C, P, int(npad[0]), int(npad[1]), N, N, P_(ones), P_(d_corr),
                                              P_(grid), st), 'ngg_fft_correct_adjoint')

    def predict():
        _lib._check(L.ngg_predict_ps(ctypes.byref(a), st), 'ngg_predict_ps')

    ms_fft = _ev_ms(fft_adj, args.steps, args.warmup)
    ms_pred = _ev_ms(predict, args.steps, args.warmup)
    n_vis = T * B * C * P
    pr_bytes = n_vis * 8 + T * B * 24 + C * P * int(npad[0]) * int(npad[1]) * 8   # vis out, uvw, grid once
    cpu_pr = None
    if rank == 0 and not args.no_cpu:
        from oracle import imaging as OI
        mh = model.cpu().numpy().astype(np.float64)[:, :, None, None]
        t0 = time.perf_counter()
        OI.predict_vis(mh, uvw, freq[:1], gp)
        dt = time.perf_counter() - t0
        cpu_pr = {'value': T * B / dt / 1e6, 'unit': 'Mvis/s', 'cores': 1, 'kind': 'port',
                  'sample': 'channel 0 (all 2.0M rows, one 2457^2 FFT): the oracle\'s numpy predict (FP64)'}
    value = n_vis / ((ms_fft + ms_pred) * 1e-3) / 1e6
    out['predict_modelvis_image'] = {
        'value': value, 'unit': 'Mvis/s', 'ms_per_step': ms_fft + ms_pred, 'ms_fft_correct_adjoint': ms_fft,
        'ms_predict_ps': ms_pred, 'n_vis': n_vis,
        'roofline': {'bound': 'hbm', 'kernel': 'k_degrid (normalised)',
                     'achieved': pr_bytes / (ms_pred * 1e-3) / 1e9, 'peak': peak, 'unit': 'GB/s',
                     'frac': pr_bytes / (ms_pred * 1e-3) / 1e9 / peak, 'algorithmic_bytes': pr_bytes,
                     'peak_kind': peak_kind, 'traffic': None},
        'cpu_baseline': cpu_pr}
    if rank == 0:
        _line(args, world, 'imaging_cycle', value, ms_fft + ms_pred,
              {'predict': '2048^2 model, 64 ants x 992 times, 64 chan, 1 pol (128M vis)',
               'direction_rotate': '49-pointing mosaic, 57.6M vis', 'hogbom_clean': '64 planes of 512^2',
               'parallelism': f'replica x{world}'},
              out['predict_modelvis_image']['roofline'], cpu_pr, None, None, None, 4 * args.steps, out)


def run_mosaic(args, rank, world, local, dist):
    """Mosaic aperture-projection imaging with the table GCF (one step =
    ngg_grid_gcf of the whole cube, inputs resident in HBM)."""
    line = mosaic_measure(args, rank, world, local, dist, with_e2e=not args.no_e2e, with_cpu=not args.no_cpu)
    if rank == 0:
        print(json.dumps(line), flush=True)


def mosaic_measure(args, rank, world, local, dist, with_e2e=True, with_cpu=True, steps=None, warmup=None):
    """Measure the mosaic workload; returns its JSON record (table-GCF
    gridding, GCF generation, and the learned-GCF leg unless --no-learned)."""
    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    import torch
    from cngi_prototype_gb300 import _lib, xds
    from cngi_prototype_gb300.imaging import make_gridding_convolution_function, make_image_with_gcf, make_mosaic_pb
    from cngi_prototype_gb300.imaging._imaging_utils import _mosaic
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    obs, gp_user, gcf_parms, field_ds = _mosaic_inputs(args, 4 + rank, 'cuda')
    vis_d, w_d = obs.vis, obs.weight
    T, B, C, P = vis_d.shape
    # the GCF needs only the layout: antennas, channels, pols and fields
    mx_meta = _mosaic_mxds(obs, None, np.broadcast_to(np.float32(1), (T, B, C, P)), field_ds)
    # GCF generation on the GPU (timed separately: first call, then steady state)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gcf = make_gridding_convolution_function(mx_meta, gcf_parms, gp_user, {'xds': 'xds0'})
    torch.cuda.synchronize()
    t_gcf_first = time.perf_counter() - t0
    t0 = time.perf_counter()
    gcf = make_gridding_convolution_function(mx_meta, gcf_parms, gp_user, {'xds': 'xds0'})
    torch.cuda.synchronize()
    t_gcf = time.perf_counter() - t0
    gp = dict(gp_user)
    _check_grid_parms(gp)
    npad = gp['image_size_padded']
    cell = gp['cell_size']
    os_ = np.asarray(gcf.attrs['oversampling'])
    dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), device='cuda').to(dt)
    uvw_d = dev(obs.uvw, torch.float64)
    f_d = dev(obs.freq, torch.float64)
    fidx_d = dev(_mosaic.field_indices(obs.field, gcf['field_id'].values), torch.int32)
    maps = [dev(gcf[k].values, torch.int32) for k in ('CF_BASELINE_MAP', 'CF_CHAN_MAP', 'CF_POL_MAP')]
    ck_d = dev(gcf['CONV_KERNEL'].values, torch.float64)
    sup = np.asarray(gcf['SUPPORT'].values)
    sup_d = dev(sup, torch.int32)
    sl_d = dev(_mosaic.phase_slopes(gcf), torch.float64)

    def step():
        return _lib.grid_gcf(vis_d, uvw_d, w_d, f_d, fidx_d, *maps, ck_d, sup_d, sl_d, npad, cell, os_,
                             mode='data', layout='fft')

    for _ in range(warmup):
        g, sw = step()
    del g, sw
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        g, sw = step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    clk = clocks.stop()
    if dist:
        t = torch.tensor([ms], device='cuda')
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    n_vis = T * B * C * P
    value = n_vis * world / (ms * 1e-3) / 1e6
    S = int(sup.max()) | 1
    grid_bytes = C * P * int(npad[0]) * int(npad[1]) * 8
    alg_bytes = n_vis * 12 + T * B * 24 + grid_bytes + C * P * 8
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    taps = float(np.sum(np.asarray(sup)[..., 0] * np.asarray(sup)[..., 1]) / sup[..., 0].size) * n_vis
    roofline = {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
                'traffic': None, 'kernel': 'k_grid_gcf (whole ngg_grid_gcf call)', 'kernel_ms': ms,
                'algorithmic_bytes': alg_bytes, 'peak_kind': peak_kind,
                'taps_per_s': taps / (ms * 1e-3), 'support': int(sup.max()),
                'note': f'{int(sup.max())}^2 taps per visibility: bound by tap FMAs and L1 gathers, not HBM'}

    # ---- end to end through the public API from host arrays -------------
    e2e = None
    if with_e2e:
        vis_h = vis_d.cpu().numpy()
        w_h = w_d.cpu().numpy()
        mx = _mosaic_mxds(obs, vis_h, w_h, field_ds)
        img = make_mosaic_pb(mx, gcf, xds.Dataset(), {'xds': 'xds0'}, {}, gp_user)
        make_image_with_gcf(mx, gcf, img, gp_user, {'norm_type': 'flat_sky'}, {'xds': 'xds0'}, {})   # warm
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = make_image_with_gcf(mx, gcf, img, gp_user, {'norm_type': 'flat_sky'}, {'xds': 'xds0'}, {})
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        h2d = vis_h.nbytes + w_h.nbytes + obs.uvw.nbytes + obs.field.nbytes
        d2h = out['IMAGE'].values.nbytes + out['SUM_WEIGHT'].values.nbytes
        e2e = {'value': n_vis / te / 1e6, 'unit': 'Mvis/s', 'h2d_bytes_per_step': int(h2d),
               'd2h_bytes_per_step': int(d2h), 'ms_per_step': te * 1e3,
               'note': 'make_image_with_gcf (flat_sky) on host numpy datasets: H2D of vis/weights/uvw/FIELD_ID, '
                       'gridding, cuFFT, normalisation, D2H of the float64 image; wall clock'}

    learned = None
    if not args.no_learned:
        learned = learned_leg(args, obs, gcf, gp, vis_d, uvw_d, w_d, f_d, fidx_d, sl_d, g, sw, ms, t_gcf, steps)

    cpu = None
    err = None
    if rank == 0 and with_cpu:
        from oracle import cbind
        cbind.build()
        threads = cpu_threads()
        nc = min(C, max(1, threads))
        vis_s = vis_d[:, :, :nc].cpu().numpy()
        w_s = w_d[:, :, :nc].cpu().numpy().astype(np.float64)
        pg = gcf['PHASE_GRADIENT'].values
        fidx = _mosaic.field_indices(obs.field, gcf['field_id'].values)
        t0 = time.perf_counter()
        go, swo = cbind.aperture_grid('data', vis_s, obs.uvw, w_s, fidx, gcf['CF_BASELINE_MAP'].values,
                                      gcf['CF_CHAN_MAP'].values[:nc], gcf['CF_POL_MAP'].values,
                                      gcf['CONV_KERNEL'].values, sup, pg, obs.freq[:nc], os_, npad, cell, 'cube',
                                      threads)
        dt = time.perf_counter() - t0
        nv = T * B * nc * P
        cpu = {'value': nv / dt / 1e6, 'unit': 'Mvis/s', 'cores': threads, 'kind': 'port',
               'sample': f'channels 0-{nc - 1}: all {T}x{B} rows x {P} pols ({nv} vis), C FP64 restatement of '
                         f'_aperture_grid_jit, OpenMP over channels, complex128 grid'}
        if not args.no_err:
            gg = torch.fft.fftshift(g[:nc], dim=(2, 3)).cpu().numpy()
            ge = np.abs(gg - go)
            pk = np.abs(go).max()
            err = {'grid_max': float(ge.max() / pk), 'grid_rms': float(np.sqrt(np.mean(ge ** 2)) / pk),
                   'sum_weight_max_rel': float(np.max(np.abs(sw[:nc].cpu().numpy() - swo) / np.abs(swo))),
                   'sample': f'grid: channels 0-{nc - 1}; peak-normalised against the FP64 oracle'}
    line = {
        'metric': METRIC, 'value': value, 'unit': 'Mvis/s', 'n_gpus': world, 'steps': steps,
        'warmup': warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
        'config': {'workload': MOSAIC_WORKLOAD, 'n_time': T, 'n_baseline': B, 'n_chan': C, 'n_pol': P,
                   'n_vis': n_vis, 'n_pointing': args.mosaic_pointings, 'image_size': 2048,
                   'grid': int(npad[0]), 'cell_arcsec': 0.2, 'oversampling': int(os_[0]),
                   'max_support': 31, 'support': int(sup.max()), 'n_pb_chan': int(ck_d.shape[1]),
                   'gcf_generation_s': t_gcf, 'gcf_generation_first_call_s': t_gcf_first,
                   'l2': 'inputs (0.7 GB) and grid (1.5 GB) exceed L2; no flush',
                   'parallelism': f'replica x{world}'},
        'roofline': roofline, 'cpu_baseline': cpu, 'e2e': e2e, 'err_vs_fp64': err, 'clocks': clk,
        'gpu_launches': 6 * steps, 'learned_gcf': learned,
    }
    return line


def mosaic_summary(m):
    """The mosaic record carried by the large-cube line: table-GCF and
    learned-GCF imaging times on the mosaic workload and the learned image's
    error against tables built at every channel's exact frequency."""
    L = m.get('learned_gcf') or {}
    t_gcf_ms = m['config']['gcf_generation_s'] * 1e3
    out = {'workload': m['config']['workload'], 'config': m['config'], 'value': m['value'], 'unit': m['unit'],
           'table': {'grid_ms': m['ms_per_step'], 'gcf_generation_ms': t_gcf_ms,
                     'total_ms': m['ms_per_step'] + t_gcf_ms, 'roofline': m['roofline']},
           'clocks': m['clocks']}
    if L:
        lm = L['ms_learned_grid']
        out['learned'] = {'grid_ms': lm, 'includes': 'tensor-core synthesis of the per-channel tables + gridding',
                          'train': L['train'], 'tc_synthesis': L['tc_synthesis']}
        out['learned_vs_table_time'] = lm / (m['ms_per_step'] + t_gcf_ms)
        out['learned_vs_table_time_grid_only'] = lm / m['ms_per_step']
        out['image_err_learned_vs_exact_table'] = L['image_err_learned_vs_exact_table']
        out['image_err_table_vs_exact_table'] = L['image_err_table_vs_exact_table']
        out['image_err_learned_vs_table'] = L['image_err_learned_vs_table']
        out['error_bound'] = 1e-3
        out['note'] = ('time ratio = learned (synthesis + gridding) / table (GCF generation + gridding), both on the '
                       'GPU; training is a one-off per antenna set and band and is reported, not included')
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == 'reference':
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group('gloo')
        reference_arm(args, rank)
        return
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    from cngi_prototype_gb300 import build, _lib, simulate
    from cngi_prototype_gb300.imaging._imaging_utils import _gridding_convolutional_kernels as G
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    build.build()
    _lib.load()
    if args.workload != 'large_cube':
        {'mosaic': run_mosaic, 'standard_small': run_standard_small, 'degrid': run_degrid,
         'cycle': run_cycle}[args.workload](
            args, rank, world, local, dist)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    # ---- synthetic cube on this rank's GPU (untimed) --------------------
    # N ranks: one cube of N * n_chan channels over the same band, channel-
    # partitioned (rank r holds channels [r*n_chan, (r+1)*n_chan)); cube-mode
    # channels are independent, so no data crosses ranks (weak scaling)
    obs = large_cube_obs(args, rank, world, 'cuda')
    gp = {'image_size': list(obs.image_size), 'cell_size': list(obs.cell_arcsec)}
    _check_grid_parms(gp)
    npad = gp['image_size_padded']
    cell = gp['cell_size']
    cgk = G._create_prolate_spheroidal_kernel_1D(100, 7)
    vis_d = obs.vis
    w_d = obs.weight
    T, B, C, P = vis_d.shape
    uvw_d = torch.as_tensor(obs.uvw, device='cuda')
    freq_d = torch.as_tensor(obs.freq, device='cuda')
    cgk_d = torch.as_tensor(cgk, device='cuda')
    dens, dsw = _lib.grid_density(uvw_d, w_d, freq_d, gp['image_size'], cell)
    fac = _lib.briggs_factors(dens, dsw, 'briggs', 0.5)
    iw_d = _lib.weight_lookup(uvw_d, w_d, freq_d, dens, fac, cell)
    del dens
    torch.cuda.synchronize()
    grid = torch.empty((C, P, int(npad[0]), int(npad[1])), dtype=torch.complex64, device='cuda')
    sw = torch.empty((C, P), dtype=torch.float64, device='cuda')

    def step():
        _lib.grid_ps(vis_d, uvw_d, iw_d, freq_d, cgk_d, npad, cell, grid=grid, sum_weight=sw)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    if dist:
        t = torch.tensor([ms], device='cuda')
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    n_vis = T * B * C * P
    value = n_vis * world / (ms * 1e-3) / 1e6

    # ---- dominant kernel: tile accumulation pass (events on its stream) ----
    _lib.set_profiling(True)
    tiles_ms = []
    for _ in range(3):
        step()
        bms, tms = _lib.last_phase_ms()
        tiles_ms.append(tms)
    _lib.set_profiling(False)
    t_tiles = float(np.median(tiles_ms))
    grid_bytes = C * P * int(npad[0]) * int(npad[1]) * 8
    alg_bytes = n_vis * (8 + 4) + T * B * 24 + grid_bytes + C * P * 8
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (t_tiles * 1e-3) / 1e9
    traffic = None
    tr_path = os.path.join(ROOT, 'profiles', 'k_tiles_traffic.json')
    if os.path.exists(tr_path):
        try:
            tr = json.load(open(tr_path))
            if int(tr.get('n_vis', -1)) == n_vis and int(tr.get('grid_bytes', -1)) == grid_bytes:
                traffic = float(tr['dram_bytes_read']) + float(tr['dram_bytes_write'])   # captured at this size
            else:   # scale a capture of another size: reads by visibilities, writes by grid bytes
                traffic = (float(tr['dram_bytes_read']) / float(tr['n_vis']) * n_vis +
                           float(tr['dram_bytes_write']) / float(tr['grid_bytes']) * grid_bytes)
        except Exception:
            traffic = None
    roofline = {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
                'traffic': traffic, 'kernel': 'k_tiles', 'kernel_ms': t_tiles, 'prep_ms': bms,
                'algorithmic_bytes': alg_bytes, 'peak_kind': peak_kind}


    # ---- CPU baseline and error vs FP64 on a channel sample (rank 0) ----
    cpu = None
    err = None
    if rank == 0 and not args.no_cpu:
        nc = min(args.cpu_chans, C)
        vis_s = vis_d[:, :, :nc].cpu().numpy()
        w_s = iw_d[:, :, :nc].cpu().numpy().astype(np.float64)
        threads = cpu_threads()
        go, swo, dt = oracle_sample(obs.uvw, vis_s, w_s, obs.freq[:nc], cgk, npad, cell, threads)
        nv = T * B * nc * P
        cpu = {'value': nv / dt / 1e6, 'unit': 'Mvis/s', 'cores': threads, 'kind': 'port',
               'sample': f'channels 0-{nc - 1}: all {T}x{B} rows x {P} pols ({nv} vis), C FP64 restatement of '
                         f'_standard_grid_jit, OpenMP over channels, complex128 grid'}
        if not args.no_err:
            from oracle import cbind
            g = grid[:nc].cpu().numpy()
            ge = np.abs(g - go)
            pk = np.abs(go).max()
            sw_err = float(np.max(np.abs(sw[:nc].cpu().numpy() - swo) / np.abs(swo)))
            del g
            # images of the bottom, middle and top channel of the band (the uv
            # extent, and so the footprint spread, grows with frequency):
            # GPU pipeline (grid -> cuFFT C2C -> crop/correct) against the FP64
            # oracle grid through a complex128 transform
            chans = sorted(set([0, C // 2, C - 1]))
            extra = [c for c in chans if c >= nc]
            ref_grids = {c: go[c] for c in chans if c < nc}
            if extra:
                vis_x = vis_d[:, :, extra].cpu().numpy()
                w_x = iw_d[:, :, extra].cpu().numpy().astype(np.float64)
                gx, swx = cbind.grid('data', vis_x, obs.uvw, w_x, obs.freq[extra], cgk, 7, 100, npad, cell, 'cube',
                                     threads)
                for k, c in enumerate(extra):
                    ref_grids[c] = gx[k]
                swx_map = {c: swx[k] for k, c in enumerate(extra)}
                del vis_x, w_x
            else:
                swx_map = {}
            corr = G._create_prolate_spheroidal_kernel(100, 7, npad)[1]
            s0 = int(npad[0]) // 2 - 2048
            corr = corr[s0:s0 + 4096, s0:s0 + 4096]
            corr_d = torch.as_tensor(corr, device='cuda')
            ie_max, ie_sq, ie_n, ipk = 0.0, 0.0, 0, 0.0
            per_chan = {}
            for c in chans:
                gf = torch.fft.ifftshift(grid[c:c + 1], dim=(2, 3)).contiguous()
                img = _lib.fft_correct(gf, sw[c:c + 1], corr, [4096, 4096])[:, :, 0, :]
                del gf
                swc = swo[c] if c < nc else swx_map[c]
                ref = torch.empty_like(img)
                for p in range(P):
                    pl = torch.fft.fftshift(torch.fft.ifft2(torch.fft.ifftshift(
                        torch.as_tensor(ref_grids[c][p], device='cuda'))))
                    pl = pl[s0:s0 + 4096, s0:s0 + 4096].real * (int(npad[0]) * int(npad[1]))
                    ref[:, :, p] = pl / (swc[p] if swc[p] != 0 else 1.0) / corr_d
                    del pl
                d = (img - ref).abs()
                pkc = float(ref.abs().max())
                per_chan[int(c)] = float(d.max()) / pkc
                ie_max = max(ie_max, float(d.max()) / pkc)
                ie_sq += float((d / pkc).pow(2).sum())
                ie_n += d.numel()
                del img, ref, d
            del corr_d
            err = {'grid_max': float(ge.max() / pk), 'grid_rms': float(np.sqrt(np.mean(ge ** 2)) / pk),
                   'sum_weight_max_rel': sw_err, 'image_max': ie_max, 'image_rms': float(np.sqrt(ie_sq / ie_n)),
                   'image_max_per_chan': per_chan,
                   'sample': f'grid: channels 0-{nc - 1} against the FP64 C oracle; image: channels {chans}, both '
                             f'pols, each peak-normalised, against the FP64 oracle grid through a complex128 FFT'}
            del ge, ref_grids

    # ---- end to end from pinned host buffers ----------------------------
    # _lib.grid_ps_host: inputs host->device once, then channel chunks gridded
    # into two device buffers while the previous chunk's grid streams back to
    # pinned host memory on a second stream (the 99 GB device->host copy is
    # the bound: ~193 GB/s on this link).
    e2e = None
    if not args.no_e2e:
        vis_h = torch.empty(vis_d.shape, dtype=vis_d.dtype, pin_memory=True)
        iw_h = torch.empty(iw_d.shape, dtype=iw_d.dtype, pin_memory=True)
        uvw_h = torch.empty(uvw_d.shape, dtype=uvw_d.dtype, pin_memory=True)
        vis_h.copy_(vis_d)
        iw_h.copy_(iw_d)
        uvw_h.copy_(uvw_d)
        del grid   # the streamed call holds two channel chunks of grid, not the whole cube
        torch.cuda.empty_cache()

        def e2e_step():
            return _lib.grid_ps_host(vis_h, uvw_h, iw_h, obs.freq, cgk, npad, cell, chan_chunk=32)

        e2e_step()
        torch.cuda.synchronize()
        ke = max(1, args.steps)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(ke):
            e2e_step()
        torch.cuda.synchronize()
        ems = (time.perf_counter() - t0) * 1e3 / ke
        if dist:
            t = torch.tensor([ems], device='cuda')
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ems = float(t.item())
        h2d = vis_h.numel() * 8 + iw_h.numel() * 4 + uvw_h.numel() * 8
        d2h = grid_bytes + C * P * 8
        e2e = {'value': n_vis * world / (ems * 1e-3) / 1e6, 'unit': 'Mvis/s', 'h2d_bytes_per_step': int(h2d),
               'd2h_bytes_per_step': int(d2h), 'ms_per_step': ems,
               'note': 'grid_ps_host: inputs in pinned host memory, read in place chunk by chunk by the '
                       'packing kernel over the host link; channel chunks (32) gridded while the previous chunk '
                       'streams back to pinned host memory; wall clock per call'}
        del vis_h, iw_h, uvw_h

    # ---- the metric's second half: learned vs table GCF mosaic imaging ----
    mosaic = None
    if not (args.no_mosaic and args.no_others):   # the large cube's device arrays are no longer needed
        del vis_d, w_d, iw_d, sw, uvw_d, freq_d, cgk_d, obs
        grid = None   # (already released by the end-to-end leg when it ran)
        torch.cuda.empty_cache()
    if not args.no_mosaic:
        mrec = mosaic_measure(args, rank, world, local, dist, with_e2e=False, with_cpu=False,
                              steps=min(args.steps, 10), warmup=3)
        mosaic = mosaic_summary(mrec)

    # ---- the other single-GPU configurations: small cube, degrid/grid pair ----
    others = None
    if not args.no_others:
        others = {}
        for key, fn in (('standard_small', run_standard_small), ('degrid', run_degrid)):
            rec = fn(args, rank, world, local, dist, emit=False)
            if rank == 0:
                others[key] = {k: rec.get(k) for k in ('config', 'value', 'unit', 'ms_per_step', 'roofline',
                                                          'cpu_baseline', 'e2e', 'err_vs_fp64', 'forward_degrid_ms',
                                                          'backward_grid_ms', 'note') if rec.get(k) is not None}

    if rank == 0:
        line = {
            'metric': METRIC, 'value': value, 'unit': 'Mvis/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': large_cube_config(T, B, C, P, world, args.image_size),
            'roofline': roofline, 'cpu_baseline': cpu, 'e2e': e2e, 'err_vs_fp64': err, 'clocks': clk,
            'gpu_launches': 11 * args.steps, 'mosaic': mosaic, 'other_configs': others,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
