"""Multi-process imaging: one process per GPU with host-side (gloo) sums.

CPU tests check shard ranges and slicing, and run world-size-2 gloo groups
whose per-rank gridding/FFT core is the oracle (so the sharding, the sums
over ranks and the normalisation are what is tested) against one process
over all the data. Failure tests: a rank that marks itself failed and
leaves, and a rank that leaves silently, both end the other rank's next
sum with ShardError instead of a hang. The GPU test runs the same groups
through the CUDA path (two processes on one GPU; nothing waits on the
device, the sums are on the host), and a one-rank NCCL group exercises the
device-side sum.
"""
import os
import socket
import subprocess
import sys
import time

import numpy as np
import pytest

from conftest import ROOT

WORKER = os.path.join(ROOT, 'tests', '_dist_worker.py')


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _launch(out_dir, scenario, core, world):
    os.makedirs(out_dir, exist_ok=True)
    port = _free_port()
    env = dict(os.environ, OMP_NUM_THREADS='1')
    procs = [subprocess.Popen([sys.executable, WORKER, str(r), str(world), str(port), str(out_dir), scenario, core],
                              env=env) for r in range(world)]
    try:
        for p in procs:
            p.wait(timeout=300)
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    res = {}
    for r in range(world):
        npz, err = os.path.join(out_dir, f'rank{r}.npz'), os.path.join(out_dir, f'rank{r}.err')
        if os.path.exists(npz):
            res[r] = dict(np.load(npz))
        elif os.path.exists(err):
            res[r] = open(err).read()
        else:
            res[r] = None
    return res


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_shard_range_partitions():
    from cngi_prototype_gb300.imaging.distributed import shard_range
    for n in (0, 1, 5, 7, 256, 1001):
        for world in (1, 2, 3, 4, 8):
            parts = [shard_range(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_shard_vis_slices_channels_or_rows():
    from cngi_prototype_gb300 import xds
    from cngi_prototype_gb300.imaging.distributed import shard_vis
    rng = np.random.default_rng(0)
    T, B, C, P = 7, 4, 5, 2
    uvw = rng.standard_normal((T, B, 3))
    vis = (rng.standard_normal((T, B, C, P)) + 1j).astype(np.complex64)
    w = rng.random((T, B, C, P)).astype(np.float32)
    mx = xds.mxds({'xds0': xds.vis_dataset(uvw, vis, w, np.arange(C) * 1e6 + 1e9, time=np.arange(T) * 3.0)})
    got_c = [shard_vis(mx, {'xds': 'xds0'}, 'cube', r, 2).attrs['xds0'] for r in range(2)]
    assert [g['DATA'].shape[2] for g in got_c] == [3, 2]
    assert np.array_equal(np.concatenate([g['DATA'].values for g in got_c], axis=2), vis)
    assert np.array_equal(np.concatenate([g.coords['chan'].values for g in got_c]), np.arange(C) * 1e6 + 1e9)
    assert np.array_equal(got_c[1]['UVW'].values, uvw)          # rows shared in cube mode
    got_t = [shard_vis(mx, {'xds': 'xds0'}, 'continuum', r, 3).attrs['xds0'] for r in range(3)]
    assert [g['DATA'].shape[0] for g in got_t] == [3, 2, 2]
    assert np.array_equal(np.concatenate([g['UVW'].values for g in got_t]), uvw)
    assert np.array_equal(np.concatenate([g.coords['time'].values for g in got_t]), np.arange(T) * 3.0)
    assert mx.attrs['xds0']['DATA'].shape == (T, B, C, P)      # input untouched


def test_single_rank_group_sums_nothing():
    from cngi_prototype_gb300.imaging.distributed import ShardGroup
    g = ShardGroup()
    assert (g.rank, g.world) == (0, 1)
    a = np.arange(6.0).reshape(2, 3)
    (b,) = g.sum([a])
    assert np.array_equal(a, b)


def _check_against_single(two, one, chan_mode, tol):
    assert all(isinstance(two[r], dict) for r in (0, 1)), two
    assert isinstance(one[0], dict), one
    full = one[0]
    if chan_mode == 'continuum':
        T = full['imaging_weight'].shape[0]
        cut = (T + 1) // 2
        assert _rel(np.concatenate([two[0]['imaging_weight'], two[1]['imaging_weight']]), full['imaging_weight']) < tol
        assert two[0]['imaging_weight'].shape[0] == cut
        for r in (0, 1):
            for k in ('psf', 'image', 'sum_weight', 'psf_sum_weight', 'time'):
                assert _rel(two[r][k], full[k]) < tol, (r, k, _rel(two[r][k], full[k]))
    else:
        for k, ax in (('imaging_weight', 2), ('psf', 3), ('image', 3), ('sum_weight', 1), ('psf_sum_weight', 1)):
            cat = np.concatenate([two[0][k], two[1][k]], axis=ax)
            assert _rel(cat, full[k]) < tol, (k, _rel(cat, full[k]))


@pytest.mark.parametrize('chan_mode', ['continuum', 'cube'])
def test_two_ranks_match_one_process_oracle_core(tmp_path, chan_mode):
    two = _launch(str(tmp_path / 'w2'), chan_mode, 'oracle', 2)
    one = _launch(str(tmp_path / 'w1'), chan_mode, 'oracle', 1)
    _check_against_single(two, one, chan_mode, 1e-12)


@pytest.mark.parametrize('scenario', ['fail_mark', 'fail_exit'])
def test_failed_rank_ends_the_others_sum(tmp_path, scenario):
    t0 = time.time()
    res = _launch(str(tmp_path / scenario), scenario, 'oracle', 2)
    assert isinstance(res[0], str) and res[0].startswith('ShardError'), res[0]
    if scenario == 'fail_mark':
        assert 'input file missing' in res[0] or 'failed' in res[0]
    assert time.time() - t0 < 120


@pytest.mark.gpu
@pytest.mark.parametrize('chan_mode', ['continuum', 'cube'])
def test_two_ranks_match_one_process_gpu(ngg, tmp_path, chan_mode):
    two = _launch(str(tmp_path / 'w2'), chan_mode, 'gpu', 2)
    one = _launch(str(tmp_path / 'w1'), chan_mode, 'gpu', 1)
    _check_against_single(two, one, chan_mode, 1e-5)


@pytest.mark.gpu
def test_device_sum_in_an_nccl_group(tmp_path):
    """ShardGroup's NCCL branch (the continuum density grid summed on the
    device): flatten, all-reduce and split CUDA tensors. A one-rank group on
    this GPU exercises the calls; the sum over one rank is the input."""
    code = f'''
import torch, torch.distributed as dist
dist.init_process_group('nccl', init_method='tcp://127.0.0.1:{_free_port()}', rank=0, world_size=1)
from cngi_prototype_gb300.imaging.distributed import ShardGroup
g = ShardGroup()
a = torch.arange(12., device='cuda').reshape(3, 4).float()
b = torch.full((5,), 0.25, device='cuda', dtype=torch.float32)
out = g._sum_device([a, b])
assert all(o.is_cuda and o.dtype == torch.float64 for o in out)
assert out[0].shape == a.shape and out[1].shape == b.shape
assert torch.equal(out[0], a.double()) and torch.equal(out[1], b.double())
dist.destroy_process_group()
print('device sum ok')
'''
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get('PYTHONPATH', ''))
    r = subprocess.run([sys.executable, '-c', code], env=env, capture_output=True, text=True, timeout=180)
    assert r.returncode == 0 and 'device sum ok' in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
