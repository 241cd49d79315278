"""ngg_degrid_ps_noalloc: degridding for callers that cannot let the library
allocate device memory (a host application that owns and budgets all of it).
The variant keeps its scratch in a fixed array inside the library; this test
calls it through the C ABI and checks it against ngg_degrid_ps on two calls
in a row with different sizes (so stale scratch from the first call would
show), and that oversized requests are rejected.

Collected last on purpose: a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _args(lib_mod, grid, uvw, weight, freq, cgk, dims, dl, vis, chan_mode=0, layout=0):
    a = lib_mod.NggDegridArgs()
    a.chan_mode = chan_mode
    a.layout = layout
    a.support = 7
    a.oversampling = 100
    a.n_time, a.n_baseline, a.n_chan, a.n_pol = dims
    a.n_u, a.n_v = int(grid.shape[-2]), int(grid.shape[-1])
    a.delta_lm[0], a.delta_lm[1] = float(dl[0]), float(dl[1])
    a.grid = grid.data_ptr()
    a.uvw = uvw.data_ptr()
    a.weight = weight.data_ptr()
    a.freq = freq.data_ptr()
    a.cgk_1D = cgk.data_ptr()
    a.vis = vis.data_ptr()
    return a


def _case(seed, T, B, C, P, nu, nv, chan_mode=0, uv_max=900.0):
    import torch
    rng = np.random.default_rng(seed)
    CG = 1 if chan_mode == 1 else C
    grid = torch.as_tensor((rng.standard_normal((CG, P, nu, nv)) + 1j * rng.standard_normal((CG, P, nu, nv)))
                           .astype(np.complex64), device='cuda')
    uvw = torch.as_tensor(rng.uniform(-uv_max, uv_max, (T, B, 3)), device='cuda')
    weight = torch.as_tensor(rng.uniform(0.5, 2.0, (T, B, C, P)).astype(np.float32), device='cuda')
    freq = torch.as_tensor(1.0e9 + (2e7 if C < 1000 else 1e4) * np.arange(C), device='cuda')
    return grid, uvw, weight, freq


def test_noalloc_degrid_matches_allocating_entry_point():
    import torch
    from cngi_prototype_gb300 import build, _lib
    from cngi_prototype_gb300.imaging._imaging_utils._gridding_convolutional_kernels import \
        _create_prolate_spheroidal_kernel_1D
    build.build()
    L = _lib.load()
    cgk = torch.as_tensor(_create_prolate_spheroidal_kernel_1D(100, 7), device='cuda')
    dl = [-5e-5, 5e-5]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # (seed, dims, grid size, chan_mode, layout): cube natural twice in a row
    # with different sizes (stale scratch from the first call would show),
    # continuum, the FFT layout, and continuum at exactly the channel limit
    # with few rows (the channel region at the end of the array, to its last
    # byte)
    cases = [(1, (37, 21, 3, 2), (96, 100), 0, 0), (2, (50, 10, 5, 1), (70, 64), 0, 0),
             (3, (23, 17, 6, 2), (80, 72), 1, 0), (4, (29, 13, 4, 2), (90, 66), 0, 1),
             (5, (2, 3, _lib.NOALLOC_MAX_CHAN, 1), (64, 64), 1, 1)]
    for seed, dims, nuv, cm, lay in cases:
        grid, uvw, weight, freq = _case(seed, *dims, *nuv, chan_mode=cm, uv_max=900.0 if dims[2] < 1000 else 300.0)
        out_ref = torch.empty(dims, dtype=torch.complex64, device='cuda')
        out_new = torch.full(dims, complex(np.nan, np.nan), dtype=torch.complex64, device='cuda')
        a = _args(_lib, grid, uvw, weight, freq, cgk, dims, dl, out_ref, cm, lay)
        assert L.ngg_degrid_ps(ctypes.byref(a), stream) == 0
        b = _args(_lib, grid, uvw, weight, freq, cgk, dims, dl, out_new, cm, lay)
        assert L.ngg_degrid_ps_noalloc(ctypes.byref(b), stream) == 0, L.ngg_last_error()
        torch.cuda.synchronize()
        r, n = out_ref.cpu().numpy(), out_new.cpu().numpy()
        assert np.abs(r).max() > 0
        assert np.abs(n - r).max() <= 1e-6 * np.abs(r).max()


def test_noalloc_degrid_rejects_sizes_beyond_its_scratch():
    import torch
    from cngi_prototype_gb300 import _lib
    L = _lib.load()
    a = _lib.NggDegridArgs()
    a.chan_mode, a.layout, a.support, a.oversampling = 0, 0, 7, 100
    a.n_time, a.n_baseline, a.n_chan, a.n_pol = 1 << 20, 2, 1, 1
    a.n_u = a.n_v = 64
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.ngg_degrid_ps_noalloc(ctypes.byref(a), stream) == 1
    assert b'scratch limit' in L.ngg_last_error()
    a.n_time, a.n_baseline, a.n_chan = 4, 4, 20000
    assert L.ngg_degrid_ps_noalloc(ctypes.byref(a), stream) == 1
    assert b'channels' in L.ngg_last_error()
