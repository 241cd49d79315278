"""Host-side logic and the C ABI surface (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden


def test_product_ps_tables_match_reference():
    from cngi_prototype_gb300.imaging._imaging_utils import _gridding_convolutional_kernels as G
    k = load_golden('ps_kernel')
    assert np.array_equal(G._create_prolate_spheroidal_kernel_1D(100, 7), k['cgk_1D'])
    assert np.array_equal(G._create_prolate_spheroidal_kernel(100, 7, [128, 128])[1], k['corr128'])
    assert np.array_equal(G._create_prolate_spheroidal_kernel(100, 7, [75, 77])[1], k['corr75x77'])
    g0, g1 = G._prolate_spheroidal_function(k['u'])
    assert np.array_equal(g0, k['grdsf']) and np.array_equal(g1, k['kernel'])


def test_check_grid_parms_semantics():
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    gp = {'image_size': [512, 512], 'cell_size': [2.0, 2.0]}
    assert _check_grid_parms(gp)
    assert list(gp['image_size_padded']) == [614, 614]
    assert gp['cell_size'][0] < 0 < gp['cell_size'][1]
    assert gp['chan_mode'] == 'cube' and list(gp['image_center']) == [256, 256]
    gp = {'image_size': [4096, 4096], 'cell_size': [1.0, 1.0]}
    assert _check_grid_parms(gp) and list(gp['image_size_padded']) == [4915, 4915]
    assert not _check_grid_parms({'image_size': [10], 'cell_size': [1.0, 1.0]})
    assert not _check_grid_parms({'image_size': [10, 10], 'cell_size': [1.0, 1.0], 'chan_mode': 'foo'})


def _declared_functions():
    txt = open(os.path.join(ROOT, 'include', 'ngg.h')).read()
    txt = re.sub(r'/\*.*?\*/', '', txt, flags=re.S)
    return sorted(set(re.findall(r'\b(ngg_[a-z_0-9]+)\s*\(', txt)))


def test_library_exports_every_declared_symbol():
    from cngi_prototype_gb300 import build, _lib
    lib = build.build()
    assert os.path.exists(lib)
    declared = _declared_functions()
    assert 'ngg_grid_ps' in declared and 'ngg_fft_correct' in declared
    L = ctypes.CDLL(lib)
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) <= set(_lib.SIGNATURES)
    out = subprocess.run(['nm', '-D', '--defined-only', lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r' T (ngg_[a-z_0-9]+)', out))
    assert set(declared) <= exported
    assert _lib.load().ngg_version() == 100


def test_grid_args_struct_layout():
    from cngi_prototype_gb300._lib import NggGridArgs, NggDegridArgs
    assert ctypes.sizeof(NggGridArgs) == 6 * 4 + 6 * 8 + 2 * 8 + 7 * 8
    assert ctypes.sizeof(NggDegridArgs) == 4 * 4 + 6 * 8 + 2 * 8 + 6 * 8


def test_product_does_not_import_the_oracle():
    pkg = os.path.join(ROOT, 'cngi_prototype_gb300')
    for dp, _, fs in os.walk(pkg):
        for f in fs:
            if f.endswith('.py'):
                src = open(os.path.join(dp, f)).read()
                assert not re.search(r'^\s*(from|import)\s+oracle', src, re.M), f


def test_gpu_calls_fail_loudly_without_cuda():
    import torch
    if torch.cuda.is_available():
        pytest.skip('a CUDA device is present')
    from cngi_prototype_gb300 import _lib
    with pytest.raises(_lib.NggError):
        _lib.grid_ps(np.zeros((1, 1, 1, 1), np.complex64), np.zeros((1, 1, 3)), np.ones((1, 1, 1, 1), np.float32),
                     [1e9], np.ones(400), [16, 16], [-1e-4, 1e-4])


def test_fft_precision_resolution():
    """'auto' (the default) is FP64 up to 2^26 padded cells of the cube, FP32
    above; explicit choices pass through; anything else is refused."""
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    from cngi_prototype_gb300.imaging._imaging_utils._pipeline import AUTO_FFT64_CELLS, fft_precision
    gp = {'image_size': [512, 512], 'cell_size': [2.0, 2.0]}
    assert _check_grid_parms(gp) and gp['fft_precision'] == 'auto'
    npad = gp['image_size_padded']
    assert fft_precision(gp, 32, 2, npad) == 'double'          # 64 planes of 614^2
    assert fft_precision(gp, 256, 2, (4915, 4915)) == 'single'
    side = int(np.sqrt(AUTO_FFT64_CELLS))
    assert fft_precision({}, 1, 1, (side, side)) == 'double'
    assert fft_precision({}, 1, 1, (side, side + 1)) == 'single'
    for p in ('single', 'double'):
        assert fft_precision({'fft_precision': p}, 1, 1, (8, 8)) == p
    bad = {'image_size': [64, 64], 'cell_size': [1.0, 1.0], 'fft_precision': 'half'}
    assert not _check_grid_parms(bad)


def test_predict_modelvis_image_argument_checks():
    """Model shape, channel and pol counts are checked before any device work."""
    from cngi_prototype_gb300 import xds
    from cngi_prototype_gb300.imaging import predict_modelvis_image
    T, B, C, P = 3, 4, 2, 2
    uvw = np.zeros((T, B, 3))
    ds = xds.vis_dataset(uvw, np.zeros((T, B, C, P), np.complex64), np.ones((T, B, C, P)), [1e9, 1.1e9])
    gp = {'image_size': [16, 16], 'cell_size': [1.0, 1.0]}
    img = lambda m: xds.Dataset({'MODEL': (('l', 'm', 'time', 'chan', 'pol'), m)})
    with pytest.raises(ValueError, match='image_size'):
        predict_modelvis_image(img(np.zeros((16, 15, 1, C, P))), ds, gp)
    with pytest.raises(ValueError, match='channels'):
        predict_modelvis_image(img(np.zeros((16, 16, 1, 3, P))), ds, gp)
    with pytest.raises(ValueError, match='pols'):
        predict_modelvis_image(img(np.zeros((16, 16, 1, C, 3))), ds, gp)
    with pytest.raises(ValueError, match='time plane'):
        predict_modelvis_image(img(np.zeros((16, 16, 2, C, P))), ds, gp)
    with pytest.raises(KeyError):
        predict_modelvis_image(xds.Dataset({}), ds, gp)


def test_abi_refuses_bad_arguments_before_any_device_work():
    """Entry points check their arguments before touching the device: with
    no GPU present they still return NGG_ERR_INVALID (1) and name the fault."""
    from cngi_prototype_gb300 import _lib
    L = _lib.load()
    msg = lambda: L.ngg_last_error().decode()
    assert L.ngg_grid_ps(None, None) == 1 and 'NULL' in msg()
    a = _lib.NggGridArgs()
    a.n_time, a.n_baseline, a.n_chan, a.n_pol = 1, 1, 2, 1
    assert L.ngg_grid_ps_chunk(ctypes.byref(a), 1, 2, None) == 1 and 'channel range' in msg()
    assert L.ngg_grid_ps_chunk(ctypes.byref(a), -1, 4, None) == 1
    assert L.ngg_predict_ps(None, None) == 1 and 'NULL' in msg()
    assert L.ngg_degrid_ps(None, None) == 1
    assert L.ngg_rotate_uvw(None, None, -1, 1, None, None, 1, 1, None, None, None) == 1
    assert L.ngg_phase_rotate(None, None, 1, 1, 1, 0, None, 1, None, None) == 1 and 'dims' in msg()
    assert L.ngg_hogbom_clean(None, None, None, 1, 8, 8, 0, 8, 0.1, 0.0, 10, 1, None, None) == 1
    # empty work is a no-op, not an error
    assert L.ngg_phase_rotate(None, None, 0, 5, 3, 2, None, 1, None, None) == 0
    assert L.ngg_hogbom_clean(None, None, None, 0, 8, 8, 8, 8, 0.1, 0.0, 10, 1, None, None) == 0
