"""ctypes binding of libngg.so (the C ABI in include/ngg.h).

Device arrays are torch CUDA tensors used purely as carriers: their data
pointers and the current CUDA stream are handed to the C entry points. There
is no CPU fallback: if the library is not built, or no CUDA device is
present, every call raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libngg.so')

NGG_OK = 0
ERRORS = {1: 'invalid argument', 2: 'out of device memory', 3: 'CUDA error', 4: 'unsupported', 5: 'timeout'}
MODES = {'data': 0, 'psf': 1}
CHAN_MODES = {'cube': 0, 'continuum': 1}
LAYOUTS = {'natural': 0, 'fft': 1}
WEIGHTINGS = {'natural': 0, 'uniform': 1, 'briggs': 2, 'briggs_abs': 3}

_i64 = ctypes.c_int64
_vp = ctypes.c_void_p


class NggGridArgs(ctypes.Structure):
    _fields_ = [('mode', ctypes.c_int), ('chan_mode', ctypes.c_int), ('layout', ctypes.c_int),
                ('support', ctypes.c_int), ('oversampling', ctypes.c_int), ('reserved0', ctypes.c_int),
                ('n_time', _i64), ('n_baseline', _i64), ('n_chan', _i64), ('n_pol', _i64),
                ('n_u', _i64), ('n_v', _i64), ('delta_lm', ctypes.c_double * 2),
                ('vis', _vp), ('uvw', _vp), ('weight', _vp), ('freq', _vp), ('cgk_1D', _vp),
                ('grid', _vp), ('sum_weight', _vp)]


class NggDegridArgs(ctypes.Structure):
    _fields_ = [('chan_mode', ctypes.c_int), ('layout', ctypes.c_int), ('support', ctypes.c_int),
                ('oversampling', ctypes.c_int),
                ('n_time', _i64), ('n_baseline', _i64), ('n_chan', _i64), ('n_pol', _i64),
                ('n_u', _i64), ('n_v', _i64), ('delta_lm', ctypes.c_double * 2),
                ('grid', _vp), ('uvw', _vp), ('weight', _vp), ('freq', _vp), ('cgk_1D', _vp), ('vis', _vp)]


# exported symbol -> (restype, argtypes)
SIGNATURES = {
    'ngg_version': (ctypes.c_int, []),
    'ngg_last_error': (ctypes.c_char_p, []),
    'ngg_grid_ps': (ctypes.c_int, [ctypes.POINTER(NggGridArgs), _vp]),
    'ngg_grid_density': (ctypes.c_int, [ctypes.c_int, _i64, _i64, _i64, _i64, _i64, _i64,
                                        ctypes.POINTER(ctypes.c_double), _vp, _vp, _vp, _vp, _vp, _vp]),
    'ngg_briggs_factors': (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_double, _i64, _i64, _i64,
                                          _vp, _vp, _vp, _vp]),
    'ngg_weight_lookup': (ctypes.c_int, [ctypes.c_int, _i64, _i64, _i64, _i64, _i64, _i64,
                                         ctypes.POINTER(ctypes.c_double), _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    'ngg_fft_correct': (ctypes.c_int, [_vp, _i64, _i64, _i64, _i64, _i64, _i64, _vp, _vp, _vp, _vp]),
    'ngg_fft_correct_adjoint': (ctypes.c_int, [_vp, ctypes.c_int, _i64, _i64, _i64, _i64, _i64, _i64,
                                               _vp, _vp, _vp, _vp]),
    'ngg_degrid_ps': (ctypes.c_int, [ctypes.POINTER(NggDegridArgs), _vp]),
    'ngg_degrid_ps_noalloc': (ctypes.c_int, [ctypes.POINTER(NggDegridArgs), _vp]),
    'ngg_cell_indices': (ctypes.c_int, [_i64, _i64, _vp, _vp, _i64, _i64, ctypes.POINTER(ctypes.c_double),
                                        ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]),
    'ngg_set_profiling': (None, [ctypes.c_int]),
    'ngg_last_phase_ms': (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    'ngg_release_cache': (None, []),
}

_lib = None


class NggError(RuntimeError):
    pass


def load():
    """Load libngg.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NggError(f'{LIB_PATH} is missing: build it with cngi_prototype_gb300.build.build()')
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc, what):
    if rc != NGG_OK:
        msg = load().ngg_last_error().decode(errors='replace')
        raise NggError(f'{what}: {ERRORS.get(rc, rc)}: {msg}')


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise NggError('no CUDA device: the GB300 kernels have no CPU path')
    return torch


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(x, dtype, name, allow_none=False):
    """Return a contiguous CUDA tensor of `dtype` (copying host data if needed)."""
    torch = _torch()
    if x is None:
        if allow_none:
            return None
        raise NggError(f'{name} is required')
    if not isinstance(x, torch.Tensor):
        x = torch.as_tensor(np.ascontiguousarray(x))
    if x.device.type != 'cuda':
        x = x.to('cuda', non_blocking=False)
    if x.dtype != dtype:
        x = x.to(dtype)
    return x.contiguous()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _dl(delta_lm):
    arr = (ctypes.c_double * 2)(float(delta_lm[0]), float(delta_lm[1]))
    return arr


def grid_ps(vis, uvw, weight, freq, cgk_1D, n_uv, delta_lm, mode='data', chan_mode='cube',
            layout='natural', support=7, oversampling=100, grid=None, sum_weight=None):
    """Standard gridder on the GPU. Returns (grid, sum_weight) CUDA tensors.

    vis complex64 (T,B,C,P) (ignored for mode='psf'), uvw float64 (T,B,3),
    weight float32 (T,B,C,P), freq float64 (C), cgk_1D float64 table,
    n_uv padded grid size, delta_lm cell size in radians with [0] negated.
    """
    torch = _torch()
    uvw_t = _dev(uvw, torch.float64, 'uvw')
    w_t = _dev(weight, torch.float32, 'weight')
    f_t = _dev(freq, torch.float64, 'freq')
    k_t = _dev(cgk_1D, torch.float64, 'cgk_1D')
    T, B, C, P = w_t.shape
    v_t = _dev(vis, torch.complex64, 'vis') if mode == 'data' else None
    n_img = 1 if chan_mode == 'continuum' else C
    nu, nv = int(n_uv[0]), int(n_uv[1])
    if grid is None:
        gdt = torch.complex64 if (mode == 'data' or layout == 'fft') else torch.float32
        grid = torch.empty((n_img, P, nu, nv), dtype=gdt, device='cuda')
    if sum_weight is None:
        sum_weight = torch.empty((n_img, P), dtype=torch.float64, device='cuda')
    a = NggGridArgs()
    a.mode = MODES[mode]
    a.chan_mode = CHAN_MODES[chan_mode]
    a.layout = LAYOUTS[layout]
    a.support = int(support)
    a.oversampling = int(oversampling)
    a.n_time, a.n_baseline, a.n_chan, a.n_pol = T, B, C, P
    a.n_u, a.n_v = nu, nv
    a.delta_lm[0], a.delta_lm[1] = float(delta_lm[0]), float(delta_lm[1])
    a.vis = _ptr(v_t).value
    a.uvw = _ptr(uvw_t).value
    a.weight = _ptr(w_t).value
    a.freq = _ptr(f_t).value
    a.cgk_1D = _ptr(k_t).value
    a.grid = _ptr(grid).value
    a.sum_weight = _ptr(sum_weight).value
    _check(load().ngg_grid_ps(ctypes.byref(a), _stream()), 'ngg_grid_ps')
    return grid, sum_weight


def grid_density(uvw, weight, freq, n_uv, delta_lm, chan_mode='cube'):
    """Weight-density plane per image channel: (density (Cimg,N0,N1) f32, sum_weight (Cimg,) f64)."""
    torch = _torch()
    uvw_t = _dev(uvw, torch.float64, 'uvw')
    w_t = _dev(weight, torch.float32, 'weight')
    f_t = _dev(freq, torch.float64, 'freq')
    T, B, C, P = w_t.shape
    n_img = 1 if chan_mode == 'continuum' else C
    nu, nv = int(n_uv[0]), int(n_uv[1])
    dens = torch.empty((n_img, nu, nv), dtype=torch.float32, device='cuda')
    dsw = torch.empty((n_img,), dtype=torch.float64, device='cuda')
    dl = _dl(delta_lm)
    _check(load().ngg_grid_density(CHAN_MODES[chan_mode], T, B, C, P, nu, nv, dl, _ptr(uvw_t), _ptr(w_t),
                                   _ptr(f_t), _ptr(dens), _ptr(dsw), _stream()), 'ngg_grid_density')
    return dens, dsw


def briggs_factors(density, density_sum_weight, weighting, robust=0.5, briggs_abs_noise=1.0):
    torch = _torch()
    n_img, nu, nv = density.shape
    f = torch.empty((2, n_img), dtype=torch.float64, device='cuda')
    _check(load().ngg_briggs_factors(WEIGHTINGS[weighting], float(robust), float(briggs_abs_noise), n_img, nu, nv,
                                     _ptr(density), _ptr(density_sum_weight), _ptr(f), _stream()),
           'ngg_briggs_factors')
    return f


def weight_lookup(uvw, weight, freq, density, factors, delta_lm, chan_mode='cube'):
    torch = _torch()
    uvw_t = _dev(uvw, torch.float64, 'uvw')
    w_t = _dev(weight, torch.float32, 'weight')
    f_t = _dev(freq, torch.float64, 'freq')
    T, B, C, P = w_t.shape
    _, nu, nv = density.shape
    out = torch.empty_like(w_t)
    dl = _dl(delta_lm)
    _check(load().ngg_weight_lookup(CHAN_MODES[chan_mode], T, B, C, P, nu, nv, dl, _ptr(uvw_t), _ptr(w_t),
                                    _ptr(f_t), _ptr(density), _ptr(factors), _ptr(out), _stream()),
           'ngg_weight_lookup')
    return out


def fft_correct(grid_fft, sum_weight, correction, image_size):
    """In-place inverse FFT of FFT-layout planes + crop + correction -> image (l,m,C,P) f64."""
    torch = _torch()
    n_img, P, nu, nv = grid_fft.shape
    nl, nm = int(image_size[0]), int(image_size[1])
    corr = _dev(correction, torch.float64, 'correction')
    sw = _dev(sum_weight, torch.float64, 'sum_weight')
    img = torch.empty((nl, nm, n_img, P), dtype=torch.float64, device='cuda')
    _check(load().ngg_fft_correct(_ptr(grid_fft), n_img, P, nu, nv, nl, nm, _ptr(sw), _ptr(corr), _ptr(img),
                                  _stream()), 'ngg_fft_correct')
    return img


def fft_correct_adjoint(image, sum_weight, correction, n_uv):
    torch = _torch()
    nl, nm, n_img, P = image.shape
    img = image.contiguous()
    if img.dtype not in (torch.float32, torch.float64):
        img = img.to(torch.float64)
    corr = _dev(correction, torch.float64, 'correction')
    sw = _dev(sum_weight, torch.float64, 'sum_weight')
    nu, nv = int(n_uv[0]), int(n_uv[1])
    grid = torch.empty((n_img, P, nu, nv), dtype=torch.complex64, device='cuda')
    _check(load().ngg_fft_correct_adjoint(_ptr(img), 1 if img.dtype == torch.float64 else 0, n_img, P, nu, nv, nl,
                                          nm, _ptr(sw), _ptr(corr), _ptr(grid), _stream()),
           'ngg_fft_correct_adjoint')
    return grid


def degrid_ps(grid, uvw, weight, freq, cgk_1D, n_time_baseline_chan_pol, delta_lm, chan_mode='cube',
              layout='natural', support=7, oversampling=100, vis=None):
    torch = _torch()
    T, B, C, P = n_time_baseline_chan_pol
    uvw_t = _dev(uvw, torch.float64, 'uvw')
    w_t = _dev(weight, torch.float32, 'weight', allow_none=True)
    f_t = _dev(freq, torch.float64, 'freq')
    k_t = _dev(cgk_1D, torch.float64, 'cgk_1D')
    g = grid.contiguous()
    if vis is None:
        vis = torch.empty((T, B, C, P), dtype=torch.complex64, device='cuda')
    a = NggDegridArgs()
    a.chan_mode = CHAN_MODES[chan_mode]
    a.layout = LAYOUTS[layout]
    a.support = int(support)
    a.oversampling = int(oversampling)
    a.n_time, a.n_baseline, a.n_chan, a.n_pol = T, B, C, P
    a.n_u, a.n_v = int(g.shape[-2]), int(g.shape[-1])
    a.delta_lm[0], a.delta_lm[1] = float(delta_lm[0]), float(delta_lm[1])
    a.grid = _ptr(g).value
    a.uvw = _ptr(uvw_t).value
    a.weight = _ptr(w_t).value if w_t is not None else None
    a.freq = _ptr(f_t).value
    a.cgk_1D = _ptr(k_t).value
    a.vis = _ptr(vis).value
    _check(load().ngg_degrid_ps(ctypes.byref(a), _stream()), 'ngg_degrid_ps')
    return vis


def cell_indices(uvw_rows, freq, n_uv, delta_lm, oversampling, mirror=False):
    """(cu, cv, ou, ov) per (row, chan) as the kernels compute them, plus the FP64-fallback count."""
    torch = _torch()
    u = _dev(uvw_rows, torch.float64, 'uvw')
    f = _dev(freq, torch.float64, 'freq')
    n, C = u.shape[0], f.shape[0]
    idx = torch.empty((n, C, 4), dtype=torch.int32, device='cuda')
    nfb = torch.zeros((1,), dtype=torch.int64, device='cuda')
    _check(load().ngg_cell_indices(n, C, _ptr(u), _ptr(f), int(n_uv[0]), int(n_uv[1]), _dl(delta_lm),
                                   int(oversampling), 1 if mirror else 0, _ptr(idx), _ptr(nfb), _stream()),
           'ngg_cell_indices')
    return idx, int(nfb.item())


def set_profiling(enable=True):
    load().ngg_set_profiling(1 if enable else 0)


def last_phase_ms():
    """(binning_ms, tiles_ms) of the last profiled ngg_grid_ps call on this thread."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(load().ngg_last_phase_ms(ctypes.byref(a), ctypes.byref(b)), 'ngg_last_phase_ms')
    return a.value, b.value
