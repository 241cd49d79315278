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


class NggImagingWeights(ctypes.Structure):
    _fields_ = [('density', _vp), ('factors', _vp), ('n_u', _i64), ('n_v', _i64), ('flag', _vp)]


class NggDegridArgs(ctypes.Structure):
    _fields_ = [('chan_mode', ctypes.c_int), ('layout', ctypes.c_int), ('support', ctypes.c_int),
                ('oversampling', ctypes.c_int),
                ('n_time', _i64), ('n_baseline', _i64), ('n_chan', _i64), ('n_pol', _i64),
                ('n_u', _i64), ('n_v', _i64), ('delta_lm', ctypes.c_double * 2),
                ('grid', _vp), ('uvw', _vp), ('weight', _vp), ('freq', _vp), ('cgk_1D', _vp), ('vis', _vp)]


class NggGcfArgs(ctypes.Structure):
    _fields_ = [('mode', ctypes.c_int), ('chan_mode', ctypes.c_int), ('layout', ctypes.c_int),
                ('oversampling', ctypes.c_int * 2), ('n_field', ctypes.c_int),
                ('n_time', _i64), ('n_baseline', _i64), ('n_chan', _i64), ('n_pol', _i64),
                ('n_u', _i64), ('n_v', _i64), ('delta_lm', ctypes.c_double * 2),
                ('n_cf_baseline', _i64), ('n_cf_chan', _i64), ('n_cf_pol', _i64), ('conv_size', _i64 * 2),
                ('vis', _vp), ('uvw', _vp), ('weight', _vp), ('freq', _vp), ('field_index', _vp),
                ('cf_baseline_map', _vp), ('cf_chan_map', _vp), ('cf_pol_map', _vp),
                ('conv_kernel', _vp), ('support', _vp), ('phase_slope', _vp), ('grid', _vp), ('sum_weight', _vp)]


class NggMlpScale(ctypes.Structure):
    _fields_ = [('x_scale', ctypes.c_double), ('y_scale', ctypes.c_double), ('f_center', ctypes.c_double),
                ('f_scale', ctypes.c_double), ('out_scale', ctypes.c_double)]


NOALLOC_MAX_ROWS = 1048576   # include/ngg.h NGG_NOALLOC_MAX_ROWS
NOALLOC_MAX_CHAN = 16384     # include/ngg.h NGG_NOALLOC_MAX_CHAN

MLP_NPARAM = 16833
MLP_NTRAINED = 16705

# exported symbol -> (restype, argtypes)
SIGNATURES = {
    'ngg_version': (ctypes.c_int, []),
    'ngg_last_error': (ctypes.c_char_p, []),
    'ngg_grid_ps': (ctypes.c_int, [ctypes.POINTER(NggGridArgs), _vp]),
    'ngg_primary_beam': (ctypes.c_int, [ctypes.c_int, _i64, _vp, _vp, _i64, _vp, _i64, _i64,
                                        ctypes.POINTER(ctypes.c_double), _i64, _i64, ctypes.c_int, _vp, _vp]),
    'ngg_grid_ps_weighted': (ctypes.c_int, [ctypes.POINTER(NggGridArgs), ctypes.POINTER(NggImagingWeights), _vp]),
    'ngg_grid_density': (ctypes.c_int, [ctypes.c_int, _i64, _i64, _i64, _i64, _i64, _i64,
                                        ctypes.POINTER(ctypes.c_double), _vp, _vp, _vp, _vp, _vp, _vp]),
    'ngg_briggs_factors': (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_double, _i64, _i64, _i64,
                                          _vp, _vp, _vp, _vp]),
    'ngg_weight_lookup': (ctypes.c_int, [ctypes.c_int, _i64, _i64, _i64, _i64, _i64, _i64,
                                         ctypes.POINTER(ctypes.c_double), _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    'ngg_fft_correct': (ctypes.c_int, [_vp, _i64, _i64, _i64, _i64, _i64, _i64, _vp, _vp, _vp, _vp]),
    'ngg_fft_correct_f64': (ctypes.c_int, [_vp, _i64, _i64, _i64, _i64, _i64, _i64, _vp, _vp, _vp, _vp]),
    'ngg_fft_correct_adjoint': (ctypes.c_int, [_vp, ctypes.c_int, _i64, _i64, _i64, _i64, _i64, _i64,
                                               _vp, _vp, _vp, _vp]),
    'ngg_degrid_ps': (ctypes.c_int, [ctypes.POINTER(NggDegridArgs), _vp]),
    'ngg_hogbom_clean': (ctypes.c_int, [_vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int, _vp, _vp]),
    'ngg_rotate_uvw': (ctypes.c_int, [_vp, _vp, _i64, _i64, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]),
    'ngg_phase_rotate': (ctypes.c_int, [_vp, _vp, _i64, _i64, _i64, _i64, _vp, ctypes.c_int, _vp, _vp]),
    'ngg_degrid_ps_noalloc': (ctypes.c_int, [ctypes.POINTER(NggDegridArgs), _vp]),
    'ngg_predict_ps': (ctypes.c_int, [ctypes.POINTER(NggDegridArgs), _vp]),
    'ngg_grid_ps_chunk': (ctypes.c_int, [ctypes.POINTER(NggGridArgs), _i64, _i64, _vp]),
    'ngg_cell_indices': (ctypes.c_int, [_i64, _i64, _vp, _vp, _i64, _i64, ctypes.POINTER(ctypes.c_double),
                                        ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]),
    'ngg_grid_gcf': (ctypes.c_int, [ctypes.POINTER(NggGcfArgs), _vp]),
    'ngg_grid_gcf_weight': (ctypes.c_int, [ctypes.POINTER(NggGcfArgs), _vp]),
    'ngg_gcf_kernels': (ctypes.c_int, [ctypes.c_int, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _i64, _i64,
                                       ctypes.POINTER(ctypes.c_double), _i64, _i64, _vp, _vp, _vp]),
    'ngg_mosaic_normalize': (ctypes.c_int, [_vp, _i64, _i64, _i64, _vp, _vp, _vp, ctypes.c_double,
                                            ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_int64), _vp]),
    'ngg_sqrt_abs': (ctypes.c_int, [_vp, _i64, _vp, _vp]),
    'ngg_mlp_forward': (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp]),
    'ngg_mlp_forward_tc': (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp]),
    'ngg_mlp_loss_grad': (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, _vp, _vp]),
    'ngg_mlp_adam': (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_int, _vp]),
    'ngg_mlp_train': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _i64, _i64, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_float, ctypes.c_float, ctypes.c_uint64, _vp, _vp]),
    'ngg_grid_gcf_learned': (ctypes.c_int, [ctypes.POINTER(NggGcfArgs), _vp, ctypes.POINTER(NggMlpScale), _vp]),
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


def _pinned_or_dev(x, dtype, name):
    """A contiguous pinned host tensor of `dtype` as is (the kernels read it in
    place), anything else as _dev makes it."""
    torch = _torch()
    if isinstance(x, torch.Tensor) and x.device.type == 'cpu' and x.is_pinned() and x.dtype == dtype \
            and x.is_contiguous():
        return x
    return _dev(x, dtype, name)


def grid_ps(vis, uvw, weight, freq, cgk_1D, n_uv, delta_lm, mode='data', chan_mode='cube',
            layout='natural', support=7, oversampling=100, grid=None, sum_weight=None, chan_offset=0,
            chan_total=None, density=None, factors=None, flag=None):
    """Standard gridder on the GPU. Returns (grid, sum_weight) CUDA tensors.

    vis complex64 (T,B,C,P) (ignored for mode='psf'), uvw float64 (T,B,3),
    weight float32 (T,B,C,P), freq float64 (C), cgk_1D float64 table,
    n_uv padded grid size, delta_lm cell size in radians with [0] negated.
    With chan_total, vis and weight are (T,B,chan_total,P) and the call grids
    their channels [chan_offset, chan_offset + len(freq)) (ngg_grid_ps_chunk);
    they may then be pinned host tensors, read in place.
    With density / factors (ngg_grid_density / ngg_briggs_factors outputs) the
    weights are natural weights and the imaging weights are formed in the
    packing pass; flag (T,B,C,P) bool leaves flagged visibilities out of DATA
    grids (ngg_grid_ps_weighted).
    """
    torch = _torch()
    uvw_t = _dev(uvw, torch.float64, 'uvw')
    f_t = _dev(freq, torch.float64, 'freq')
    k_t = _dev(cgk_1D, torch.float64, 'cgk_1D')
    if chan_total is None:
        w_t = _dev(weight, torch.float32, 'weight')
        T, B, C, P = w_t.shape
        v_t = _dev(vis, torch.complex64, 'vis') if mode == 'data' else None
    else:
        w_t = _pinned_or_dev(weight, torch.float32, 'weight')
        T, B, Ct, P = w_t.shape
        C = int(f_t.shape[0])
        if Ct != int(chan_total) or not (0 <= int(chan_offset) and int(chan_offset) + C <= Ct):
            raise ValueError('chan_offset/chan_total do not match the weight array')
        v_t = _pinned_or_dev(vis, torch.complex64, 'vis') if mode == 'data' else None
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
    if density is not None or flag is not None:
        if chan_total is not None:
            raise ValueError('density/flag need the whole-cube call (no chan_total)')
        iw = NggImagingWeights()
        keep = []
        if density is not None:
            if factors is None:
                raise ValueError('density needs factors')
            d_t = _dev(density, torch.float32, 'density')
            fa_t = _dev(factors, torch.float64, 'factors')
            keep += [d_t, fa_t]
            iw.density, iw.factors = _ptr(d_t).value, _ptr(fa_t).value
            iw.n_u, iw.n_v = int(d_t.shape[1]), int(d_t.shape[2])
        if flag is not None:
            fl_t = _dev(flag, torch.uint8, 'flag')
            if tuple(fl_t.shape) != (T, B, C, P):
                raise ValueError('flag must have the shape of vis')
            keep.append(fl_t)
            iw.flag = _ptr(fl_t).value
        _check(load().ngg_grid_ps_weighted(ctypes.byref(a), ctypes.byref(iw), _stream()), 'ngg_grid_ps_weighted')
        del keep
    elif chan_total is None:
        _check(load().ngg_grid_ps(ctypes.byref(a), _stream()), 'ngg_grid_ps')
    else:
        _check(load().ngg_grid_ps_chunk(ctypes.byref(a), int(chan_offset), int(chan_total), _stream()),
               'ngg_grid_ps_chunk')
    return grid, sum_weight


def primary_beam(function, dish_diameters, blockage_diameters, freq, image_size, cell, image_center, ipower=2):
    """Airy primary beams (n0, n1, C, n_types) float64 CUDA tensor (ngg_primary_beam)."""
    torch = _torch()
    if function not in ('airy', 'casa_airy'):
        raise NggError(f"pb function must be 'airy' or 'casa_airy', got {function!r}")
    d = _dev(np.asarray(dish_diameters, dtype=np.float64), torch.float64, 'dish')
    b = _dev(np.asarray(blockage_diameters, dtype=np.float64), torch.float64, 'blockage')
    f = _dev(np.asarray(freq, dtype=np.float64), torch.float64, 'freq')
    n0, n1 = int(image_size[0]), int(image_size[1])
    out = torch.empty((n0, n1, int(f.shape[0]), int(d.shape[0])), dtype=torch.float64, device='cuda')
    cl = (ctypes.c_double * 2)(float(cell[0]), float(cell[1]))
    _check(load().ngg_primary_beam(1 if function == 'casa_airy' else 0, int(d.shape[0]), _ptr(d), _ptr(b),
                                   int(f.shape[0]), _ptr(f), n0, n1, cl, int(image_center[0]), int(image_center[1]),
                                   int(ipower), _ptr(out), _stream()), 'ngg_primary_beam')
    return out


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


def fft_correct(grid_fft, sum_weight, correction, image_size, precision='single'):
    """Inverse FFT of FFT-layout planes + crop + correction -> image (l,m,C,P) f64.

    precision 'single': in-place complex64 transform (grid destroyed);
    'double': complex128 transform in library scratch (grid kept)."""
    torch = _torch()
    n_img, P, nu, nv = grid_fft.shape
    nl, nm = int(image_size[0]), int(image_size[1])
    corr = _dev(correction, torch.float64, 'correction')
    sw = _dev(sum_weight, torch.float64, 'sum_weight')
    img = torch.empty((nl, nm, n_img, P), dtype=torch.float64, device='cuda')
    if precision not in ('single', 'double'):
        raise ValueError(f"precision must be 'single' or 'double', got {precision!r}")
    name = 'ngg_fft_correct' if precision == 'single' else 'ngg_fft_correct_f64'
    _check(getattr(load(), name)(_ptr(grid_fft), n_img, P, nu, nv, nl, nm, _ptr(sw), _ptr(corr), _ptr(img),
                                 _stream()), name)
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


def hogbom_clean(dirty, psf, gain, threshold, n_iter, scale_by_peak=True):
    """Hogbom minor cycle on every plane (ngg_hogbom_clean). dirty (l, m, time,
    chan, pol) and psf (l', m', time, chan, pol), float64; returns (model,
    residual) CUDA float64 (l, m, time, chan, pol) and the subtractions per
    plane (time, chan, pol) int32."""
    torch = _torch()
    d = _dev(dirty, torch.float64, 'dirty')
    p = _dev(psf, torch.float64, 'psf')
    nx, ny = int(d.shape[0]), int(d.shape[1])
    px, py = int(p.shape[0]), int(p.shape[1])
    planes = tuple(int(x) for x in d.shape[2:])
    if tuple(int(x) for x in p.shape[2:]) != planes:
        raise ValueError('psf and dirty image must have the same (time, chan, pol) planes')
    n = int(np.prod(planes)) if planes else 1
    res = d.reshape(nx, ny, n).permute(2, 0, 1).contiguous()
    ps = p.reshape(px, py, n).permute(2, 0, 1).contiguous()
    mdl = torch.zeros_like(res)
    its = torch.zeros(n, dtype=torch.int32, device='cuda')
    _check(load().ngg_hogbom_clean(_ptr(res), _ptr(ps), _ptr(mdl), n, nx, ny, px, py, float(gain), float(threshold),
                                   int(n_iter), 1 if scale_by_peak else 0, _ptr(its), _stream()), 'ngg_hogbom_clean')
    back = lambda t: t.permute(1, 2, 0).reshape((nx, ny) + planes)
    return back(mdl), back(res), its.reshape(planes)


def grid_ps_host(vis, uvw, weight, freq, cgk_1D, n_uv, delta_lm, out=None, on_chunk=None, chan_chunk=32,
                 mode='data', layout='natural', support=7, oversampling=100):
    """Cube gridding from host arrays to host grids, streamed by channel chunk.

    Pinned host torch tensors (vis complex64, weight float32) are read in
    place by the packing kernel, chunk by chunk, over the host link
    (ngg_grid_ps_chunk), so the inputs' host-to-device traffic overlaps the
    grid's copy back instead of preceding it; other inputs are copied to the
    device once. Chunk i is gridded into one of two
    device grid buffers while chunk i-1 is copied back on a second stream, so
    the device-to-host copy of the grid -- the bulk of the traffic for a cube
    -- overlaps the gridding, and device memory holds two chunks instead of
    the whole grid. Each chunk's grid goes to out[c0:c1] (a host tensor of
    shape (C, P, Nu, Nv)) or, with out=None, to a pinned staging buffer that
    on_chunk(c0, c1, host_view) receives once it is complete (the buffer is
    reused after on_chunk returns). Returns sum_weight (C, P) float64 on the host.
    """
    torch = _torch()
    cur = torch.cuda.current_stream()
    side = torch.cuda.Stream()
    uvw_t = _dev(uvw, torch.float64, 'uvw')
    w_t = _pinned_or_dev(weight, torch.float32, 'weight')
    v_t = _pinned_or_dev(vis, torch.complex64, 'vis') if mode == 'data' else None
    T, B, C, P = w_t.shape
    freq = np.asarray(freq, dtype=np.float64)
    nu, nv = int(n_uv[0]), int(n_uv[1])
    gdt = torch.complex64 if (mode == 'data' or layout == 'fft') else torch.float32
    cc = max(1, min(int(chan_chunk), C)) if C else 1
    bufs = [torch.empty((cc, P, nu, nv), dtype=gdt, device='cuda') for _ in range(min(2, max(C, 1)))]
    stage = None
    if out is None:
        stage = [torch.empty((cc, P, nu, nv), dtype=gdt, pin_memory=True) for _ in range(len(bufs))]
    done = [None] * len(bufs)       # event: the buffer's copy back has finished
    pending = [None] * len(bufs)    # (c0, c1) whose staged copy awaits on_chunk
    sw_h = torch.empty((C, P), dtype=torch.float64)
    sw_d = torch.empty((C, P), dtype=torch.float64, device='cuda')
    for i, c0 in enumerate(range(0, C, cc)):
        c1 = min(C, c0 + cc)
        k = i % len(bufs)
        if done[k] is not None:
            cur.wait_event(done[k])
            if pending[k] is not None and on_chunk is not None:
                done[k].synchronize()
                on_chunk(pending[k][0], pending[k][1], stage[k][:pending[k][1] - pending[k][0]])
                pending[k] = None
        g = bufs[k][:c1 - c0]
        grid_ps(v_t, uvw_t, w_t, freq[c0:c1], cgk_1D, (nu, nv), delta_lm, mode=mode, chan_mode='cube', layout=layout,
                support=support, oversampling=oversampling, grid=g, sum_weight=sw_d[c0:c1], chan_offset=c0,
                chan_total=C)
        ready = torch.cuda.Event()
        ready.record(cur)
        side.wait_event(ready)
        with torch.cuda.stream(side):
            if out is not None:
                out[c0:c1].copy_(g, non_blocking=True)
            else:
                stage[k][:c1 - c0].copy_(g, non_blocking=True)
                pending[k] = (c0, c1)
            ev = torch.cuda.Event()
            ev.record(side)
        done[k] = ev
        g.record_stream(side)
    sw_h.copy_(sw_d)
    side.synchronize()
    if on_chunk is not None:
        for k in range(len(bufs)):
            if pending[k] is not None:
                on_chunk(pending[k][0], pending[k][1], stage[k][:pending[k][1] - pending[k][0]])
    cur.wait_stream(side)
    return sw_h.numpy()


def direction_rotate(vis, uvw, row_field, freq, rotmat, phase_rotation, common_tangent_reprojection=True,
                     single_precision=True):
    """uvw rotation and visibility phase rotation (ngg_rotate_uvw + ngg_phase_rotate).
    vis complex64 (T,B,C,P) or None (uvw only); returns (uvw_rot (T,B,3) f64,
    vis_rot complex64 or complex128 (T,B,C,P), or None), CUDA tensors."""
    torch = _torch()
    uvw_t = _dev(uvw, torch.float64, 'uvw')
    T, B = int(uvw_t.shape[0]), int(uvw_t.shape[1])
    rf = _dev(row_field, torch.int32, 'row_field')
    mats = _dev(rotmat, torch.float64, 'rotmat')
    ph = _dev(phase_rotation, torch.float64, 'phase_rotation')
    n_field = int(mats.shape[0])
    if rf.numel() != T:
        raise ValueError('row_field must have one entry per time row')
    if T * B and (int(rf.min()) < 0 or int(rf.max()) >= n_field):
        raise ValueError('row_field index outside the field matrices')
    uvw_rot = torch.empty((T, B, 3), dtype=torch.float64, device='cuda')
    pd = torch.empty((T, B), dtype=torch.float64, device='cuda')
    _check(load().ngg_rotate_uvw(_ptr(uvw_t), _ptr(rf), T, B, _ptr(mats), _ptr(ph), n_field,
                                 1 if common_tangent_reprojection else 0, _ptr(uvw_rot), _ptr(pd), _stream()),
           'ngg_rotate_uvw')
    if vis is None:
        return uvw_rot, None
    v = _dev(vis, torch.complex64, 'vis')
    _, _, C, P = v.shape
    foc = _dev(np.asarray(freq, dtype=np.float64) / 299792458.0, torch.float64, 'freq_over_c')
    out = torch.empty(v.shape, dtype=torch.complex64 if single_precision else torch.complex128, device='cuda')
    _check(load().ngg_phase_rotate(_ptr(v), _ptr(pd), T, B, C, P, _ptr(foc), 1 if single_precision else 0,
                                   _ptr(out), _stream()), 'ngg_phase_rotate')
    return uvw_rot, out


def degrid_ps(grid, uvw, weight, freq, cgk_1D, n_time_baseline_chan_pol, delta_lm, chan_mode='cube',
              layout='natural', support=7, oversampling=100, vis=None, normalize=False):
    """Degrid (ngg_degrid_ps, the gridder's adjoint) or, with normalize,
    predict (ngg_predict_ps: each visibility divided by its kernel sum)."""
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
    name = 'ngg_predict_ps' if normalize else 'ngg_degrid_ps'
    _check(getattr(load(), name)(ctypes.byref(a), _stream()), name)
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


def _gcf_args(uvw_t, w_t, f_t, fidx_t, maps, ck_t, sup_t, slope_t, n_uv, delta_lm, oversampling, chan_mode,
              layout, mode):
    T, B, C, P = w_t.shape
    a = NggGcfArgs()
    a.mode = MODES[mode]
    a.chan_mode = CHAN_MODES[chan_mode]
    a.layout = LAYOUTS[layout]
    a.oversampling[0], a.oversampling[1] = int(oversampling[0]), int(oversampling[1])
    a.n_field = int(slope_t.shape[0])
    a.n_time, a.n_baseline, a.n_chan, a.n_pol = T, B, C, P
    a.n_u, a.n_v = int(n_uv[0]), int(n_uv[1])
    a.delta_lm[0], a.delta_lm[1] = float(delta_lm[0]), float(delta_lm[1])
    a.n_cf_baseline, a.n_cf_chan, a.n_cf_pol = (int(x) for x in ck_t.shape[:3])
    a.conv_size[0], a.conv_size[1] = int(ck_t.shape[3]), int(ck_t.shape[4])
    a.uvw = _ptr(uvw_t).value
    a.weight = _ptr(w_t).value
    a.freq = _ptr(f_t).value
    a.field_index = _ptr(fidx_t).value
    a.cf_baseline_map, a.cf_chan_map, a.cf_pol_map = (_ptr(m).value for m in maps)
    a.conv_kernel = _ptr(ck_t).value
    a.support = _ptr(sup_t).value
    a.phase_slope = _ptr(slope_t).value
    return a


def _gcf_inputs(uvw, weight, freq, field_index, cf_baseline_map, cf_chan_map, cf_pol_map, conv_kernel, support,
                phase_slope):
    torch = _torch()
    uvw_t = _dev(uvw, torch.float64, 'uvw')
    w_t = _dev(weight, torch.float32, 'weight')
    f_t = _dev(freq, torch.float64, 'freq')
    fidx_t = _dev(field_index, torch.int32, 'field_index')
    maps = [_dev(m, torch.int32, n) for m, n in ((cf_baseline_map, 'cf_baseline_map'), (cf_chan_map, 'cf_chan_map'),
                                                 (cf_pol_map, 'cf_pol_map'))]
    ck_t = _dev(conv_kernel, torch.float64, 'conv_kernel')
    sup_t = _dev(support, torch.int32, 'support')
    slope_t = _dev(phase_slope, torch.float64, 'phase_slope')
    if ck_t.dim() != 5 or tuple(sup_t.shape) != tuple(ck_t.shape[:3]) + (2,):
        raise NggError('conv_kernel must be (n_cf_baseline, n_cf_chan, n_cf_pol, R0, R1) and support (..., 2)')
    T, B, C, P = w_t.shape
    if tuple(fidx_t.shape) != (T, B) or maps[0].numel() != B or maps[1].numel() != C or maps[2].numel() != P:
        raise NggError('field_index must be (T, B) and the CF maps (B,), (C,), (P,)')
    return uvw_t, w_t, f_t, fidx_t, maps, ck_t, sup_t, slope_t


def grid_gcf(vis, uvw, weight, freq, field_index, cf_baseline_map, cf_chan_map, cf_pol_map, conv_kernel, support,
             phase_slope, n_uv, delta_lm, oversampling, mode='data', chan_mode='cube', layout='natural'):
    """Mosaic gridder with a GCF table: (grid complex64 (Cimg,P,Nu,Nv), sum_weight (Cimg,P) f64)."""
    torch = _torch()
    ins = _gcf_inputs(uvw, weight, freq, field_index, cf_baseline_map, cf_chan_map, cf_pol_map, conv_kernel,
                      support, phase_slope)
    w_t = ins[1]
    T, B, C, P = w_t.shape
    v_t = _dev(vis, torch.complex64, 'vis') if mode == 'data' else None
    n_img = 1 if chan_mode == 'continuum' else C
    grid = torch.empty((n_img, P, int(n_uv[0]), int(n_uv[1])), dtype=torch.complex64, device='cuda')
    sw = torch.empty((n_img, P), dtype=torch.float64, device='cuda')
    a = _gcf_args(*ins, n_uv, delta_lm, oversampling, chan_mode, layout, mode)
    a.vis = _ptr(v_t).value
    a.grid = _ptr(grid).value
    a.sum_weight = _ptr(sw).value
    _check(load().ngg_grid_gcf(ctypes.byref(a), _stream()), 'ngg_grid_gcf')
    return grid, sw


def grid_gcf_weight(uvw, weight, freq, field_index, cf_baseline_map, cf_chan_map, cf_pol_map, weight_conv_kernel,
                    support, phase_slope, n_uv, delta_lm, oversampling, chan_mode='cube', layout='natural'):
    """Mosaic weight grid (every tap at the grid centre): (grid, sum_weight)."""
    torch = _torch()
    ins = _gcf_inputs(uvw, weight, freq, field_index, cf_baseline_map, cf_chan_map, cf_pol_map, weight_conv_kernel,
                      support, phase_slope)
    T, B, C, P = ins[1].shape
    n_img = 1 if chan_mode == 'continuum' else C
    grid = torch.empty((n_img, P, int(n_uv[0]), int(n_uv[1])), dtype=torch.complex64, device='cuda')
    sw = torch.empty((n_img, P), dtype=torch.float64, device='cuda')
    a = _gcf_args(*ins, n_uv, delta_lm, oversampling, chan_mode, layout, 'psf')
    a.grid = _ptr(grid).value
    a.sum_weight = _ptr(sw).value
    _check(load().ngg_grid_gcf_weight(ctypes.byref(a), _stream()), 'ngg_grid_gcf_weight')
    return grid, sw


def gcf_kernels(function, dish_diameters, blockage_diameters, pairs, freq, n, cell, center):
    """FP64 baseline GCFs before cropping: (conv_kernel, weight_conv_kernel), each (n_pairs, n_freq, n0, n1)."""
    torch = _torch()
    d_t = _dev(np.asarray(dish_diameters, dtype=np.float64), torch.float64, 'dish_diameters')
    b_t = _dev(np.asarray(blockage_diameters, dtype=np.float64), torch.float64, 'blockage_diameters')
    p_t = _dev(np.asarray(pairs, dtype=np.int32).reshape(-1, 2), torch.int32, 'pairs')
    f_t = _dev(np.asarray(freq, dtype=np.float64), torch.float64, 'freq')
    n0, n1 = int(n[0]), int(n[1])
    npair, nf = int(p_t.shape[0]), int(f_t.shape[0])
    ck = torch.empty((npair, nf, n0, n1), dtype=torch.float64, device='cuda')
    wk = torch.empty_like(ck)
    _check(load().ngg_gcf_kernels(1 if function == 'casa_airy' else 0, int(d_t.shape[0]), _ptr(d_t), _ptr(b_t),
                                  npair, _ptr(p_t), nf, _ptr(f_t), n0, n1, _dl(cell), int(center[0]), int(center[1]),
                                  _ptr(ck), _ptr(wk), _stream()), 'ngg_gcf_kernels')
    return ck, wk


def mosaic_normalize(image, ps_corr=None, norm_image=None, pb=None, pb_limit=0.0, oversampling=(1, 1),
                     single_precision=False, centre=None):
    """In-place mosaic normalisation of image (l, m, C, P) float64 (see ngg.h)."""
    torch = _torch()
    if image.dtype != torch.float64 or not image.is_cuda or not image.is_contiguous():
        raise NggError('image must be a contiguous float64 CUDA tensor')
    nl, nm = int(image.shape[0]), int(image.shape[1])
    npl = int(image.numel() // max(nl * nm, 1))
    ps_t = _dev(ps_corr, torch.float64, 'ps_corr', allow_none=True)
    n_t = _dev(norm_image, torch.float64, 'norm_image', allow_none=True)
    pb_t = _dev(pb, torch.float64, 'pb', allow_none=True)
    for t, n in ((n_t, 'norm_image'), (pb_t, 'pb')):
        if t is not None and t.numel() != image.numel():
            raise NggError(f'{n} must have the shape of image')
    if ps_t is not None and ps_t.numel() != nl * nm:
        raise NggError('ps_corr must be (n_l, n_m)')
    os_ = (ctypes.c_int * 2)(int(oversampling[0]), int(oversampling[1]))
    cen = (ctypes.c_int64 * 2)(int(centre[0]), int(centre[1])) if centre is not None else None
    _check(load().ngg_mosaic_normalize(_ptr(image), nl, nm, npl, _ptr(ps_t), _ptr(n_t), _ptr(pb_t), float(pb_limit),
                                       os_, 1 if single_precision else 0, cen, _stream()), 'ngg_mosaic_normalize')
    return image


def sqrt_abs(x):
    torch = _torch()
    x = _dev(x, torch.float64, 'x')
    out = torch.empty_like(x)
    _check(load().ngg_sqrt_abs(_ptr(x), int(x.numel()), _ptr(out), _stream()), 'ngg_sqrt_abs')
    return out


def _params(params):
    torch = _torch()
    p = _dev(params, torch.float32, 'params')
    if p.numel() != MLP_NPARAM:
        raise NggError(f'params must hold {MLP_NPARAM} float32 values')
    return p


def mlp_forward(params, z, tensor_cores=False):
    """Network output for z (n, 3) float32: FP32 CUDA cores, or the tcgen05 BF16 path."""
    torch = _torch()
    p = _params(params)
    z_t = _dev(z, torch.float32, 'z')
    n = int(z_t.shape[0])
    y = torch.empty((n,), dtype=torch.float32, device='cuda')
    f = load().ngg_mlp_forward_tc if tensor_cores else load().ngg_mlp_forward
    _check(f(_ptr(p), _ptr(z_t), n, _ptr(y), _stream()), 'ngg_mlp_forward' + ('_tc' if tensor_cores else ''))
    return y


def mlp_loss_grad(params, z, target):
    torch = _torch()
    p = _params(params)
    z_t = _dev(z, torch.float32, 'z')
    t_t = _dev(target, torch.float32, 'target')
    g = torch.empty((MLP_NPARAM,), dtype=torch.float32, device='cuda')
    loss = torch.empty((1,), dtype=torch.float64, device='cuda')
    _check(load().ngg_mlp_loss_grad(_ptr(p), _ptr(z_t), _ptr(t_t), int(z_t.shape[0]), _ptr(g), _ptr(loss), _stream()),
           'ngg_mlp_loss_grad')
    return float(loss.item()), g


def mlp_adam(params, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """In-place Adam step on the CUDA tensors params / m / v."""
    _check(load().ngg_mlp_adam(_ptr(params), _ptr(grad), _ptr(m), _ptr(v), float(lr), float(beta1), float(beta2),
                               float(eps), int(step), _stream()), 'ngg_mlp_adam')


def mlp_train(params, m, v, z, target, n_steps, step0=0, batch=65536, lr0=3e-3, lr1=3e-5, seed=0):
    """n_steps Adam steps on random batches, in place; returns the per-step loss (CUDA float64)."""
    torch = _torch()
    z_t = _dev(z, torch.float32, 'z')
    t_t = _dev(target, torch.float32, 'target')
    hist = torch.empty((max(int(n_steps), 1),), dtype=torch.float64, device='cuda')
    _check(load().ngg_mlp_train(_ptr(params), _ptr(m), _ptr(v), _ptr(z_t), _ptr(t_t), int(z_t.shape[0]), int(batch),
                                int(n_steps), int(step0), float(lr0), float(lr1), ctypes.c_uint64(int(seed)),
                                _ptr(hist), _stream()), 'ngg_mlp_train')
    return hist[:int(n_steps)]


def grid_gcf_learned(vis, uvw, weight, freq, field_index, support, phase_slope, params, scale, conv_size, n_uv,
                     delta_lm, oversampling, mode='data', chan_mode='cube', layout='natural'):
    """Mosaic gridder with per-channel GCF tables synthesised by the network.
    support int32 (C, 2) per channel; scale: dict of NggMlpScale fields."""
    torch = _torch()
    uvw_t = _dev(uvw, torch.float64, 'uvw')
    w_t = _dev(weight, torch.float32, 'weight')
    f_t = _dev(freq, torch.float64, 'freq')
    fidx_t = _dev(field_index, torch.int32, 'field_index')
    sup_t = _dev(support, torch.int32, 'support')
    slope_t = _dev(phase_slope, torch.float64, 'phase_slope')
    p = _params(params)
    T, B, C, P = w_t.shape
    if tuple(sup_t.shape) != (C, 2):
        raise NggError('support must be (n_chan, 2)')
    v_t = _dev(vis, torch.complex64, 'vis') if mode == 'data' else None
    n_img = 1 if chan_mode == 'continuum' else C
    grid = torch.empty((n_img, P, int(n_uv[0]), int(n_uv[1])), dtype=torch.complex64, device='cuda')
    sw = torch.empty((n_img, P), dtype=torch.float64, device='cuda')
    a = NggGcfArgs()
    a.mode = MODES[mode]
    a.chan_mode = CHAN_MODES[chan_mode]
    a.layout = LAYOUTS[layout]
    a.oversampling[0], a.oversampling[1] = int(oversampling[0]), int(oversampling[1])
    a.n_field = int(slope_t.shape[0])
    a.n_time, a.n_baseline, a.n_chan, a.n_pol = T, B, C, P
    a.n_u, a.n_v = int(n_uv[0]), int(n_uv[1])
    a.delta_lm[0], a.delta_lm[1] = float(delta_lm[0]), float(delta_lm[1])
    a.n_cf_baseline, a.n_cf_chan, a.n_cf_pol = 1, C, 1
    a.conv_size[0], a.conv_size[1] = int(conv_size[0]), int(conv_size[1])
    a.vis = _ptr(v_t).value
    a.uvw = _ptr(uvw_t).value
    a.weight = _ptr(w_t).value
    a.freq = _ptr(f_t).value
    a.field_index = _ptr(fidx_t).value
    a.support = _ptr(sup_t).value
    a.phase_slope = _ptr(slope_t).value
    a.grid = _ptr(grid).value
    a.sum_weight = _ptr(sw).value
    sc = NggMlpScale(**{k: float(scale[k]) for k in ('x_scale', 'y_scale', 'f_center', 'f_scale', 'out_scale')})
    _check(load().ngg_grid_gcf_learned(ctypes.byref(a), _ptr(p), ctypes.byref(sc), _stream()), 'ngg_grid_gcf_learned')
    return grid, sw


def set_profiling(enable=True):
    load().ngg_set_profiling(1 if enable else 0)


def last_phase_ms():
    """(binning_ms, tiles_ms) of the last profiled ngg_grid_ps call on this thread."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(load().ngg_last_phase_ms(ctypes.byref(a), ctypes.byref(b)), 'ngg_last_phase_ms')
    return a.value, b.value
