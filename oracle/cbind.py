"""ctypes binding and build recipe for oracle/ngg_oracle.c (test infrastructure)."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'ngg_oracle.c')
LIB = os.path.join(HERE, 'libngg_oracle.so')

_lib = None


def build(force=False):
    """Compile the C oracle (gcc, OpenMP, no FP contraction, portable flags)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ['gcc', '-O3', '-fopenmp', '-ffp-contract=off', '-fno-fast-math', '-fPIC', '-shared',
           '-std=c11', SRC, '-o', LIB + '.tmp', '-lm']
    subprocess.check_call(cmd)
    os.replace(LIB + '.tmp', LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.ngg_oracle_grid.argtypes = [ctypes.c_int, P, P, P, i64, i64, i64, i64, P, P, ctypes.c_int,
                                      ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int, P, P]
        L.ngg_oracle_grid.restype = ctypes.c_int
        L.ngg_oracle_weight_degrid.argtypes = [P, P, P, P, i64, i64, i64, i64, P, P, P, ctypes.c_int,
                                               ctypes.c_int, P]
        L.ngg_oracle_weight_degrid.restype = ctypes.c_int
        L.ngg_oracle_aperture_grid.argtypes = [ctypes.c_int, P, P, P, P, i64, i64, i64, i64, P, P, P, P, i64, i64,
                                               i64, P, P, P, i64, i64, i64, P, P, P, ctypes.c_int, ctypes.c_int,
                                               P, P]
        L.ngg_oracle_aperture_grid.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


MODES = {'data': 0, 'psf': 1, 'density': 2}


def grid(mode, vis, uvw, weight, freq, cgk_1D, support, oversampling, n_uv, delta_lm,
         chan_mode='cube', n_threads=0):
    """Standard gridder in FP64. Returns (grid[Cimg,P,Nu,Nv], sum_weight[Cimg,P])."""
    uvw = np.ascontiguousarray(uvw, dtype=np.float64)
    weight = np.ascontiguousarray(weight, dtype=np.float64)
    T, B, C, P = weight.shape
    v = None
    if mode == 'data':
        v = np.ascontiguousarray(vis, dtype=np.complex64)
    freq = np.ascontiguousarray(freq, dtype=np.float64)
    cgk = np.ascontiguousarray(cgk_1D, dtype=np.float64)
    n_uv = np.ascontiguousarray(np.asarray(n_uv), dtype=np.int64)
    dl = np.ascontiguousarray(np.asarray(delta_lm), dtype=np.float64)
    cont = 1 if chan_mode == 'continuum' else 0
    n_img = 1 if cont else C
    gdt = np.complex128 if mode == 'data' else np.float64
    g = np.empty((n_img, P, int(n_uv[0]), int(n_uv[1])), dtype=gdt)
    sw = np.empty((n_img, P), dtype=np.float64)
    rc = lib().ngg_oracle_grid(MODES[mode], _p(v), _p(uvw), _p(weight), T, B, C, P, _p(freq), _p(cgk),
                               int(support), int(oversampling), _p(n_uv), _p(dl), cont, int(n_threads),
                               _p(g), _p(sw))
    if rc != 0:
        raise RuntimeError('ngg_oracle_grid failed')
    return g, sw


def weight_degrid(density_uvcp, uvw, weight, briggs, freq, n_uv, delta_lm, chan_mode='cube',
                  n_threads=0):
    density_uvcp = np.ascontiguousarray(density_uvcp, dtype=np.float64)
    uvw = np.ascontiguousarray(uvw, dtype=np.float64)
    weight = np.ascontiguousarray(weight, dtype=np.float64)
    briggs = np.ascontiguousarray(briggs, dtype=np.float64)
    T, B, C, P = weight.shape
    n_uv = np.ascontiguousarray(np.asarray(n_uv), dtype=np.int64)
    dl = np.ascontiguousarray(np.asarray(delta_lm), dtype=np.float64)
    out = np.empty(weight.shape, dtype=np.float64)
    rc = lib().ngg_oracle_weight_degrid(_p(density_uvcp), _p(uvw), _p(weight), _p(briggs), T, B, C, P,
                                        _p(np.ascontiguousarray(freq, dtype=np.float64)), _p(n_uv), _p(dl),
                                        1 if chan_mode == 'continuum' else 0, int(n_threads), _p(out))
    if rc != 0:
        raise RuntimeError('ngg_oracle_weight_degrid failed')
    return out


APERTURE_KINDS = {'data': 0, 'psf': 1, 'weight': 2}


def aperture_grid(kind, vis, uvw, imaging_weight, field_index, cf_baseline_map, cf_chan_map, cf_pol_map, table,
                  support, phase_gradient, freq, oversampling, n_uv, delta_lm, chan_mode='cube', n_threads=0):
    """Mosaic gridders in FP64 (_aperture_grid_jit / _aperture_weight_grid_jit).
    field_index: (T, B) index into the phase-gradient planes, < 0 skips.
    Returns (grid complex128 (Cimg, P, Nu, Nv), sum_weight (Cimg, P))."""
    i64 = np.int64
    uvw = np.ascontiguousarray(uvw, dtype=np.float64)
    w = np.ascontiguousarray(imaging_weight, dtype=np.float64)
    T, B, C, P = w.shape
    v = np.ascontiguousarray(vis, dtype=np.complex64) if kind == 'data' else None
    fidx = np.ascontiguousarray(field_index, dtype=i64)
    maps = [np.ascontiguousarray(m, dtype=i64) for m in (cf_baseline_map, cf_chan_map, cf_pol_map)]
    tab = np.ascontiguousarray(table, dtype=np.float64)
    sup = np.ascontiguousarray(support, dtype=i64)
    pg = np.ascontiguousarray(phase_gradient, dtype=np.complex128)
    os_ = np.ascontiguousarray(oversampling, dtype=i64)
    nuv = np.ascontiguousarray(n_uv, dtype=i64)
    dl = np.ascontiguousarray(delta_lm, dtype=np.float64)
    f = np.ascontiguousarray(freq, dtype=np.float64)
    cont = 1 if chan_mode == 'continuum' else 0
    n_img = 1 if cont else C
    g = np.empty((n_img, P, int(nuv[0]), int(nuv[1])), dtype=np.complex128)
    sw = np.empty((n_img, P), dtype=np.float64)
    ncfb, ncfc, ncfp, R0, R1 = tab.shape
    rc = lib().ngg_oracle_aperture_grid(APERTURE_KINDS[kind], _p(v), _p(uvw), _p(w), _p(fidx), T, B, C, P, _p(f),
                                        _p(maps[0]), _p(maps[1]), _p(maps[2]), ncfb, ncfc, ncfp, _p(tab), _p(sup),
                                        _p(pg), pg.shape[0], R0, R1, _p(os_), _p(nuv), _p(dl), cont,
                                        int(n_threads), _p(g), _p(sw))
    if rc != 0:
        raise RuntimeError('ngg_oracle_aperture_grid failed')
    return g, sw
