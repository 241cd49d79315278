"""numpy FP64 restatement of the reference's standard-gridder imaging path.

Test infrastructure (see ``oracle/__init__.py``). Every function cites the
reference file:line (paths relative to the reference project) whose behaviour
it restates. Accumulations are done with ``np.add.at`` over index arrays laid
out in the reference's loop order, so each grid cell and each sum-of-weights
entry receives its addends in exactly the same sequence as the reference's
scalar loops; small cases are therefore bit-identical to the reference.
"""
import numpy as np

C_LIGHT = 299792458.0
ARCSEC_TO_RAD = np.pi / (3600 * 180)


# --------------------------------------------------------------------------
# parameter handling
# --------------------------------------------------------------------------
def check_grid_parms(grid_parms):
    """Fill derived grid parameters in place.

    Restates ngcasa/imaging/_imaging_utils/_check_imaging_parms.py:23-41:
    defaults (image_center = image_size//2, fft_padding 1.2, chan_mode cube),
    image_size_padded = int(fft_padding * image_size), cell_size arcsec -> rad
    with the sign of cell_size[0] flipped.
    """
    g = grid_parms
    g.setdefault('fft_padding', 1.2)
    g.setdefault('chan_mode', 'cube')
    g.setdefault('image_center', np.array(g['image_size']) // 2)
    if g['chan_mode'] not in ('cube', 'continuum'):
        raise ValueError("chan_mode must be 'cube' or 'continuum'")
    g['image_size'] = np.array(g['image_size']).astype(int)
    g['image_size_padded'] = (g['fft_padding'] * g['image_size']).astype(int)
    g['image_center'] = np.array(g['image_center'])
    g['cell_size'] = ARCSEC_TO_RAD * np.array(g['cell_size'], dtype=np.float64)
    g['cell_size'][0] = -g['cell_size'][0]
    return True


def uv_scale(freq_chan, delta_lm, n_uv):
    """uv_scale[2, n_chan] (ngcasa/imaging/_imaging_utils/_standard_grid.py:273-276)."""
    freq_chan = np.asarray(freq_chan, dtype=np.float64)
    s = np.zeros((2, len(freq_chan)), dtype=np.double)
    s[0, :] = -(freq_chan * delta_lm[0] * n_uv[0]) / C_LIGHT
    s[1, :] = -(freq_chan * delta_lm[1] * n_uv[1]) / C_LIGHT
    return s


# --------------------------------------------------------------------------
# prolate spheroidal kernel (_gridding_convolutional_kernels.py)
# --------------------------------------------------------------------------
_PS_P = np.array([[8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1],
                  [4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2]])
_PS_Q = np.array([[1.0000000e0, 8.212018e-1, 2.078043e-1],
                  [1.0000000e0, 9.599102e-1, 2.918724e-1]])


def prolate_spheroidal_function(u):
    """Schwab's rational approximation, M=6 alpha=1.

    Restates _gridding_convolutional_kernels.py:101-148 (the coefficient table
    is the published Schwab table). Returns (grdsf,
    (1-u^2)*grdsf); zero for |u|>1.
    """
    u = np.abs(np.asarray(u, dtype=np.float64))
    uend = np.zeros(u.shape, dtype=np.float64)
    part = np.zeros(u.shape, dtype=np.int64)
    part[(u >= 0.0) & (u < 0.75)] = 0
    part[(u >= 0.75) & (u <= 1.0)] = 1
    uend[(u >= 0.0) & (u < 0.75)] = 0.75
    uend[(u >= 0.75) & (u <= 1.0)] = 1.0
    delusq = u ** 2 - uend ** 2
    top = _PS_P[part, 0]
    for k in range(1, _PS_P.shape[1]):
        top += _PS_P[part, k] * np.power(delusq, k)
    bot = _PS_Q[part, 0]
    for k in range(1, _PS_Q.shape[1]):
        bot += _PS_Q[part, k] * np.power(delusq, k)
    grdsf = np.zeros(u.shape, dtype=np.float64)
    ok = bot > 0.0
    grdsf[ok] = top[ok] / bot[ok]
    grdsf[np.abs(u > 1.0)] = 0.0
    return grdsf, (1 - u ** 2) * grdsf


def create_prolate_spheroidal_kernel_1D(oversampling, support):
    """Half-kernel table of length oversampling*(support//2+1).

    Restates _gridding_convolutional_kernels.py:151-158; entries at and beyond
    oversampling*(support//2) are zero.
    """
    support_center = support // 2
    u = np.arange(oversampling * support_center) / (support_center * oversampling)
    k = np.zeros(oversampling * (support_center + 1))
    _, k[0:oversampling * support_center] = prolate_spheroidal_function(u)
    return k


def _coordinates(npixel):
    return (np.arange(npixel) - npixel // 2) / npixel


def create_prolate_spheroidal_correction(n_uv):
    """Grid-correction image outer(grdsf(|2x|)) over the padded grid.

    Restates _gridding_convolutional_kernels.py:86-93 (the second return value
    of _create_prolate_spheroidal_kernel).
    """
    cu = prolate_spheroidal_function(np.abs(2.0 * _coordinates(int(n_uv[0]))))[0]
    cv = prolate_spheroidal_function(np.abs(2.0 * _coordinates(int(n_uv[1]))))[0]
    return np.outer(cu, cv)


def remove_padding(image, image_size):
    """Centre crop (ngcasa/imaging/_imaging_utils/_remove_padding.py:20-31)."""
    image_size = np.asarray(image_size)
    padded = np.array(image.shape[0:2])
    start = padded // 2 - image_size // 2
    end = start + image_size
    return image[start[0]:end[0], start[1]:end[1]]


# --------------------------------------------------------------------------
# standard gridder (_standard_grid.py:123-371)
# --------------------------------------------------------------------------
def _positions(uvw, scale, uv_center):
    """Pixel positions, nearest cells and the NaN mask for a block of rows.

    Restates _standard_grid.py:299-318: u = uvw_u*uv_scale, u_pos = u +
    centre, centre index int(u_pos+0.5) (truncation toward zero), and the
    mirrored position -u + centre used by the weight-density mode.
    """
    u = uvw[:, :, 0][:, :, None] * scale[0][None, None, :]
    v = uvw[:, :, 1][:, :, None] * scale[1][None, None, :]
    ok = ~np.isnan(u) & ~np.isnan(v)
    u = np.where(ok, u, 0.0)
    v = np.where(ok, v, 0.0)
    u_pos = u + uv_center[0]
    v_pos = v + uv_center[1]
    cu = np.trunc(u_pos + 0.5)
    cv = np.trunc(v_pos + 0.5)
    u_pos_c = -u + uv_center[0]
    v_pos_c = -v + uv_center[1]
    cu_c = np.trunc(u_pos_c + 0.5)
    cv_c = np.trunc(v_pos_c + 0.5)
    return ok, u_pos, v_pos, cu, cv, cu_c, cv_c


def standard_grid(vis_data, uvw, weight, freq_chan, cgk_1D, n_uv, delta_lm,
                  support, oversampling, do_psf, do_imaging_weight=False,
                  complex_grid=None, chan_mode='cube', rows_per_block=64):
    """Convolutional gridding with a separable 1-D kernel table.

    Restates _standard_grid_numpy_wrap / _standard_grid_psf_numpy_wrap
    (_standard_grid.py:123-236) and _standard_grid_jit (:242-371):

    * data mode (do_psf False): grid[c,p,u,v] += conv * vis*weight (complex);
    * psf mode (do_psf True): grid += conv * weight (real grid);
    * weight-density mode (do_psf and do_imaging_weight): weight is the
      two-pol average, the mirrored cell (-u,-v) is also incremented and
      sum_weight is incremented twice (:327-333, :349-369).

    A visibility is skipped when u or v is NaN, when any tap would leave the
    grid (:320), or when the weighted datum is NaN or zero (:340).
    sum_weight[c,p] += weight * sum(conv) (:366).

    vis_data: (T,B,C,P) complex or None in psf mode; uvw (T,B,3) float64;
    weight (T,B,C,P); freq_chan (C,). Returns (grid[Cimg,P,Nu,Nv],
    sum_weight[Cimg,P]).
    """
    uvw = np.asarray(uvw, dtype=np.float64)
    weight = np.asarray(weight)
    n_uv = np.asarray(n_uv).astype(np.int64)
    T, B = uvw.shape[:2]
    C, P = weight.shape[2], weight.shape[3]
    if chan_mode == 'cube':
        n_imag_chan = C
        chan_map = np.arange(C)
    else:
        n_imag_chan = 1
        chan_map = np.zeros(C, dtype=np.int64)
    if complex_grid is None:
        complex_grid = not do_psf
    gdtype = np.complex128 if complex_grid else np.double
    grid = np.zeros((n_imag_chan, P, int(n_uv[0]), int(n_uv[1])), dtype=gdtype)
    sum_weight = np.zeros((n_imag_chan, P), dtype=np.double)
    if T == 0 or B == 0 or C == 0 or P == 0:
        return grid, sum_weight

    scale = uv_scale(freq_chan, delta_lm, n_uv)
    support_center = int(support // 2)
    uv_center = n_uv // 2
    taps = np.arange(-support_center, support - support_center)
    S = len(taps)
    cgk_1D = np.asarray(cgk_1D, dtype=np.float64)
    n_u, n_v = int(n_uv[0]), int(n_uv[1])

    for t0 in range(0, T, rows_per_block):
        t1 = min(T, t0 + rows_per_block)
        ok, u_pos, v_pos, cu, cv, cu_c, cv_c = _positions(uvw[t0:t1], scale, uv_center)
        ok = ok & (cu + support_center < n_u) & (cv + support_center < n_v) \
            & (cu - support_center >= 0) & (cv - support_center >= 0)
        # offsets into the oversampled table (:321-324)
        off_u = np.floor((cu - u_pos) * oversampling + 0.5)
        off_v = np.floor((cv - v_pos) * oversampling + 0.5)
        w = weight[t0:t1].astype(np.float64) if weight.dtype != np.float64 else weight[t0:t1]
        nt = t1 - t0
        # weighted data per pol (:326-336)
        if do_psf:
            if P >= 2 and do_imaging_weight:
                avg = (w[..., 0] + w[..., 1]) / 2.0
                wd = np.repeat(avg[..., None], P, axis=-1)
                selw = wd
            else:
                wd = w
                selw = w
        else:
            vd = vis_data[t0:t1]
            wd = vd * w  # complex64 * float64 -> complex128, as in the reference
            selw = w
        valid = ok[..., None] & ~np.isnan(wd) & (wd != 0.0)   # (t,B,C,P)
        idx = np.nonzero(valid)   # lexicographic (t,b,c,p) = reference loop order
        if len(idx[0]) == 0:
            continue
        ti, bi, ci, pi = idx
        ou = off_u[ti, bi, ci].astype(np.int64)
        ov = off_v[ti, bi, ci].astype(np.int64)
        cuv = cu[ti, bi, ci].astype(np.int64)
        cvv = cv[ti, bi, ci].astype(np.int64)
        conv_v = cgk_1D[np.abs(oversampling * taps[None, :] + ov[:, None])]   # (n,S) over i_v
        conv_u = cgk_1D[np.abs(oversampling * taps[None, :] + ou[:, None])]   # (n,S) over i_u
        conv = conv_u[:, None, :] * conv_v[:, :, None]                        # (n, i_v, i_u)
        val = wd[ti, bi, ci, pi]
        contrib = conv * val[:, None, None]
        a_chan = chan_map[ci]
        uu = cuv[:, None, None] + taps[None, None, :]
        vv = cvv[:, None, None] + taps[None, :, None]
        shp = conv.shape
        if do_imaging_weight:
            cuc = cu_c[ti, bi, ci].astype(np.int64)
            cvc = cv_c[ti, bi, ci].astype(np.int64)
            uuc = cuc[:, None, None] + taps[None, None, :]
            vvc = cvc[:, None, None] + taps[None, :, None]
            # per tap: main cell then mirrored cell, in (i_v, i_u) order
            U = np.stack([np.broadcast_to(uu, shp), np.broadcast_to(uuc, shp)], axis=-1)
            V = np.stack([np.broadcast_to(vv, shp), np.broadcast_to(vvc, shp)], axis=-1)
            Cc = np.broadcast_to(a_chan[:, None, None, None], U.shape)
            Pp = np.broadcast_to(pi[:, None, None, None], U.shape)
            X = np.stack([contrib, contrib], axis=-1)
            inb = (U >= 0) & (U < n_u) & (V >= 0) & (V < n_v)
            np.add.at(grid, (Cc[inb], Pp[inb], U[inb], V[inb]), X[inb])
        else:
            Cc = np.broadcast_to(a_chan[:, None, None], shp)
            Pp = np.broadcast_to(pi[:, None, None], shp)
            np.add.at(grid, (Cc.ravel(), Pp.ravel(), np.broadcast_to(uu, shp).ravel(),
                             np.broadcast_to(vv, shp).ravel()), contrib.ravel())
        # norm = sequential sum over (i_v, i_u)
        flat = conv.reshape(len(ti), -1)
        norm = np.zeros(len(ti))
        for k in range(flat.shape[1]):
            norm = norm + flat[:, k]
        sw = selw[ti, bi, ci, pi] * norm
        if do_imaging_weight:
            np.add.at(sum_weight, (np.repeat(a_chan, 2), np.repeat(pi, 2)), np.repeat(sw, 2))
        else:
            np.add.at(sum_weight, (a_chan, pi), sw)
    return grid, sum_weight


def grid_weight_density(uvw, weight, freq_chan, grid_parms):
    """Weight-density grid for Briggs/uniform weighting.

    Restates calc_briggs_weights' gridding setup (make_imaging_weight.py:
    153-161): unpadded grid, oversampling 0, support 1, cgk_1D=[1], psf mode
    with do_imaging_weight. Returns (density[C,P,N,N], sum_weight[C,P]).
    """
    return standard_grid(None, uvw, weight, freq_chan, np.ones(1),
                         np.asarray(grid_parms['image_size']),
                         grid_parms['cell_size'], 1, 0, True, True, False,
                         grid_parms.get('chan_mode', 'cube'))


def calculate_briggs_parms(density_uvcp, sum_weight, imaging_weights_parms):
    """Briggs factors [2,C,P] (make_imaging_weight.py:198-213).

    briggs: f0 = (5*10^-robust)^2 / (sum(W^2)/sum_weight), f1 = 1;
    uniform: f0 = 1, f1 = 0. The reference's briggs_abs branch references an
    undefined name (make_imaging_weight.py:207-208); here briggs_abs follows
    its documented intent, f0 = robust^2, f1 = 2*noise^2.
    """
    weighting = imaging_weights_parms['weighting']
    if weighting == 'briggs':
        robust = imaging_weights_parms['robust']
        f = np.ones((2,) + sum_weight.shape)
        sq = np.sum(density_uvcp ** 2, axis=(0, 1))
        f[0] = np.square(5.0 * 10.0 ** (-robust)) / (sq / sum_weight)
    elif weighting == 'briggs_abs':
        robust = imaging_weights_parms['robust']
        f = np.ones((2,) + sum_weight.shape)
        f[0] = np.square(robust)
        f[1] = 2.0 * np.square(imaging_weights_parms.get('briggs_abs_noise', 1.0))
    else:
        f = np.zeros((2,) + sum_weight.shape)
        f[0] = 1.0
    return f


def standard_imaging_weight_degrid(density_uvcp, uvw, natural_weight, briggs_factors,
                                   freq_chan, n_uv, delta_lm, chan_mode='cube'):
    """Nearest-cell weight-density lookup -> imaging weights (T,B,C,P) f64.

    Restates _standard_imaging_weight_degrid_numpy_wrap (_standard_grid.py:
    443-464) and _standard_imaging_weight_degrid_jit (:466-518): cell =
    int(pos+0.5), kept when 0<=cell<n; two-pol weights are averaged; divided
    by f0*W+f1 when both the pol's own weight and W are finite and non-zero.
    Rows whose cell is off the grid or whose uvw is NaN stay 0.
    """
    uvw = np.asarray(uvw, dtype=np.float64)
    w = np.asarray(natural_weight, dtype=np.float64)
    n_uv = np.asarray(n_uv).astype(np.int64)
    T, B = uvw.shape[:2]
    C, P = w.shape[2], w.shape[3]
    out = np.zeros(w.shape, dtype=np.double)
    if w.size == 0:
        return out
    chan_map = np.arange(C) if chan_mode == 'cube' else np.zeros(C, dtype=np.int64)
    scale = uv_scale(freq_chan, delta_lm, n_uv)
    ok, u_pos, v_pos, cu, cv, _, _ = _positions(uvw, scale, n_uv // 2)
    ok = ok & (cu < n_uv[0]) & (cv < n_uv[1]) & (cu >= 0) & (cv >= 0)
    cui = np.where(ok, cu, 0).astype(np.int64)
    cvi = np.where(ok, cv, 0).astype(np.int64)
    for p in range(P):
        if P == 2:
            iw = (w[..., 0] + w[..., 1]) / 2.0
        else:
            iw = w[..., p].copy()
        a_chan = np.broadcast_to(chan_map[None, None, :], (T, B, C))
        W = density_uvcp[cui, cvi, a_chan, p]
        good = ok & ~np.isnan(w[..., p]) & (w[..., p] != 0.0) & ~np.isnan(W) & (W != 0.0)
        f0 = briggs_factors[0][a_chan, p]
        f1 = briggs_factors[1][a_chan, p]
        iw = np.where(good, iw / np.where(good, f0 * W + f1, 1.0), iw)
        out[..., p] = np.where(ok, iw, 0.0)
    return out


def make_imaging_weight(uvw, weight, freq_chan, grid_parms, imaging_weights_parms):
    """Imaging weights as make_imaging_weight computes them per cube chunk.

    Restates make_imaging_weight.py:94-109 + calc_briggs_weights (:144-255)
    for a single chunk: natural -> the input weight is reused; otherwise the
    density grid, Briggs factors and nearest-cell lookup.
    """
    if imaging_weights_parms['weighting'] == 'natural':
        return np.asarray(weight, dtype=np.float64)
    g = dict(grid_parms)
    dens, sw = grid_weight_density(uvw, weight, freq_chan, g)
    f = calculate_briggs_parms(np.moveaxis(dens, (0, 1), (2, 3)), sw, imaging_weights_parms)
    return standard_imaging_weight_degrid(np.moveaxis(dens, (0, 1), (2, 3)), uvw, weight, f,
                                          freq_chan, np.asarray(g['image_size']), g['cell_size'],
                                          g.get('chan_mode', 'cube'))


# --------------------------------------------------------------------------
# FFT, crop and gridding correction (make_image.py:116-130, make_psf.py:117-131)
# --------------------------------------------------------------------------
def uncorrected_image(grid_cpuv, image_size):
    """fftshift(ifft2(ifftshift(grid))) cropped, real part times Npad^2.

    grid_cpuv is the gridder output (C,P,Nu,Nv); returns (N0,N1,C,P).
    """
    g = np.moveaxis(grid_cpuv, (0, 1), (2, 3))
    img = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(g, axes=(0, 1)), axes=(0, 1)), axes=(0, 1))
    npad = np.array(g.shape[0:2])
    return remove_padding(img, np.asarray(image_size)).real * (npad[0] * npad[1])


def correct_image(uncorrected, sum_weight, correcting_cgk):
    """(image / sum_weight(0->1)) / grdsf (make_image.py:123-128)."""
    sw = np.array(sum_weight, dtype=np.float64, copy=True)
    sw[sw == 0] = 1
    return (uncorrected / sw[None, None, :, :]) / correcting_cgk[:, :, None, None]


def make_image_arrays(vis_data, uvw, imaging_weight, freq_chan, grid_parms, do_psf=False):
    """Dirty image or PSF (N0,N1,C,P) plus sum_weight, as make_image/make_psf.

    Restates make_image.py:105-130 / make_psf.py:104-131 with oversampling
    100, support 7, the PS kernel and its correction image.
    """
    g = dict(grid_parms)
    os_, sup = 100, 7
    npad = np.asarray(g['image_size_padded'])
    corr = remove_padding(create_prolate_spheroidal_correction(npad), g['image_size'])
    cgk = create_prolate_spheroidal_kernel_1D(os_, sup)
    grid, sw = standard_grid(None if do_psf else vis_data, uvw, imaging_weight, freq_chan, cgk,
                             npad, g['cell_size'], sup, os_, do_psf, False, not do_psf,
                             g.get('chan_mode', 'cube'))
    img = uncorrected_image(grid, g['image_size'])
    return correct_image(img, sw, corr), sw


# --------------------------------------------------------------------------
# model visibility prediction (predict_modelvis_image.py:20-39, a stub)
# --------------------------------------------------------------------------
def predict_vis(model, uvw, freq_chan, grid_parms, oversampling=100, support=7):
    """Model visibilities (T,B,C,P) complex128 of a model image (N0,N1,C_img,P).

    The reference only names the steps (predict_modelvis_image.py:36-39:
    flat-sky normalisation, stokes_to_corr, Fourier transform, degrid). This
    restates them with the standard gridder's own geometry run backwards:
    model / grdsf embedded at the centre of the padded grid (the crop of
    make_image.py:119 reversed), forward FFT in ifftshift order (the adjoint
    of make_image.py:116-117's inverse FFT times Npad^2), then per
    visibility the 7x7 footprint of _standard_grid.py:299-357 (same cells,
    oversampling offsets and edge rule) read back and divided by its kernel
    sum. C_img == 1 maps every channel to plane 0 (continuum).
    """
    npad = np.asarray(grid_parms['image_size_padded'])
    size = np.asarray(grid_parms['image_size'])
    C_img, P = model.shape[2], model.shape[3]
    T, B = uvw.shape[:2]
    C = len(freq_chan)
    cgk = create_prolate_spheroidal_kernel_1D(oversampling, support)
    corr = remove_padding(create_prolate_spheroidal_correction(npad), size)
    scale = uv_scale(freq_chan, grid_parms['cell_size'], npad)
    centre = npad // 2
    half = support // 2
    st = npad // 2 - size // 2
    out = np.zeros((T, B, C, P), dtype=np.complex128)
    grids = {}
    for c in range(C):
        ci = 0 if C_img == 1 else c
        u_pos = uvw[:, :, 0] * scale[0, c] + centre[0]
        v_pos = uvw[:, :, 1] * scale[1, c] + centre[1]
        ok = ~np.isnan(u_pos) & ~np.isnan(v_pos)
        u_pos = np.where(ok, u_pos, 0.0)
        v_pos = np.where(ok, v_pos, 0.0)
        cu = np.trunc(u_pos + 0.5).astype(np.int64)
        cv = np.trunc(v_pos + 0.5).astype(np.int64)
        ou = np.floor((cu - u_pos) * oversampling + 0.5).astype(np.int64)
        ov = np.floor((cv - v_pos) * oversampling + 0.5).astype(np.int64)
        ok &= (cu - half >= 0) & (cu + half < npad[0]) & (cv - half >= 0) & (cv + half < npad[1])
        tu = [cgk[np.abs(oversampling * i + ou)] for i in range(-half, half + 1)]
        tv = [cgk[np.abs(oversampling * i + ov)] for i in range(-half, half + 1)]
        norm = sum(tu) * sum(tv)
        for p in range(P):
            if (ci, p) not in grids:
                plane = np.zeros((npad[0], npad[1]))
                plane[st[0]:st[0] + size[0], st[1]:st[1] + size[1]] = model[:, :, ci, p] / corr
                grids[(ci, p)] = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(plane)))
            g = grids[(ci, p)]
            acc = np.zeros((T, B), dtype=np.complex128)
            for a, iu in enumerate(range(-half, half + 1)):
                gu = np.clip(cu + iu, 0, npad[0] - 1)
                for b, iv in enumerate(range(-half, half + 1)):
                    acc += tu[a] * tv[b] * g[gu, np.clip(cv + iv, 0, npad[1] - 1)]
            out[:, :, c, p] = np.where(ok, acc / norm, 0.0)
    return out
