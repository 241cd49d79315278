"""numpy FP64 restatement of the reference's mosaic (aperture-projection) path.

Test infrastructure (see ``oracle/__init__.py``): GCF generation
(make_gridding_convolution_function), the GCF-table gridders
(_aperture_grid.py) and the mosaic normalisation (_normalize.py,
make_mosaic_pb.py, make_image_with_gcf.py). Every function cites the
reference file:line (paths relative to the reference project) it restates.

The gridders build their addends in the reference's loop order (time,
baseline, chan, pol, v-tap, u-tap) and accumulate them with ``np.add.at``,
which adds in index-array order, so each cell receives the same additions in
the same sequence as the reference's scalar loops; tap sums (``norm``) are
sequential (``np.cumsum``), as in the reference.
"""
import numpy as np
from scipy.special import jn

C_LIGHT = 299792458.0


# --------------------------------------------------------------------------
# GCF maps and kernels
# --------------------------------------------------------------------------
def create_cf_baseline_map(unique_ant_indx, baseline_ant, n_unique_ant):
    """ngcasa/imaging/make_gridding_convolution_function.py:522-539: antenna-type
    pairs (i <= j) in row-major order, and each baseline's pair index."""
    n_pairs = int((n_unique_ant ** 2 + n_unique_ant) / 2)
    pairs = np.zeros((n_pairs, 2), dtype=int)
    k = 0
    for i in range(n_unique_ant):
        for j in range(i, n_unique_ant):
            pairs[k] = [i, j]
            k += 1
    uai = np.asarray(unique_ant_indx)
    ba = np.asarray(baseline_ant)
    t = np.stack([uai[ba[:, 0]], uai[ba[:, 1]]], axis=1)
    cf_map = np.zeros(ba.shape[0], dtype=int)
    for k, (i, j) in enumerate(pairs):
        cf_map[(t[:, 0] == i) & (t[:, 1] == j)] = k
    return cf_map, pairs


def create_cf_chan_map(freq_chan, chan_tolerance_factor):
    """make_gridding_convolution_function.py:546-575: one PB frequency per
    fractional bandwidth `chan_tolerance_factor` (at least one), centred in
    equal sub-bands; each channel maps to the nearest PB frequency."""
    freq_chan = np.asarray(freq_chan, dtype=np.float64)
    n_chan = len(freq_chan)
    tol = np.max(freq_chan) * chan_tolerance_factor
    n_pb = int(np.floor((np.max(freq_chan) - np.min(freq_chan)) / tol) + 0.5)
    if n_pb == 0:
        n_pb = 1
    if n_pb >= n_chan:
        return np.arange(n_chan), freq_chan
    dbw = (np.max(freq_chan) - np.min(freq_chan)) / n_pb
    pb_freq = np.arange(n_pb) * dbw + np.min(freq_chan) + dbw / 2
    cf_map = np.array([np.abs(pb_freq - f).argmin() for f in freq_chan], dtype=int)
    return cf_map, pb_freq


def airy_patterns(function, pb_freq, n_pol, dish, blockage, ipower, cell, image_size, image_center):
    """_make_pb_symmetric.py:_airy_disk_rorder / _casa_airy_disk_rorder:
    voltage pattern (type, freq, pol, n0, n1) raised to `ipower`, centre 1."""
    k = (2 * np.pi * np.asarray(pb_freq, dtype=np.float64)) / C_LIGHT
    c = np.asarray(image_center)
    n = np.asarray(image_size)
    x = np.arange(-c[0], n[0] - c[0]) * cell[0]
    y = np.arange(-c[1], n[1] - c[1]) * cell[1]
    out = np.zeros((len(blockage), len(k), 1, n[0], n[1]))
    for i, (dd, bd) in enumerate(zip(dish, blockage)):
        aperture = dd / 2
        xg, yg = np.meshgrid(x, y, indexing='ij')
        r = np.moveaxis(np.sqrt(xg ** 2 + yg ** 2)[:, :, None] * k * aperture, 2, 0)
        r[:, c[0], c[1]] = 1.0
        if bd == 0.0:
            out[i, :, 0] = (2.0 * jn(1, r) / r) ** ipower
        elif function == 'casa_airy':
            ar = (dd / bd) ** 2
            lr = dd / bd
            out[i, :, 0] = ((ar * 2.0 * jn(1, r) / r - 2.0 * jn(1, r * lr) / (r * lr)) / (ar - 1.0)) ** ipower
        else:
            e = bd / dd
            out[i, :, 0] = ((2.0 * jn(1, r) / r - 2.0 * e * jn(1, r * e) / r) / (1.0 - e ** 2)) ** ipower
    out[:, :, 0, c[0], c[1]] = 1.0
    return np.tile(out, (1, 1, n_pol, 1, 1))


def baseline_patterns(function, pb_freq, pairs, dish, blockage, ipower, grid_parms, oversampling):
    """make_gridding_convolution_function.py:393-410: patterns on the padded
    grid with cell = cell_size * oversampling, product over each pair."""
    npad = np.asarray(grid_parms['image_size_padded'])
    cell = np.asarray(grid_parms['cell_size']) * np.asarray(oversampling)
    pat = airy_patterns(function, pb_freq, 1, dish, blockage, ipower, cell, npad, npad // 2)
    out = np.zeros((len(pairs), len(pb_freq), 1, npad[0], npad[1]))
    for q, (a0, a1) in enumerate(pairs):
        for f in range(len(pb_freq)):
            out[q, f, 0] = pat[a0, f, 0] * pat[a1, f, 0]
    return out


def pattern_to_kernel(bp):
    """make_gridding_convolution_function.py:273-274: real(fftshift(fft2(ifftshift)))."""
    return np.real(np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(bp, axes=(3, 4)), axes=(3, 4)), axes=(3, 4)))


def calc_conv_size(sub_a_term, imsize, support_cut_level, oversampling, max_support):
    """make_gridding_convolution_function.py:412-459: walk +x and +y from the
    centre until the kernel drops to support_cut_level * max|kernel|; the
    odd support is (int(0.5 + walk/os) + 1) * 2 + 1, the larger of the two."""
    a = np.abs(sub_a_term)
    cut = support_cut_level * a.max()
    if not a.min() < cut:
        raise ValueError('support_cut_level too small or imsize too small')
    cx, cy = imsize[0] // 2, imsize[1] // 2
    ix = cx
    while sub_a_term[ix, cy] > cut:
        ix += 1
        if not ix < imsize[0]:
            raise ValueError('support_cut_level too small or imsize too small')
    sx = (int(0.5 + (ix - cx) / oversampling[0]) + 1) * 2 + 1
    iy = cy
    while sub_a_term[cx, iy] > cut:
        iy += 1
        if not iy < imsize[1]:
            raise ValueError('support_cut_level too small or imsize too small')
    sy = (int(0.5 + (iy - cy) / oversampling[1]) + 1) * 2 + 1
    if not (sx < max_support[0] and sy < max_support[1]):
        raise ValueError('support_cut_level too small or imsize too small')
    s = max(sx, sy)
    return [s, s]


def resize_and_calc_support(conv_kernel, weight_kernel, oversampling, max_support, support_cut_level, npad):
    """make_gridding_convolution_function.py:360-390: support from the weight
    kernel; both kernels cropped to (max_support + 1) * os around the centre
    and divided by their sum over the (support + 1) * os window / (os0 * os1)."""
    os_ = np.asarray(oversampling)
    rs = (np.asarray(max_support) + 1) * os_
    shp = conv_kernel.shape[:3]
    sup = np.zeros(shp + (2,), dtype=int)
    st = np.asarray(npad) // 2 - rs // 2
    ck = np.zeros(shp + tuple(rs))
    wk = np.zeros(shp + tuple(rs))
    for idx in np.ndindex(*shp):
        sup[idx] = calc_conv_size(weight_kernel[idx], npad, support_cut_level, os_, max_support)
        es = (sup[idx] + 1) * os_
        e0 = rs // 2 - es // 2
        for src, dst in ((conv_kernel, ck), (weight_kernel, wk)):
            dst[idx] = src[idx][st[0]:st[0] + rs[0], st[1]:st[1] + rs[1]]
            nf = np.real(np.sum(dst[idx][e0[0]:e0[0] + es[0], e0[1]:e0[1] + es[1]]) / (os_[0] * os_[1]))
            dst[idx] = dst[idx] / nf
    return ck, wk, sup


def sin_pixel_offsets(field_phase_dir, phase_center, cell_rad):
    """Pixel offsets of the field centres from the phase centre in the SIN
    (orthographic) projection with pixel size cell_rad, the quantity
    make_phase_gradient obtains from a RA---SIN/DEC--SIN WCS
    (make_gridding_convolution_function.py:331-347):
    l = cos(d) sin(a - a0), m = sin(d) cos(d0) - cos(d) sin(d0) cos(a - a0),
    pixel offset = degrees(l, m) / degrees(cell)."""
    a0, d0 = phase_center
    fpd = np.asarray(field_phase_dir, dtype=np.float64).reshape(-1, 2)
    a, d = fpd[:, 0], fpd[:, 1]
    l = np.cos(d) * np.sin(a - a0)
    m = np.sin(d) * np.cos(d0) - np.cos(d) * np.sin(d0) * np.cos(a - a0)
    cdelt = np.asarray(cell_rad) * (180 / np.pi)
    return np.stack([np.rad2deg(l) / cdelt[0], np.rad2deg(m) / cdelt[1]], axis=1)


def phase_slopes(field_phase_dir, phase_center, npad, cell_rad, oversampling):
    """make_gridding_convolution_function.py:348: -pix * 2 pi / (npad * os)."""
    pix = sin_pixel_offsets(field_phase_dir, phase_center, cell_rad)
    return -pix * 2 * np.pi / (np.asarray(npad) * np.asarray(oversampling))


def phase_gradient(slopes, conv_size):
    """make_gridding_convolution_function.py:350-359: exp(i (x px + y py)) on
    the table offsets from its centre, (n_field, R0, R1)."""
    cs = np.asarray(conv_size)
    c = cs // 2
    x = np.arange(-c[0], cs[0] - c[0])
    y = np.arange(-c[1], cs[1] - c[1])
    xg, yg = np.meshgrid(x, y, indexing='ij')
    return np.moveaxis(np.exp(1j * (xg[:, :, None] * slopes[:, 0] + yg[:, :, None] * slopes[:, 1])), 2, 0)


# --------------------------------------------------------------------------
# GCF-table gridders
# --------------------------------------------------------------------------
def _prep(uvw, freq_chan, n_uv, delta_lm):
    n_uv = np.asarray(n_uv)
    scale = np.zeros((2, len(freq_chan)))
    scale[0] = -(freq_chan * delta_lm[0] * n_uv[0]) / C_LIGHT
    scale[1] = -(freq_chan * delta_lm[1] * n_uv[1]) / C_LIGHT
    return n_uv, scale, n_uv // 2


def _cmul(a, b):
    """a * b with the scalar formula (re = ar br - ai bi, im = ar bi + ai br),
    each product and sum rounded separately, as numpy's scalar complex
    multiply evaluates it (array loops may fuse into FMAs)."""
    b = complex(b)
    out = np.empty(a.shape, dtype=np.complex128)
    out.real = a.real * b.real - a.imag * b.imag
    out.imag = a.real * b.imag + a.imag * b.real
    return out


def aperture_grid(vis_data, uvw, imaging_weight, field, field_id, cf_baseline_map, cf_chan_map, cf_pol_map,
                  conv_kernel, support, phase_grad, freq_chan, n_uv, delta_lm, oversampling, chan_mode='cube',
                  do_psf=False, weight_grid=False):
    """_aperture_grid.py:376-513 (_aperture_grid_jit), and with weight_grid
    :180-291 (_aperture_weight_grid_jit: taps at the grid centre, zero
    offsets, sum_weight += w Re(norm)). Grid complex128 (Cimg, P, Nu, Nv)."""
    T, B, C, P = imaging_weight.shape
    n_uv, scale, uvc = _prep(uvw, np.asarray(freq_chan, dtype=np.float64), n_uv, delta_lm)
    chan_map = np.zeros(C, dtype=int) if chan_mode == 'continuum' else np.arange(C)
    n_img = 1 if chan_mode == 'continuum' else C
    grid = np.zeros((n_img, P, n_uv[0], n_uv[1]), dtype=np.complex128)
    sw = np.zeros((n_img, P))
    maxs = np.max(support)
    R0, R1 = conv_kernel.shape[-2:]
    cc0, cc1 = R0 // 2, R1 // 2
    os0, os1 = oversampling
    idx_l, val_l = [], []
    prev = -1
    ckpg = None
    field_id = np.asarray(field_id)
    for t in range(T):
        for b in range(B):
            if field[t, b] <= -1:
                continue
            fi = np.where(field_id == field[t, b])[0][0]
            if fi != prev:
                ckpg = conv_kernel * phase_grad[fi]
                prev = fi
            cfb = cf_baseline_map[b]
            for c in range(C):
                u = uvw[t, b, 0] * scale[0, c]
                v = uvw[t, b, 1] * scale[1, c]
                if np.isnan(u) or np.isnan(v):
                    continue
                up, vp = u + uvc[0], v + uvc[1]
                cu, cv = int(up + 0.5), int(vp + 0.5)
                if not (cu + maxs < n_uv[0] and cv + maxs < n_uv[1] and cu - maxs >= 0 and cv - maxs >= 0):
                    continue
                if weight_grid:
                    ou, ov = cc0, cc1
                    gu, gv = uvc[0], uvc[1]
                else:
                    ou = int(np.floor((cu - up) * os0 + 0.5)) + cc0
                    ov = int(np.floor((cv - vp) * os1 + 0.5)) + cc1
                    gu, gv = cu, cv
                cfc = cf_chan_map[c]
                for p in range(P):
                    w = imaging_weight[t, b, c, p]
                    wd = w if (do_psf or weight_grid) else vis_data[t, b, c, p] * w
                    if np.isnan(wd) or wd == 0.0:
                        continue
                    cfp = cf_pol_map[p]
                    su, sv = support[cfb, cfc, cfp]
                    iv = np.arange(-(sv // 2), sv - sv // 2)
                    iu = np.arange(-(su // 2), su - su // 2)
                    ivg, iug = np.meshgrid(iv, iu, indexing='ij')          # v outer, u inner
                    conv = ckpg[cfb, cfc, cfp, os0 * iug + ou, os1 * ivg + ov].ravel()
                    cells = (((chan_map[c] * P + p) * n_uv[0] + gu + iug) * n_uv[1] + gv + ivg).ravel()
                    idx_l.append(cells)
                    val_l.append(_cmul(conv, wd))
                    norm = np.cumsum(conv)[-1]
                    if do_psf or weight_grid:
                        sw[chan_map[c], p] = sw[chan_map[c], p] + w * np.real(norm)
                    else:
                        sw[chan_map[c], p] = sw[chan_map[c], p] + w * np.real(norm ** 2)
    if idx_l:
        np.add.at(grid.reshape(-1), np.concatenate(idx_l), np.concatenate(val_l))
    return grid, sw


# --------------------------------------------------------------------------
# mosaic images
# --------------------------------------------------------------------------
def _remove_padding(image, image_size):
    n = np.asarray(image.shape[:2])
    s = n // 2 - np.asarray(image_size) // 2
    return image[s[0]:s[0] + image_size[0], s[1]:s[1] + image_size[1]]


def grid_to_image(grid, image_size):
    """make_mosaic_pb.py:140 / make_image_with_gcf.py:157-160: (u, v, C, P)
    grid -> real(fftshift(ifft2(ifftshift))) cropped, times Nu*Nv."""
    g = np.moveaxis(grid, (0, 1), (2, 3))
    n = g.shape[0] * g.shape[1]
    im = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(g, axes=(0, 1)), axes=(0, 1)), axes=(0, 1))
    return _remove_padding(im, image_size).real * n


def mosaic_pb(weight_grid, sum_weight, image_size):
    """make_mosaic_pb.py:140-150: WEIGHT_PB = image / sum_weight (0 -> 1),
    PB = sqrt(|WEIGHT_PB|). Returns (pb, weight_pb), (l, m, C, P)."""
    wi = grid_to_image(weight_grid, image_size)
    s = sum_weight.copy()
    s[s == 0] = 1
    wi = wi / s[None, None]
    return np.sqrt(np.abs(wi)), wi


def normalize(image, sum_weight, pb, weight_pb, ps_corr_image, oversampling, norm_type='flat_sky', pb_limit=0.2,
              single_precision=True):
    """_normalize.py:14-90 (direction 'forward'): image / sum_weight (0 -> 1)
    / (sinc oversampling correction * normalising image), zero where
    PB < pb_limit, optionally rounded through float32."""
    s = sum_weight.copy()
    s[s == 0] = 1
    if norm_type == 'flat_noise':
        nimg = ps_corr_image[:, :, None, None] * pb
    elif norm_type == 'flat_sky':
        nimg = ps_corr_image[:, :, None, None] * weight_pb
    else:
        nimg = ps_corr_image[:, :, None, None]
    n = np.asarray(image.shape[:2])
    c = n // 2
    sx = np.sinc(np.arange(-c[0], n[0] - c[0]) / (n[0] * oversampling[0]))
    sy = np.sinc(np.arange(-c[1], n[1] - c[1]) / (n[1] * oversampling[1]))
    osc = np.dot(sx[:, None], sy[None, :])
    out = (image / s[None, None]) / (osc[:, :, None, None] * nimg)
    if pb_limit > 0:
        out[pb < pb_limit] = 0.0
    if single_precision:
        out = out.astype(np.float32).astype(np.float64)
    return out
