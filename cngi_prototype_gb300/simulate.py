"""Seeded synthetic interferometer observations.

No public dataset is available offline, so the imaging configurations are
driven by synthetic visibilities with the shapes, layouts and value
distributions of the workloads they stand in for:

* antenna layouts in a local ENU frame (uniform disk or 3-arm log spiral);
* Earth-rotation synthesis uvw: ENU -> local equatorial XYZ at latitude
  ``lat`` (X = -sin(lat) N + cos(lat) U, Y = E, Z = cos(lat) N + sin(lat) U),
  hour angle H = omega_E (t - t_mid), and the standard rotation to (u, v, w)
  for declination ``dec``;
* point-source skies, V(u,v) = sum_k S_k exp(-2 pi i (u l_k + v m_k) f/c)
  (w ignored, as the gridder ignores it), plus complex Gaussian noise.

Arrays use the visibility layout of the reference's vis datasets:
DATA/WEIGHT/FLAG are (time, baseline, chan, pol) and UVW is
(time, baseline, 3) in metres.
"""
import numpy as np

C_LIGHT = 299792458.0
OMEGA_EARTH = 7.2921e-5  # rad/s


def disk_layout(n_ant, radius_m, rng):
    """n_ant antennas uniform in a disk of the given radius (ENU metres)."""
    r = radius_m * np.sqrt(rng.random(n_ant))
    th = 2 * np.pi * rng.random(n_ant)
    return np.stack([r * np.cos(th), r * np.sin(th), np.zeros(n_ant)], axis=1)


def log_spiral_layout(n_ant, radius_m, rng, n_arms=3, r_min=20.0, turns=0.6):
    """3-arm logarithmic spiral reaching ``radius_m``; small radial jitter."""
    per_arm = int(np.ceil(n_ant / n_arms))
    pos = []
    for a in range(n_arms):
        k = np.arange(per_arm)
        r = r_min * (radius_m / r_min) ** (k / max(per_arm - 1, 1))
        th = 2 * np.pi * a / n_arms + 2 * np.pi * turns * np.log(r / r_min) / np.log(radius_m / r_min)
        r = r * (1 + 0.02 * rng.standard_normal(per_arm))
        pos.append(np.stack([r * np.cos(th), r * np.sin(th), np.zeros(per_arm)], axis=1))
    return np.concatenate(pos)[:n_ant]


def baseline_pairs(n_ant):
    a1, a2 = np.triu_indices(n_ant, k=1)
    return a1.astype(np.int32), a2.astype(np.int32)


def earth_rotation_uvw(enu, n_time, dt_s, lat_deg=34.0, dec_deg=45.0):
    """uvw (T, B, 3) float64 in metres for all antenna pairs i<j."""
    lat = np.deg2rad(lat_deg)
    dec = np.deg2rad(dec_deg)
    e, n, u = enu[:, 0], enu[:, 1], enu[:, 2]
    X = -np.sin(lat) * n + np.cos(lat) * u
    Y = e
    Z = np.cos(lat) * n + np.sin(lat) * u
    a1, a2 = baseline_pairs(len(enu))
    bx, by, bz = X[a2] - X[a1], Y[a2] - Y[a1], Z[a2] - Z[a1]
    t = (np.arange(n_time) - (n_time - 1) / 2.0) * dt_s
    H = OMEGA_EARTH * t
    sH, cH = np.sin(H)[:, None], np.cos(H)[:, None]
    uu = sH * bx + cH * by
    vv = -np.sin(dec) * cH * bx + np.sin(dec) * sH * by + np.cos(dec) * bz
    ww = np.cos(dec) * cH * bx - np.cos(dec) * sH * by + np.sin(dec) * bz
    return np.stack([uu, vv, ww], axis=-1).astype(np.float64)


def pixel_to_lm(px, py, image_size, cell_rad):
    """Direction cosines of image pixel (px, py) for this gridder's geometry.

    With the cell_size[0] sign flip, a source at (l, m) = ((px - N0/2) c0,
    -(py - N1/2) c1) peaks at pixel (px, py) of the dirty image.
    """
    l = (np.asarray(px) - image_size[0] // 2) * cell_rad[0]
    m = -(np.asarray(py) - image_size[1] // 2) * cell_rad[1]
    return l, m


def point_source_vis(uvw, freq, l, m, flux, n_pol=2, noise_sigma=0.0, rng=None,
                     device=None, dtype=np.complex64):
    """Visibilities (T,B,C,P) of point sources; optional complex noise.

    Runs in numpy, or with torch on ``device`` for large cubes (generation is
    input preparation, not part of any timed region).
    """
    T, B = uvw.shape[:2]
    C = len(freq)
    if device is None:
        out = np.zeros((T, B, C), dtype=np.complex128)
        for c in range(C):
            k = 2 * np.pi * freq[c] / C_LIGHT
            acc = np.zeros((T, B), dtype=np.complex128)
            for s in range(len(flux)):
                ph = -k * (uvw[..., 0] * l[s] + uvw[..., 1] * m[s])
                acc += flux[s] * np.exp(1j * ph)
            out[..., c] = acc
        vis = np.repeat(out[..., None], n_pol, axis=-1).astype(dtype)
        if noise_sigma > 0:
            rng = rng or np.random.default_rng(0)
            vis = vis + (noise_sigma * (rng.standard_normal(vis.shape) + 1j * rng.standard_normal(vis.shape))).astype(dtype)
        return vis
    import torch
    dev = torch.device(device)
    u = torch.as_tensor(uvw[..., 0], device=dev, dtype=torch.float64)
    v = torch.as_tensor(uvw[..., 1], device=dev, dtype=torch.float64)
    lt = torch.as_tensor(np.asarray(l), device=dev, dtype=torch.float64)
    mt = torch.as_tensor(np.asarray(m), device=dev, dtype=torch.float64)
    st = torch.as_tensor(np.asarray(flux), device=dev, dtype=torch.float64)
    vis = torch.empty((T, B, C, n_pol), dtype=torch.complex64, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(rng.integers(1 << 31)) if rng is not None else 0)
    for c in range(C):
        k = 2 * np.pi * float(freq[c]) / C_LIGHT
        re = torch.zeros((T, B), dtype=torch.float64, device=dev)
        im = torch.zeros((T, B), dtype=torch.float64, device=dev)
        for s0 in range(0, len(flux), 16):
            ph = -k * (u[..., None] * lt[s0:s0 + 16] + v[..., None] * mt[s0:s0 + 16])
            re += (st[s0:s0 + 16] * torch.cos(ph)).sum(-1)
            im += (st[s0:s0 + 16] * torch.sin(ph)).sum(-1)
        base = torch.complex(re.float(), im.float())
        for p in range(n_pol):
            vc = base
            if noise_sigma > 0:
                nr = torch.randn((T, B), generator=gen, device=dev) * noise_sigma
                ni = torch.randn((T, B), generator=gen, device=dev) * noise_sigma
                vc = vc + torch.complex(nr, ni)
            vis[:, :, c, p] = vc
    return vis


def point_source_vis_torch(uvw, freq, l, m, flux, n_pol, noise_sigma, seed, device='cuda'):
    """Large-cube generator on the GPU: (T,B,C,P) complex64 torch tensor.

    The phase 2 pi f (u l + v m)/c is formed and range-reduced in FP64 per
    (row, source, channel) and evaluated with FP32 sin/cos; noise is drawn
    per pol with a seeded torch generator.
    """
    import torch
    dev = torch.device(device)
    T, B = uvw.shape[:2]
    C = len(freq)
    u = torch.as_tensor(uvw[..., 0].reshape(-1), device=dev, dtype=torch.float64)
    v = torch.as_tensor(uvw[..., 1].reshape(-1), device=dev, dtype=torch.float64)
    lt = torch.as_tensor(np.asarray(l), device=dev, dtype=torch.float64)
    mt = torch.as_tensor(np.asarray(m), device=dev, dtype=torch.float64)
    st = torch.as_tensor(np.asarray(flux), device=dev, dtype=torch.float32)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    vis = torch.empty((T * B, C, n_pol), dtype=torch.complex64, device=dev)
    two_pi = 2.0 * np.pi
    n_src = len(flux)
    rows_per = max(1, (1 << 27) // max(n_src, 1))
    for r0 in range(0, T * B, rows_per):
        r1 = min(T * B, r0 + rows_per)
        base = -(u[r0:r1, None] * lt[None, :] + v[r0:r1, None] * mt[None, :]) / C_LIGHT   # turns per Hz
        for c in range(C):
            turns = base * float(freq[c])
            turns = turns - torch.round(turns)
            ph = (turns * two_pi).float()
            re = (torch.cos(ph) * st).sum(-1)
            im = (torch.sin(ph) * st).sum(-1)
            for p in range(n_pol):
                vr = re
                vi = im
                if noise_sigma > 0:
                    vr = vr + noise_sigma * torch.randn(r1 - r0, generator=gen, device=dev)
                    vi = vi + noise_sigma * torch.randn(r1 - r0, generator=gen, device=dev)
                vis[r0:r1, c, p] = torch.complex(vr, vi)
    return vis.view(T, B, C, n_pol)


class Observation(dict):
    """Plain container for a synthetic observation (arrays + imaging parms)."""
    __getattr__ = dict.__getitem__


def make_observation(n_ant, layout, radius_m, n_time, dt_s, freq, n_pol, n_src,
                     flux_range, src_radius_rad, noise_sigma, image_size, cell_arcsec,
                     seed, flag_fraction=0.0, flux_law='uniform', vis_device=None,
                     with_vis=True):
    rng = np.random.default_rng(seed)
    enu = disk_layout(n_ant, radius_m, rng) if layout == 'disk' else log_spiral_layout(n_ant, radius_m, rng)
    uvw = earth_rotation_uvw(enu, n_time, dt_s)
    T, B = uvw.shape[:2]
    C = len(freq)
    if flux_law == 'uniform':
        flux = rng.uniform(flux_range[0], flux_range[1], n_src)
    else:  # N(>S) ~ S^-1.5 between the bounds, inverse-CDF sampling
        a, b = flux_range
        x = rng.random(n_src)
        flux = (a ** -1.5 - x * (a ** -1.5 - b ** -1.5)) ** (-1 / 1.5)
    r = src_radius_rad * np.sqrt(rng.random(n_src))
    th = 2 * np.pi * rng.random(n_src)
    l, m = r * np.cos(th), r * np.sin(th)
    obs = Observation(uvw=uvw, freq=np.asarray(freq, dtype=np.float64), l=l, m=m, flux=flux,
                      enu=enu, image_size=list(image_size), cell_arcsec=list(cell_arcsec))
    weight = None
    flag = None
    if vis_device is None:
        weight = np.ones((T, B, C, n_pol), dtype=np.float32)
        if flag_fraction > 0:
            flag = rng.random((T, B, C, n_pol)) < flag_fraction
    obs['weight'] = weight
    obs['flag'] = flag
    if with_vis and vis_device is None:
        vis = point_source_vis(uvw, obs['freq'], l, m, flux, n_pol, noise_sigma, rng)
        if flag is not None:
            vis[flag] = np.nan
            weight[flag] = np.nan
        obs['vis'] = vis
    elif with_vis:
        import torch
        vis = point_source_vis_torch(uvw, obs['freq'], l, m, flux, n_pol, noise_sigma, seed + 1000, vis_device)
        w = torch.ones((T, B, C, n_pol), dtype=torch.float32, device=vis_device)
        if flag_fraction > 0:
            gen = torch.Generator(device=vis_device)
            gen.manual_seed(seed + 2000)
            fl = torch.rand((T, B, C, n_pol), generator=gen, device=vis_device) < flag_fraction
            vis[fl] = complex('nan')
            w[fl] = float('nan')
            del fl
        obs['vis'] = vis
        obs['weight'] = w
    return obs


def config_standard_small(seed=1, n_time=600, n_chan=32):
    """Plain standard gridding workload: 27 antennas in a 1 km-radius disk,
    600 x 10 s integrations, 32 channels 1.000-1.128 GHz (4 MHz), RR/LL,
    20 sources, 512^2 image at 2 arcsec, natural weighting."""
    freq = 1.000e9 + (np.arange(n_chan) + 0.5) * 4e6
    return make_observation(27, 'disk', 1000.0, n_time, 10.0, freq, 2, 20, (0.1, 1.0),
                            np.deg2rad(0.5), 0.1, (512, 512), (2.0, 2.0), seed)


def config_large_cube(seed=2, n_time=1024, n_chan=256, vis_device=None, with_vis=True, chan_range=None,
                      image_size=4096):
    """Large cube: 64 antennas, 3-arm log spiral of 2.5 km radius, 1024 x 8 s,
    256 channels over 1.0-1.5 GHz, RR/LL, 200 power-law sources
    (1 mJy-1 Jy), 5% random flags, Briggs 0.5, 4096^2 image at 1 arcsec.
    chan_range=(c0, c1) keeps channels c0..c1-1 of the n_chan (one rank's
    shard of a channel-partitioned cube; same sky and rows). image_size N
    images the same field with N^2 pixels of 4096/N arcsec."""
    freq = 1.0e9 + (np.arange(n_chan) + 0.5) * (0.5e9 / n_chan)
    if chan_range is not None:
        freq = freq[chan_range[0]:chan_range[1]]
    fov = 4096 * np.deg2rad(1.0 / 3600) / 2
    cell = 4096.0 / image_size
    return make_observation(64, 'log_spiral', 2500.0, n_time, 8.0, freq, 2, 200, (1e-3, 1.0),
                            fov, 0.05, (image_size, image_size), (cell, cell), seed, flag_fraction=0.05,
                            flux_law='power', vis_device=vis_device, with_vis=with_vis)


# ---------------------------------------------------------------------------
# mosaic observations
# ---------------------------------------------------------------------------
def sin_to_radec(l, m, phase_center):
    """Inverse SIN (orthographic) projection: direction cosines (l, m) about
    phase_center (ra0, dec0) -> (ra, dec) in radians."""
    a0, d0 = phase_center
    n = np.sqrt(1.0 - l ** 2 - m ** 2)
    dec = np.arcsin(m * np.cos(d0) + n * np.sin(d0))
    ra = a0 + np.arctan2(l, n * np.cos(d0) - m * np.sin(d0))
    return ra, dec


def hex_offsets(n, spacing):
    """n points of a hexagonal grid of the given spacing, nearest the origin first."""
    k = int(np.ceil(np.sqrt(n))) + 2
    pts = []
    for j in range(-k, k + 1):
        for i in range(-k, k + 1):
            pts.append(((i + 0.5 * (j % 2)) * spacing, j * spacing * np.sqrt(3) / 2))
    pts = np.array(pts)
    pts = pts - pts[np.argmin(np.hypot(pts[:, 0], pts[:, 1]))]
    order = np.lexsort((np.arctan2(pts[:, 1], pts[:, 0]), np.round(np.hypot(pts[:, 0], pts[:, 1]) / spacing, 6)))
    return pts[order[:n]]


def casa_airy_voltage(r, freq, dish, blockage):
    """CASA obscured-aperture Airy voltage pattern at angle r (radians)."""
    from scipy.special import j1
    x = np.asarray(r) * (2 * np.pi * freq / C_LIGHT) * dish / 2
    x = np.where(x == 0, 1e-30, x)
    if blockage == 0:
        return 2 * j1(x) / x
    A, L = (dish / blockage) ** 2, dish / blockage
    return (A * 2 * j1(x) / x - 2 * j1(x * L) / (x * L)) / (A - 1.0)


def config_mosaic(seed=4, n_chan=16, n_int=30, n_pointing=49, n_comp=300, n_pol=2, vis_device='cuda',
                  n_ant=50, radius_m=750.0, dt_s=6.0):
    """Mosaic aperture-projection workload: 50 x 12 m antennas (0.75 m
    blockage, CASA Airy) uniform in a 750 m-radius disk (1225 baselines),
    49 pointings on a hexagonal grid at half-beam spacing (FWHM 1.02 lambda/D
    at 100.8 GHz), 30 integrations of 6 s per pointing (1470 times), 16
    channels over 100-101.6 GHz, RR/LL, a sky of 300 Gaussian components
    (flux U[0.05, 1] Jy, FWHM U[0.2, 2] arcsec) spread over the mosaic, noise
    sigma 0.05 Jy. 2048^2 image at 0.2 arcsec, GCF oversampling 20, max
    support 31.

    Each visibility is V = sum_k S_k P_f(k) exp(-2 pi^2 s_k^2 |uv|^2)
    exp(+2 pi i (u l_k + v m_k)): the sign puts a component at direction
    (l, m) at the image pixel the reference's SIN WCS gives that direction,
    pixel offset (l / cell0, m / cell1) with cell0 < 0 -- the pixel where
    make_mosaic_pb places a pointing in that direction. P_f = the baseline's
    primary beam (voltage pattern squared) of the row's pointing f at the
    component. Data are in the common phase-centre frame (as after
    direction_rotate). Returns an Observation; vis / weight are CUDA tensors
    when vis_device is set.
    """
    rng = np.random.default_rng(seed)
    dish, block = 12.0, 0.75
    enu = disk_layout(n_ant, radius_m, rng)
    T = n_int * n_pointing
    uvw = earth_rotation_uvw(enu, T, dt_s)
    B = uvw.shape[1]
    a1, a2 = baseline_pairs(n_ant)
    freq = 100.0e9 + (np.arange(n_chan) + 0.5) * (1.6e9 / n_chan)
    fwhm = 1.02 * (C_LIGHT / 100.8e9) / dish
    pc = np.array([np.deg2rad(150.0), np.deg2rad(45.0)])
    off = hex_offsets(n_pointing, fwhm / 2)                        # (l, m) of each pointing
    ra, dec = sin_to_radec(off[:, 0], off[:, 1], pc)
    field_phase_dir = np.stack([ra, dec], axis=1)
    extent = np.abs(off).max(axis=0) + fwhm / 2
    cl = rng.uniform(-extent[0], extent[0], n_comp)
    cm = rng.uniform(-extent[1], extent[1], n_comp)
    flux = rng.uniform(0.05, 1.0, n_comp)
    sig = np.deg2rad(rng.uniform(0.2, 2.0, n_comp) / 3600) / (2 * np.sqrt(2 * np.log(2)))
    field = np.repeat(np.arange(n_pointing), n_int)[:, None].repeat(B, axis=1).astype(np.int32)
    # primary-beam gain of every (pointing, component, channel)
    dist = np.hypot(cl[None, :] - off[:, 0:1], cm[None, :] - off[:, 1:2])
    pbg = np.stack([casa_airy_voltage(dist, f, dish, block) ** 2 for f in freq], axis=-1)   # (F, K, C)
    obs = Observation(uvw=uvw, freq=freq, field=field, field_phase_dir=field_phase_dir, phase_center=pc,
                      antenna1=a1, antenna2=a2, pointing_lm=off, comp_lm=np.stack([cl, cm], 1), comp_flux=flux,
                      comp_sigma=sig, image_size=[2048, 2048], cell_arcsec=[0.2, 0.2], dish=dish, blockage=block,
                      oversampling=[20, 20], max_support=[31, 31])
    if vis_device is None:
        return obs
    import torch
    dev = torch.device(vis_device)
    u = torch.as_tensor(uvw[..., 0].reshape(-1), device=dev, dtype=torch.float64)
    v = torch.as_tensor(uvw[..., 1].reshape(-1), device=dev, dtype=torch.float64)
    fr = torch.as_tensor(field.reshape(-1), device=dev, dtype=torch.int64)
    lt = torch.as_tensor(cl, device=dev, dtype=torch.float64)
    mt = torch.as_tensor(cm, device=dev, dtype=torch.float64)
    s2 = torch.as_tensor(2 * np.pi ** 2 * sig ** 2, device=dev, dtype=torch.float64)
    amp = torch.as_tensor(flux[None, :, None] * pbg, device=dev, dtype=torch.float32)      # (F, K, C)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed) + 4000)
    vis = torch.empty((T * B, n_chan, n_pol), dtype=torch.complex64, device=dev)
    rows_per = max(1, (1 << 26) // n_comp)
    for r0 in range(0, T * B, rows_per):
        r1 = min(T * B, r0 + rows_per)
        base = (u[r0:r1, None] * lt[None, :] + v[r0:r1, None] * mt[None, :]) / C_LIGHT      # turns per Hz
        q2 = (u[r0:r1] ** 2 + v[r0:r1] ** 2) / C_LIGHT ** 2                                  # (uv / lambda)^2 per Hz^2
        for c in range(n_chan):
            a = amp[:, :, c][fr[r0:r1]]                                                       # (rows, K)
            f = float(freq[c])
            turns = base * f
            turns = turns - torch.round(turns)
            ph = (turns * (2 * np.pi)).float()
            g = torch.exp(-(q2[:, None] * f * f) * s2[None, :]).float() * a
            re = (torch.cos(ph) * g).sum(-1)
            im = (torch.sin(ph) * g).sum(-1)
            for p in range(n_pol):
                nr = 0.05 * torch.randn(r1 - r0, generator=gen, device=dev)
                ni = 0.05 * torch.randn(r1 - r0, generator=gen, device=dev)
                vis[r0:r1, c, p] = torch.complex(re + nr, im + ni)
    obs['vis'] = vis.view(T, B, n_chan, n_pol)
    obs['weight'] = torch.ones((T, B, n_chan, n_pol), dtype=torch.float32, device=dev)
    return obs
