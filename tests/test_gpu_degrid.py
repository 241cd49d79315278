"""The degridder is the exact adjoint of the imaging operator, and the
autograd pair's backward matches finite differences and the residual image."""
import numpy as np
import pytest

from oracle import imaging as O

pytestmark = pytest.mark.gpu


def _obs(seed=21, n_ant=10, T=40, C=2, P=1, N=64, cell=25.0):
    from cngi_prototype_gb300 import simulate
    rng = np.random.default_rng(seed)
    enu = simulate.disk_layout(n_ant, 400.0, rng)
    uvw = simulate.earth_rotation_uvw(enu, T, 120.0)
    B = uvw.shape[1]
    freq = 1.0e9 + np.arange(C) * 5e7
    w = rng.uniform(0.5, 2.0, (T, B, C, P)).astype(np.float32)
    gp = {'image_size': [N, N], 'cell_size': [cell, cell]}
    O.check_grid_parms(gp)
    return uvw, w, freq, gp, rng


def _op(uvw, w, freq, gp):
    from cngi_prototype_gb300.imaging.degrid import ImagingOperator
    return ImagingOperator(uvw, w, freq, gp)


def test_adjoint_identity(ngg):
    import torch
    uvw, w, freq, gp, rng = _obs()
    op = _op(uvw, w, freq, gp)
    T, B, C, P = w.shape
    N = gp['image_size'][0]
    for _ in range(3):
        x = torch.as_tensor(rng.standard_normal((N, N, C, P)), device='cuda')
        y = torch.as_tensor((rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P)))
                            .astype(np.complex64), device='cuda')
        ax = op.degrid(x).to(torch.complex128)
        dy = op.image(y)
        lhs = float(torch.sum(torch.conj(ax) * y.to(torch.complex128)).real)
        rhs = float(torch.sum(x * dy))
        # the inner products cancel (random signs), so the FP32 error is measured
        # against the norms that bound them (Cauchy-Schwarz), not their values
        scale = float(torch.linalg.vector_norm(ax) * torch.linalg.vector_norm(y.to(torch.complex128)) +
                      torch.linalg.vector_norm(x) * torch.linalg.vector_norm(dy))
        assert abs(lhs - rhs) <= 1e-6 * scale, (lhs, rhs, scale)


def _numpy_degrid(x, uvw, w, freq, gp, sw, corr):
    """FP64 D^T: scale, embed, forward FFT in ifftshift order, 49-tap gather."""
    npad = np.asarray(gp['image_size_padded'])
    N = np.asarray(gp['image_size'])
    C, P = x.shape[2], x.shape[3]
    T, B = uvw.shape[:2]
    cgk = O.create_prolate_spheroidal_kernel_1D(100, 7)
    out = np.zeros((T, B, C, P), dtype=np.complex128)
    s = O.uv_scale(freq, gp['cell_size'], npad)
    for c in range(C):
        for p in range(P):
            plane = np.zeros((npad[0], npad[1]))
            st = npad // 2 - N // 2
            swv = sw[c, p] if sw[c, p] != 0 else 1.0
            plane[st[0]:st[0] + N[0], st[1]:st[1] + N[1]] = x[:, :, c, p] / swv / corr
            g = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(plane)))   # adjoint of ifftshift.ifft2.fftshift (x N^2)
            u = uvw[:, :, 0] * s[0, c]
            v = uvw[:, :, 1] * s[1, c]
            up, vp = u + npad[0] // 2, v + npad[1] // 2
            cu, cv = np.trunc(up + 0.5).astype(int), np.trunc(vp + 0.5).astype(int)
            ou = np.floor((cu - up) * 100 + 0.5).astype(int)
            ov = np.floor((cv - vp) * 100 + 0.5).astype(int)
            ok = (cu - 3 >= 0) & (cu + 3 < npad[0]) & (cv - 3 >= 0) & (cv + 3 < npad[1])
            acc = np.zeros((T, B), dtype=np.complex128)
            for iu in range(-3, 4):
                tu = cgk[np.abs(100 * iu + ou)]
                for iv in range(-3, 4):
                    tv = cgk[np.abs(100 * iv + ov)]
                    gu = np.clip(cu + iu, 0, npad[0] - 1)
                    gv = np.clip(cv + iv, 0, npad[1] - 1)
                    acc += tu * tv * g[gu, gv]
            out[:, :, c, p] = np.where(ok, acc * w[:, :, c, p], 0.0)
    return out


def test_degrid_matches_fp64_adjoint(ngg):
    import torch
    uvw, w, freq, gp, rng = _obs(seed=22, C=2, P=2)
    op = _op(uvw, w, freq, gp)
    N = gp['image_size'][0]
    x = rng.standard_normal((N, N, 2, 2))
    got = op.degrid(torch.as_tensor(x, device='cuda')).cpu().numpy()
    corr = O.remove_padding(O.create_prolate_spheroidal_correction(gp['image_size_padded']), gp['image_size'])
    ref = _numpy_degrid(x, uvw, w.astype(np.float64), freq, gp, op.sum_weight.cpu().numpy(), corr)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def test_backward_matches_finite_differences(ngg):
    import torch
    from cngi_prototype_gb300.imaging.degrid import degrid
    uvw, w, freq, gp, rng = _obs(seed=23)
    op = _op(uvw, w, freq, gp)
    T, B, C, P = w.shape
    N = gp['image_size'][0]
    x_true = torch.as_tensor(rng.uniform(0, 1, (N, N, C, P)), device='cuda')
    v_data = (op.degrid(x_true).to(torch.complex128) +
              torch.as_tensor(0.1 * (rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P))),
                              device='cuda')).to(torch.complex64)
    # The map is linear, so its backward does not depend on x; a small x keeps
    # the model visibilities small next to eps*A(delta), so the FP32 rounding of
    # A(x +- eps delta) does not swamp the central difference.
    x = torch.as_tensor(rng.uniform(0, 1e-3, (N, N, C, P)), device='cuda', dtype=torch.float64).requires_grad_(True)

    def loss(img):
        r = degrid(img, op).to(torch.complex128) - v_data.to(torch.complex128)
        return torch.sum(r.real ** 2 + r.imag ** 2)

    L = loss(x)
    L.backward()
    grad = x.grad.detach().cpu().numpy()
    eps = 1e-3
    idx = rng.integers(0, N, (256, 2))
    ch = rng.integers(0, C, 256)
    fd = np.empty(256)
    with torch.no_grad():
        for k in range(256):
            d = torch.zeros_like(x)
            d[idx[k, 0], idx[k, 1], ch[k], 0] = eps
            fd[k] = (float(loss(x + d)) - float(loss(x - d))) / (2 * eps)
    an = grad[idx[:, 0], idx[:, 1], ch, 0]
    rel = np.abs(fd - an) / np.abs(an).max()
    assert np.median(rel) < 1e-4 and rel.max() < 1e-3, (np.median(rel), rel.max())
    assert np.corrcoef(fd, an)[0, 1] > 0.999999


def test_gradient_is_twice_the_residual_image(ngg):
    """d chi2 / d image = 2 D(model - data): the reference gridder's residual image."""
    import torch
    from cngi_prototype_gb300.imaging.degrid import degrid
    uvw, w, freq, gp, rng = _obs(seed=24)
    op = _op(uvw, w, freq, gp)
    T, B, C, P = w.shape
    N = gp['image_size'][0]
    v_data = torch.as_tensor((rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P)))
                             .astype(np.complex64), device='cuda')
    x = torch.as_tensor(rng.uniform(0, 1, (N, N, C, P)), device='cuda').requires_grad_(True)
    vm = degrid(x, op)
    r = vm.to(torch.complex128) - v_data.to(torch.complex128)
    torch.sum(r.real ** 2 + r.imag ** 2).backward()
    resid = (vm.detach() - v_data).cpu().numpy()
    ref, _ = O.make_image_arrays(resid, uvw, w.astype(np.float64), freq, gp)   # FP64 reference gridder
    g = x.grad.cpu().numpy()
    # a noise-like residual image has a small peak next to its total flux, so
    # FP32 gridding errors are larger relative to the peak than for a sky image
    assert np.abs(g - 2 * ref).max() <= 5e-5 * np.abs(2 * ref).max()
