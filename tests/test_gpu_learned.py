"""Learned GCF: the GPU network's forward (FP32 and tcgen05 tensor cores),
its hand-written backward and Adam step against the CPU oracle; training on
the GCFs the method generates; learned mosaic gridding against the table
path, and what the network gains over the table."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import imaging as O
from oracle import mlp as OM
from oracle import mosaic as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def case():
    rng = np.random.default_rng(0)
    p = OM.init_params(3)
    z = rng.uniform(-1, 1, (3000, 3)).astype(np.float32)
    t = rng.standard_normal(3000).astype(np.float32)
    return p, z, t


def test_forward_matches_oracle(ngg, case):
    p, z, _ = case
    ref, _ = OM.forward(p, z)
    got = ngg.mlp_forward(p, z).cpu().numpy()
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()


def test_tensor_core_forward_matches_oracle(ngg, case):
    """Split-BF16 operands on tcgen05 with FP32 accumulation: FP32-level error;
    an odd sample count exercises the partial last tile."""
    p, z, _ = case
    ref, _ = OM.forward(p, z[:2999])
    got = ngg.mlp_forward(p, z[:2999], tensor_cores=True).cpu().numpy()
    assert np.abs(got - ref).max() <= 2e-4 * np.abs(ref).max()
    assert np.corrcoef(got, ref)[0, 1] > 0.9999999


def test_loss_gradient_matches_oracle(ngg, case):
    p, z, t = case
    L_ref, g_ref = OM.loss_grad(p, z, t)
    L, g = ngg.mlp_loss_grad(p, z, t)
    g = g.cpu().numpy()
    assert abs(L - L_ref) <= 1e-6 * L_ref
    assert np.linalg.norm(g - g_ref) <= 1e-5 * np.linalg.norm(g_ref)
    assert np.all(g[OM.N_TRAINED:] == 0)                      # the Fourier matrix is not trained


def test_adam_step_matches_oracle(ngg, case):
    import torch
    p, z, t = case
    _, g = ngg.mlp_loss_grad(p, z, t)
    pt = torch.as_tensor(p, device='cuda').clone()
    m = torch.zeros(ngg.MLP_NTRAINED, device='cuda')
    v = torch.zeros_like(m)
    gn = g.cpu().numpy().astype(np.float64)
    pr, mr, vr = p.astype(np.float64), np.zeros(ngg.MLP_NPARAM), np.zeros(ngg.MLP_NPARAM)
    for step in (1, 2, 3):
        ngg.mlp_adam(pt, g, m, v, step, 1e-3)
        pr, mr, vr = OM.adam(pr, gn, mr, vr, step, 1e-3)
    assert np.abs(pt.cpu().numpy() - pr).max() <= 1e-6


def _golden_gp():
    gp = {'image_size': [64, 64], 'cell_size': [2.0, 2.0], 'fft_padding': 1.2}
    O.check_grid_parms(gp)
    return gp


@pytest.fixture(scope='module')
def trained(ngg):
    """A network trained (30k steps, a few seconds) on the golden mosaic
    geometry's GCFs at 10 frequencies over the channels' band +- 10%."""
    from cngi_prototype_gb300.imaging.learned_gcf import LearnedGCF
    d = load_golden('mosaic')
    f = d['freq']
    bw = f.max() - f.min()
    lg = LearnedGCF.fit('casa_airy', 12.0, 0.75, (f.min() - 0.1 * bw, f.max() + 0.1 * bw), _golden_gp(), [4, 4],
                        [15, 15], n_freq=10, steps=30000, batch=16384)
    return lg, d


def test_training_fits_the_gcf(ngg, trained):
    from cngi_prototype_gb300.imaging.make_gridding_convolution_function import gcf_tables
    lg, d = trained
    h = lg.info['loss_history']
    assert h[-100:].mean() < 1e-4 * h[:10].mean()
    ck, _, sup = gcf_tables('casa_airy', [12.0], [0.75], np.array([[0, 0]]), d['freq'], _golden_gp(), [4, 4],
                            [15, 15], 0.025)
    for c, f in enumerate(d['freq']):       # channel frequencies are not training frequencies
        tab = lg.table(f, tensor_cores=True)
        w = tab.shape[0] // 2
        ref = ck[0, c, 0, 32 - w:32 + w + 1, 32 - w:32 + w + 1].cpu().numpy()
        assert np.sqrt(np.mean((tab - ref) ** 2)) <= 1e-3 * np.abs(ref).max()
        assert np.abs(tab - ref).max() <= 5e-3 * np.abs(ref).max()


def _dirty(g, sw):
    im = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(g, axes=(2, 3))), axes=(2, 3)).real
    return im / np.where(sw == 0, 1, sw)[:, :, None, None]


def test_learned_mosaic_grid_and_gain(ngg, trained):
    """Learned gridding against an FP64 oracle grid made with tables at every
    channel's exact frequency; the gain: the reference's default table path
    (one GCF per PB channel, chan_tolerance_factor 0.005) is farther from that
    answer than the learned path, and its tables are far larger."""
    from cngi_prototype_gb300.imaging.make_gridding_convolution_function import gcf_tables
    lg, d = trained
    gp = _golden_gp()
    npad = gp['image_size_padded']
    f = d['freq']
    C = len(f)
    fidx = np.where(d['field'] >= 0, d['field'], -1)
    sl = M.phase_slopes(d['field_phase_dir'], d['phase_center'], npad, gp['cell_size'], d['oversampling'])
    pg = M.phase_gradient(sl, (64, 64))
    iw = d['imaging_weight'].astype(np.float32).astype(np.float64)
    ck_x, _, sup_x = gcf_tables('casa_airy', [12.0], [0.75], np.array([[0, 0]]), f, gp, [4, 4], [15, 15], 0.025)
    ref, rsw = M.aperture_grid(d['vis'], d['uvw'], iw, d['field'], np.arange(2), np.zeros(15, int), np.arange(C),
                               np.zeros(2, int), ck_x.cpu().numpy(), sup_x, pg, f, npad, gp['cell_size'], [4, 4])
    gl, swl = lg.grid(d['vis'], d['uvw'], iw.astype(np.float32), f, fidx.astype(np.int32), sl, npad, gp['cell_size'])
    gl, swl = gl.cpu().numpy(), swl.cpu().numpy()
    i_ref, i_l = _dirty(ref, rsw), _dirty(gl, swl)
    pk = np.abs(i_ref).max()
    err_learned = np.abs(i_l - i_ref).max() / pk
    # the reference's default: GCFs at the PB channels of create_cf_chan_map
    gt, swt = M.aperture_grid(d['vis'], d['uvw'], iw, d['field'], np.arange(2), d['cf_baseline_map'],
                              d['cf_chan_map'], d['cf_pol_map'], d['conv_kernel'], d['support'], pg, f, npad,
                              gp['cell_size'], [4, 4])
    err_table = np.abs(_dirty(gt, swt) - i_ref).max() / pk
    assert err_learned <= 1e-3, err_learned
    assert err_learned < err_table, (err_learned, err_table)
    assert np.allclose(swl, rsw, rtol=3e-3)


def test_learned_rejects_bad_layout(ngg, trained):
    lg, d = trained
    with pytest.raises(ngg.NggError, match='support'):
        ngg.grid_gcf_learned(d['vis'], d['uvw'], d['imaging_weight'], d['freq'], np.zeros((20, 15), np.int32),
                             np.zeros((2, 2), np.int32), np.zeros((2, 2)), lg.params, lg.scale, lg.conv_size,
                             (76, 76), (1e-5, 1e-5), (4, 4))
