"""grid_ps_host: channel-chunk streamed gridding from host arrays to host
grids equals one device-resident ngg_grid_ps call (to FP32 atomic order)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('chunk', [1, 2, 5])
def test_streamed_equals_resident(ngg, chunk):
    import torch
    from cngi_prototype_gb300.imaging._imaging_utils import _gridding_convolutional_kernels as G
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    d = load_golden('std_cube')
    gp = {'image_size': [int(x) for x in d['image_size']], 'cell_size': [float(x) for x in d['cell_arcsec']]}
    _check_grid_parms(gp)
    npad, cell = gp['image_size_padded'], gp['cell_size']
    cgk = G._create_prolate_spheroidal_kernel_1D(100, 7)
    w = d['weight'].astype(np.float32)
    g_ref, sw_ref = ngg.grid_ps(d['vis'], d['uvw'], w, d['freq'], cgk, npad, cell)
    g_ref, sw_ref = g_ref.cpu().numpy(), sw_ref.cpu().numpy()
    C, P = w.shape[2], w.shape[3]
    out = torch.zeros((C, P, int(npad[0]), int(npad[1])), dtype=torch.complex64, pin_memory=True)
    sw = ngg.grid_ps_host(torch.as_tensor(d['vis']).pin_memory(), d['uvw'], torch.as_tensor(w).pin_memory(), d['freq'],
                          cgk, npad, cell, out=out, chan_chunk=chunk)
    pk = np.abs(g_ref).max()
    assert np.abs(out.numpy() - g_ref).max() <= 1e-6 * pk
    assert np.allclose(sw, sw_ref, rtol=1e-12, atol=0)
    got = {}
    ngg.grid_ps_host(d['vis'], d['uvw'], w, d['freq'], cgk, npad, cell, chan_chunk=chunk,
                     on_chunk=lambda c0, c1, h: got.__setitem__(c0, h.numpy().copy()))
    cat = np.concatenate([got[k] for k in sorted(got)])
    assert cat.shape == g_ref.shape and np.abs(cat - g_ref).max() <= 1e-6 * pk


@pytest.mark.parametrize('where', ['device', 'pinned'])
def test_grid_ps_chunk_reads_a_channel_range_in_place(ngg, where):
    """ngg_grid_ps_chunk on channels [c0, c1) of the whole arrays (device or
    pinned host memory) equals ngg_grid_ps on the sliced arrays."""
    import torch
    from cngi_prototype_gb300.imaging._imaging_utils import _gridding_convolutional_kernels as G
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_grid_parms
    d = load_golden('std_cube')
    gp = {'image_size': [int(x) for x in d['image_size']], 'cell_size': [float(x) for x in d['cell_arcsec']]}
    _check_grid_parms(gp)
    npad, cell = gp['image_size_padded'], gp['cell_size']
    cgk = G._create_prolate_spheroidal_kernel_1D(100, 7)
    vis = d['vis'].astype(np.complex64)
    w = d['weight'].astype(np.float32)
    C = w.shape[2]
    c0, c1 = 1, C - 1
    g_ref, sw_ref = ngg.grid_ps(np.ascontiguousarray(vis[:, :, c0:c1]), d['uvw'], np.ascontiguousarray(w[:, :, c0:c1]),
                                d['freq'][c0:c1], cgk, npad, cell)
    vt, wt = torch.as_tensor(vis), torch.as_tensor(w)
    if where == 'device':
        vt, wt = vt.cuda(), wt.cuda()
    else:
        vt, wt = vt.pin_memory(), wt.pin_memory()
    g, sw = ngg.grid_ps(vt, d['uvw'], wt, d['freq'][c0:c1], cgk, npad, cell, chan_offset=c0, chan_total=C)
    g_ref = g_ref.cpu().numpy()
    assert np.abs(g.cpu().numpy() - g_ref).max() <= 1e-6 * np.abs(g_ref).max()
    assert np.array_equal(sw.cpu().numpy(), sw_ref.cpu().numpy())
    with pytest.raises(ValueError):
        ngg.grid_ps(vt, d['uvw'], wt, d['freq'][c0:], cgk, npad, cell, chan_offset=c0 + 1, chan_total=C)
