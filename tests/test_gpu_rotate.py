"""direction_rotate on the GPU against the reference's outputs
(tests/golden/rotate.npz) and, at large phases, against the oracle.

Tolerances: uvw 1e-12 relative (the row-vector product's rounding order);
complex64 output within 4 ulps of |vis| (the reference rounds its FP64
product to complex64; the phasor here is FP32 after a reduction of the phase
to a fraction of a turn in FP32 pairs, or in FP64 beyond 2^22 turns, ~1e-7);
complex128 output 1e-12 of |vis|.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('tag,ctr', [('ctr', True), ('noctr', False)])
def test_kernels_match_reference(ngg, tag, ctr):
    from cngi_prototype_gb300.imaging.direction_rotate import _row_fields
    d = load_golden('rotate')
    ids = d[f'rot_field_id_{tag}']
    rf = _row_fields(d['field_id'], ids)
    amax = np.abs(d['vis']).max()
    for single in (True, False):
        uvw_rot, vis_rot = ngg.direction_rotate(d['vis'], d['uvw'], rf, d['freq'], d[f'rotmat_{tag}'],
                                                d[f'phase_rotation_{tag}'], ctr, single)
        u = uvw_rot.cpu().numpy()
        assert np.abs(u - d[f'uvw_rot_{tag}']).max() <= 1e-12 * np.abs(d['uvw']).max()
        v = vis_rot.cpu().numpy()
        ref = d[f'vis_rot_{tag}_{"single" if single else "double"}']
        assert v.dtype == (np.complex64 if single else np.complex128)
        err = np.abs(v.astype(np.complex128) - ref).max()
        assert err <= (4 * 2.0 ** -24 * amax if single else 1e-12 * amax), err


def test_large_phases_against_oracle(ngg):
    """Baselines to 15 km at 100-116 GHz and field offsets to 0.05 rad:
    phases of ~3e5 turns, which the FP64 reduction to a fraction of a turn
    must carry."""
    from oracle import rotate as O
    rng = np.random.default_rng(5)
    T, B, C, P = 8, 40, 5, 2
    uvw = rng.uniform(-15000.0, 15000.0, (T, B, 3))
    field = np.repeat(np.array([0, 0, 1, 1, 1, 2, 2, 2])[:, None], B, axis=1)
    vis = (rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P))).astype(np.complex64)
    freq = 100e9 + np.arange(C) * 4e9
    dirs = [(0.5 + 0.02, 0.3), (0.5, 0.3 - 0.03), (0.5 - 0.05, 0.3 + 0.01)]
    for ctr in (True, False):
        mats, phase = O.rotation_mats(dirs, (0.5, 0.3), ctr)
        ids = np.array([0, 1, 2])
        ref_uvw = O.rotate_uvw(uvw, field, mats, ids)
        rf = O.row_fields(field, ids).astype(np.int32)
        for single in (True, False):
            ref = O.apply_phasor(vis, ref_uvw, field, freq, phase, ids, ctr, single)
            _, v = ngg.direction_rotate(vis, uvw, rf, freq, mats, phase, ctr, single)
            err = np.abs(v.cpu().numpy().astype(np.complex128) - ref).max() / np.abs(vis).max()
            # FP64 rounding of a ~3e5-turn phase (and of the uvw product order): ~1e-9 rad
            assert err < (5e-7 if single else 5e-9), (ctr, single, err)


def test_api_adds_rotated_group(ngg):
    from cngi_prototype_gb300 import xds
    from cngi_prototype_gb300.imaging import direction_rotate
    d = load_golden('rotate')
    vds = xds.vis_dataset(d['uvw'], d['vis'], np.ones(d['vis'].shape, np.float32), d['freq'],
                          field_id=d['field_id'])
    fds = xds.Dataset({'PHASE_DIR': (('field_id', 'd1', 'd2'), d['phase_dir'][:, None, :])},
                      coords={'field_id': ('field_id', d['field_ids'])})
    mx = xds.mxds({'xds0': vds}, FIELD=fds)
    out = direction_rotate(mx, {'new_phase_center': list(d['new_phase_center'])}, {'xds': 'xds0'})
    ds = out.attrs['xds0']
    assert 'DATA_ROT' in ds and 'UVW_ROT' in ds and 'DATA_ROT' not in mx.attrs['xds0']
    ref = d['vis_rot_ctr_single']
    assert np.abs(ds['DATA_ROT'].values.astype(np.complex128) - ref).max() <= 4 * 2.0 ** -24 * np.abs(d['vis']).max()
    assert np.abs(ds['UVW_ROT'].values - d['uvw_rot_ctr']).max() <= 1e-12 * np.abs(d['uvw']).max()
    grp = ds.attrs['data_groups'][0]
    new = [g for g in grp.values() if g.get('data') == 'DATA_ROT']
    assert new and new[0]['uvw'] == 'UVW_ROT'


@pytest.mark.parametrize('P', [1, 3, 4])
def test_pol_counts_and_fp64_fallback_phases(ngg, P):
    """Pol counts other than two (the per-pol path) and phases past 2^22 turns
    (15,000 km baselines, field offsets to 0.05 rad: up to ~2e8 turns), which
    take the FP64 reduction, against the oracle."""
    from oracle import rotate as O
    rng = np.random.default_rng(10 + P)
    T, B, C = 6, 24, 3
    uvw = rng.uniform(-1.5e7, 1.5e7, (T, B, 3))
    uvw[:, : B // 2] *= 1e-3   # half the baselines below the threshold
    field = np.repeat(np.array([0, 0, 1, 1, 2, 2])[:, None], B, axis=1)
    vis = (rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P))).astype(np.complex64)
    freq = 100e9 + np.arange(C) * 8e9
    dirs = [(0.5 + 0.02, 0.3), (0.5, 0.3 - 0.03), (0.5 - 0.05, 0.3 + 0.01)]
    mats, phase = O.rotation_mats(dirs, (0.5, 0.3), True)
    ids = np.array([0, 1, 2])
    ref_uvw = O.rotate_uvw(uvw, field, mats, ids)
    rf = O.row_fields(field, ids).astype(np.int32)
    pd = np.einsum('tbk,tk->tb', ref_uvw[:, :, :2], phase[rf, :2])
    assert np.abs(pd).max() * freq.max() / 299792458.0 > 2.0 ** 22   # the fallback is exercised
    ref = O.apply_phasor(vis, ref_uvw, field, freq, phase, ids, True, True)
    _, v = ngg.direction_rotate(vis, uvw, rf, freq, mats, phase, True, True)
    err = np.abs(v.cpu().numpy().astype(np.complex128) - ref) / np.abs(vis).max()
    small = np.abs(pd) * freq.max() / 299792458.0 < 2.0 ** 22
    assert err[small].max() < 5e-7
    # ~2e8-turn phases: the FP64 products themselves differ by ~1e-16 relative
    # between the oracle's and the kernel's operation order, ~1e-7 rad here
    assert err.max() < 2e-6, err.max()
