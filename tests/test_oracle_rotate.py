"""direction_rotate: the oracle against the reference's own outputs
(tests/golden/rotate.npz, made by make_golden.py rotate), and the host-side
rotation matrices and row-field mapping of the library's API."""
import numpy as np
import pytest

from conftest import load_golden


def _cases():
    return [('ctr', True), ('noctr', False)]


@pytest.mark.parametrize('tag,ctr', _cases())
def test_oracle_matches_reference_bit_for_bit(tag, ctr):
    from oracle import rotate as O
    d = load_golden('rotate')
    rot_ids = d[f'rot_field_id_{tag}']
    uvw_rot = O.rotate_uvw(d['uvw'], d['field_id'], d[f'rotmat_{tag}'], rot_ids)
    assert np.array_equal(uvw_rot, d[f'uvw_rot_{tag}'])
    for single in (True, False):
        v = O.apply_phasor(d['vis'], d[f'uvw_rot_{tag}'], d['field_id'], d['freq'], d[f'phase_rotation_{tag}'],
                           rot_ids, ctr, single)
        assert np.array_equal(v, d[f'vis_rot_{tag}_{"single" if single else "double"}'])


@pytest.mark.parametrize('tag,ctr', _cases())
def test_oracle_rotation_matrices(tag, ctr):
    """Explicit elementary rotations agree with the reference's scipy Euler matrices."""
    from oracle import rotate as O
    d = load_golden('rotate')
    ids, pdirs = d['field_ids'], d['phase_dir']
    sel = [pdirs[int(np.where(ids == f)[0][0])] for f in d[f'rot_field_id_{tag}']]
    mats, phase = O.rotation_mats(sel, d['new_phase_center'], ctr)
    assert np.abs(mats - d[f'rotmat_{tag}']).max() < 1e-15
    assert np.abs(phase - d[f'phase_rotation_{tag}']).max() < 1e-18


@pytest.mark.parametrize('tag,ctr', _cases())
def test_api_host_matrices_and_row_fields(tag, ctr):
    from cngi_prototype_gb300 import xds
    from cngi_prototype_gb300.imaging.direction_rotate import _row_fields, calc_rotation_mats
    d = load_golden('rotate')
    fds = xds.Dataset({'PHASE_DIR': (('field_id', 'd1', 'd2'), d['phase_dir'][:, None, :])},
                      coords={'field_id': ('field_id', d['field_ids'])})
    mats, phase, ids = calc_rotation_mats(d['field_id'], fds, {'new_phase_center': list(d['new_phase_center']),
                                                             'common_tangent_reprojection': ctr})
    assert np.array_equal(ids, d[f'rot_field_id_{tag}'])
    assert np.abs(mats - d[f'rotmat_{tag}']).max() < 1e-15
    assert np.abs(phase - d[f'phase_rotation_{tag}']).max() < 1e-18
    rf = _row_fields(d['field_id'], ids)
    assert list(rf) == [1, 1, 1, 1, 0, 0, 0, 2, 2, 2]


def test_row_fields_rejects_mixed_rows():
    from cngi_prototype_gb300.imaging.direction_rotate import _row_fields
    f = np.array([[1, 1], [1, 2]])
    with pytest.raises(ValueError):
        _row_fields(f, np.array([1, 2]))


def test_rotation_parms_defaults():
    from cngi_prototype_gb300.imaging._imaging_utils._check_imaging_parms import _check_rotation_parms
    p = {'new_phase_center': [0.1, 0.2]}
    assert _check_rotation_parms(p)
    assert p['common_tangent_reprojection'] is True and p['single_precision'] is True
    assert not _check_rotation_parms({'new_phase_center': [0.1]})
