"""direction_rotate -- same signature and semantics as
ngcasa/imaging/direction_rotate.py:28-123: rotate uvw to a new phase centre
and phase-rotate the visibilities (on the GPU), adding UVW_ROT and DATA_ROT
in a new data group.

The per-field rotation matrices are computed on the host as the reference
does (calc_rotation_mats, :127-173, with scipy's Rotation); the rotation of
every row and the phasor of every visibility run in libngg
(ngg_rotate_uvw, ngg_phase_rotate). With single_precision (default) the
rotated visibilities are complex64 -- the values the reference produces when
it rounds its FP64 product to complex64 (:245-246), kept at the documented
64-bit width; otherwise complex128.
"""
import copy

import numpy as np

from .. import _lib
from ..xds import set_var
from ._imaging_utils._check_imaging_parms import _check_rotation_parms
from ._imaging_utils._pipeline import _arr
from ._imaging_utils._sel import _check_sel_parms, _register_group


def _directional_cosine(phase_center):
    """direction_rotate.py:175-187."""
    ra, dec = phase_center
    return np.array([np.cos(ra) * np.cos(dec), np.sin(ra) * np.cos(dec), np.sin(dec)])


def _field_phase_dirs(field_ds, field_ids):
    """(n, 2) phase directions (ra, dec) of the given field ids, from
    PHASE_DIR (field_id, d1, d2) at d1 = 0 (the reference's
    PHASE_DIR.sel(field_id=..., d1=0))."""
    pd = field_ds['PHASE_DIR'] if not hasattr(field_ds, 'PHASE_DIR') else field_ds.PHASE_DIR
    if hasattr(pd, 'sel') and hasattr(pd, 'coords') and not isinstance(getattr(pd, 'coords'), dict):
        return np.asarray(pd.sel(field_id=field_ids, d1=0).values, dtype=np.float64)
    vals = np.asarray(pd.values if hasattr(pd, 'values') else pd, dtype=np.float64)
    ids = np.asarray(field_ds['field_id'].values if 'field_id' in field_ds else np.arange(vals.shape[0]))
    idx = []
    for f in field_ids:
        hit = np.where(ids == f)[0]
        if len(hit) == 0:
            raise ValueError(f'field {f} has no PHASE_DIR')
        idx.append(int(hit[0]))
    return vals[idx, 0, :] if vals.ndim == 3 else vals[idx]


def calc_rotation_mats(field_id, field_ds, rotation_parms):
    """(uvw_rotmat (n,3,3), phase_rotation (n,3), rot_field_id (n,)) for the
    fields present in FIELD_ID (direction_rotate.py:127-173)."""
    from scipy.spatial.transform import Rotation as R
    ra0, dec0 = rotation_parms['new_phase_center']
    rot_new = R.from_euler('XZ', [[np.pi / 2 - dec0, -ra0 + np.pi / 2]]).as_matrix()[0]
    cos_new = _directional_cosine((ra0, dec0))
    fid = np.unique(np.asarray(field_id))
    fid = fid[fid > -1]
    dirs = _field_phase_dirs(field_ds, fid)
    mats = np.zeros((len(fid), 3, 3))
    phase = np.zeros((len(fid), 3))
    for i, (ra, dec) in enumerate(dirs):
        rot_field = R.from_euler('ZX', [[-np.pi / 2 + ra, dec - np.pi / 2]]).as_matrix()[0]
        mats[i] = np.matmul(rot_new, rot_field).T
        if rotation_parms['common_tangent_reprojection']:
            mats[i, 2, 0:2] = 0.0   # common tangent plane (joint mosaics)
        phase[i] = np.matmul(rot_new, cos_new - _directional_cosine((ra, dec)))
    return mats, phase, fid


def _row_fields(field_id, rot_field_id):
    """Index into rot_field_id of each time row's field; the reference asserts
    one field per time row (:200-204, :228-232)."""
    f = np.asarray(field_id)
    out = np.empty(f.shape[0], dtype=np.int32)
    pos = {int(v): i for i, v in enumerate(rot_field_id)}
    for t in range(f.shape[0]):
        u = np.unique(f[t][f[t] > -1])
        if len(u) != 1:
            raise ValueError('direction_rotate only supports xds where field_id remains constant over baseline.')
        out[t] = pos[int(u[0])]
    return out


def direction_rotate(mxds, rotation_parms, sel_parms):
    """Rotate uvw and phase-rotate the visibilities to
    rotation_parms['new_phase_center'] (radians, same frame as the fields'
    PHASE_DIR). rotation_parms['common_tangent_reprojection'] (default True)
    keeps w out of the phase and zeroes the w row's u, v terms, as a joint
    mosaic needs. Adds UVW_ROT and DATA_ROT (sel_parms['data_group_out']
    overrides the names) in a new data group; the inputs are not modified."""
    _mxds = mxds.copy(deep=False)
    _rp = copy.deepcopy(rotation_parms)
    _sp = copy.deepcopy(sel_parms)
    assert _check_rotation_parms(_rp), '######### ERROR: rotation_parms checking failed'
    assert 'xds' in _sp, '######### ERROR: xds must be specified in sel_parms'
    _vis = _mxds.attrs[_sp['xds']].copy(deep=False)
    _mxds.attrs[_sp['xds']] = _vis
    _check_sel_parms(_vis, _sp, new_or_modified_data_variables={'uvw': 'UVW_ROT', 'data': 'DATA_ROT'})
    gin, gout = _sp['data_group_in'], _sp['data_group_out']
    field_id = np.asarray(_arr(_vis['FIELD_ID']))
    field_ds = _mxds.attrs['FIELD'] if 'FIELD' in _mxds.attrs else _mxds.FIELD
    mats, phase, rot_ids = calc_rotation_mats(field_id, field_ds, _rp)
    row_field = _row_fields(field_id, rot_ids)
    vis = _arr(_vis[gin['data']]) if 'data' in gin else None
    uvw_rot, vis_rot = _lib.direction_rotate(vis, _arr(_vis[gin['uvw']]), row_field, _vis.coords['chan'].values,
                                             mats, phase, _rp['common_tangent_reprojection'], _rp['single_precision'])
    set_var(_vis, gout['uvw'], uvw_rot.cpu().numpy(), _vis[gin['uvw']].dims)
    if vis_rot is not None:
        set_var(_vis, gout['data'], vis_rot.cpu().numpy(), _vis[gin['data']].dims)
    _register_group(_vis, gout)
    return _mxds
