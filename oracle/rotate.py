"""Oracle (test infrastructure only): CPU restatement of direction_rotate.

Follows ngcasa/imaging/direction_rotate.py: calc_rotation_mats (:127-173),
_directional_cosine (:175-187), apply_rotation_matrix (:189-211) and
apply_phasor (:215-248). The rotation matrices are built from explicit
elementary rotations (the reference calls scipy's Rotation.from_euler with
intrinsic 'XZ' / 'ZX' sequences, i.e. R = R1 @ R2 for the first and second
axis); they agree with scipy's to rounding (1e-16), which the fixtures check.
"""
import numpy as np

C_LIGHT = 299792458.0


def _rx(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])


def _rz(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


def directional_cosine(phase_center):
    """(ra, dec) -> (cos ra cos dec, sin ra cos dec, sin dec)."""
    ra, dec = phase_center
    return np.array([np.cos(ra) * np.cos(dec), np.sin(ra) * np.cos(dec), np.sin(dec)])


def rotation_mats(field_phase_dirs, new_phase_center, common_tangent_reprojection=True):
    """Per field: the 3x3 uvw rotation and the phase-rotation vector."""
    ra0, dec0 = new_phase_center
    rot_new = _rx(np.pi / 2 - dec0) @ _rz(-ra0 + np.pi / 2)
    cos_new = directional_cosine((ra0, dec0))
    n = len(field_phase_dirs)
    mats = np.zeros((n, 3, 3))
    phase = np.zeros((n, 3))
    for i, (ra, dec) in enumerate(field_phase_dirs):
        rot_field = _rz(-np.pi / 2 + ra) @ _rx(dec - np.pi / 2)
        mats[i] = (rot_new @ rot_field).T
        if common_tangent_reprojection:
            mats[i, 2, 0:2] = 0.0
        phase[i] = rot_new @ (cos_new - directional_cosine((ra, dec)))
    return mats, phase


def row_fields(field_id, rot_field_id):
    """Index into rot_field_id of each time row's (single) field."""
    out = np.empty(field_id.shape[0], dtype=np.int64)
    for t in range(field_id.shape[0]):
        u = np.unique(field_id[t][field_id[t] > -1])
        assert len(u) == 1, 'field_id must be constant over baseline'
        out[t] = np.where(rot_field_id == u[0])[0][0]
    return out


def rotate_uvw(uvw, field_id, mats, rot_field_id):
    rf = row_fields(field_id, rot_field_id)
    out = np.zeros(uvw.shape, uvw.dtype)
    for t in range(uvw.shape[0]):   # row vector times matrix, per time row (:209)
        out[t] = uvw[t] @ mats[rf[t]]
    return out


def apply_phasor(vis, uvw_rot, field_id, freq, phase, rot_field_id, common_tangent_reprojection=True,
                 single_precision=True):
    k = 2 if common_tangent_reprojection else 3
    rf = row_fields(field_id, rot_field_id)
    pd = np.zeros(uvw_rot.shape[:2])
    for t in range(uvw_rot.shape[0]):   # (:234)
        pd[t] = uvw_rot[t, :, 0:k] @ phase[rf[t], 0:k]
    phasor = np.exp(2.0 * 1j * np.pi * pd[:, :, None] * np.asarray(freq)[None, None, :] / C_LIGHT)
    out = vis * phasor[:, :, :, None]
    if single_precision:
        out = out.astype(np.complex64).astype(np.complex128)
    return out
