"""Parameter checking with the reference's defaults and derived values.

Mirrors ngcasa/imaging/_imaging_utils/_check_imaging_parms.py: each checker
fills defaults in place, prints an '######### ERROR' line and returns False on
a bad value, and derives the same quantities (_check_grid_parms :23-41:
image_size_padded = int(fft_padding*image_size), cell_size arcsec -> rad with
the sign of cell_size[0] flipped).
"""
import numbers

import numpy as np

ARCSEC_TO_RAD = np.pi / (3600 * 180)


def _err(msg):
    print('######### ERROR:', msg)
    return False


def _check(parms, key, types, default=None, acceptable=None, rng=None, list_len=None, elem_types=None):
    if key not in parms:
        if default is None:
            return _err(f"Parameter {key} must be specified")
        parms[key] = default
        return True
    v = parms[key]
    if list_len is not None:
        if not isinstance(v, (list, tuple, np.ndarray)):
            return _err(f"Parameter {key} must be a list")
        if list_len != -1 and len(v) != list_len:
            return _err(f"Parameter {key} must have length {list_len}")
        for x in v:
            if elem_types and not isinstance(x, elem_types):
                return _err(f"Parameter {key} must be a list of {elem_types}")
            if rng is not None and (x < rng[0] or x > rng[1]):
                return _err(f"Invalid {key}. Must be within the range {rng}.")
        return True
    if not isinstance(v, types):
        return _err(f"Parameter {key} must be of type {types}")
    if acceptable is not None and v not in acceptable:
        return _err(f"Invalid {key}. Can only be one of {acceptable}.")
    if rng is not None and (v < rng[0] or v > rng[1]):
        return _err(f"Invalid {key}. Must be within the range {rng}.")
    return True


_INT = (int, np.integer)


def _check_grid_parms(grid_parms):
    ok = True
    ok &= _check(grid_parms, 'image_size', None, list_len=2, elem_types=_INT)
    if 'image_size' in grid_parms:
        ok &= _check(grid_parms, 'image_center', None, default=list(np.array(grid_parms['image_size']) // 2),
                     list_len=2, elem_types=_INT)
    ok &= _check(grid_parms, 'cell_size', None, list_len=2, elem_types=numbers.Number)
    ok &= _check(grid_parms, 'fft_padding', numbers.Number, default=1.2, rng=[1, 10])
    ok &= _check(grid_parms, 'chan_mode', str, default='cube', acceptable=['cube', 'continuum'])
    # not in the reference: precision of the inverse FFT ('double' removes the
    # FP32 transform's error floor, up to ~6e-6 of the peak in the image
    # corners, at ~15-25x the transform time; 'auto' takes 'double' while the
    # padded planes of the cube hold at most 2^26 cells, 'single' above)
    ok &= _check(grid_parms, 'fft_precision', str, default='auto', acceptable=['auto', 'single', 'double'])
    if ok:
        grid_parms['image_size'] = np.array(grid_parms['image_size']).astype(int)
        grid_parms['image_size_padded'] = (grid_parms['fft_padding'] * grid_parms['image_size']).astype(int)
        grid_parms['image_center'] = np.array(grid_parms['image_center'])
        grid_parms['cell_size'] = ARCSEC_TO_RAD * np.array(grid_parms['cell_size'], dtype=np.float64)
        grid_parms['cell_size'][0] = -grid_parms['cell_size'][0]
    return bool(ok)


def _check_imaging_weights_parms(p):
    ok = _check(p, 'weighting', str, default='natural', acceptable=['natural', 'uniform', 'briggs', 'briggs_abs'])
    if ok and p['weighting'] == 'briggs_abs':
        ok &= _check(p, 'briggs_abs_noise', numbers.Number, default=1.0)
    if ok and p['weighting'] in ('briggs', 'briggs_abs'):
        ok &= _check(p, 'robust', numbers.Number, default=0.5, rng=[-2, 2])
    return bool(ok)


def _check_pb_parms(img_dataset, pb_parms):
    """_check_pb_parms (_check_imaging_parms.py:148-164): function (default
    'casa_airy'), dish and blockage diameter lists of equal length."""
    ok = _check(pb_parms, 'function', str, default='casa_airy', acceptable=['casa_airy', 'airy'])
    ok &= _check(pb_parms, 'list_dish_diameters', list, list_len=-1, elem_types=numbers.Number)
    ok &= _check(pb_parms, 'list_blockage_diameters', list, list_len=-1, elem_types=numbers.Number)
    if ok and len(pb_parms['list_dish_diameters']) != len(pb_parms['list_blockage_diameters']):
        ok = _err('Parameter list_dish_diameters and list_blockage_diameters must be the same length.')
    del img_dataset
    return bool(ok)


def _check_rotation_parms(p):
    """_check_imaging_parms.py:96-106 of the reference."""
    ok = _check(p, 'new_phase_center', None, list_len=2, elem_types=numbers.Number)
    ok &= _check(p, 'common_tangent_reprojection', bool, default=True)
    ok &= _check(p, 'single_precision', bool, default=True)
    return bool(ok)


def _check_norm_parms(p):
    ok = _check(p, 'norm_type', str, default='flat_sky', acceptable=['flat_noise', 'flat_sky', 'none'])
    ok &= _check(p, 'single_precision', bool, default=True)
    ok &= _check(p, 'pb_limit', numbers.Number, default=0.2)
    return bool(ok)


def _check_gcf_parms(p):
    """_check_imaging_parms.py:45-84: defaults and array conversion of gcf_parms."""
    ok = _check(p, 'function', str, default='casa_airy', acceptable=['casa_airy', 'airy'])
    for k in ('freq_chan', 'list_dish_diameters', 'list_blockage_diameters', 'unique_ant_indx', 'pol'):
        ok &= _check(p, k, None, list_len=-1, elem_types=numbers.Number)
    ok &= _check(p, 'chan_tolerance_factor', numbers.Number, default=0.005)
    ok &= _check(p, 'oversampling', None, default=[10, 10], list_len=2, elem_types=_INT)
    ok &= _check(p, 'max_support', None, default=[15, 15], list_len=2, elem_types=_INT)
    ok &= _check(p, 'support_cut_level', numbers.Number, default=2.5e-2)
    ok &= _check(p, 'a_chan_num_chunk', _INT, default=3)
    if ok and len(p['list_dish_diameters']) != len(p['list_blockage_diameters']):
        ok = _err('Parameter list_dish_diameters and list_blockage_diameters must be the same length.')
    if ok:
        p['oversampling'] = np.array(p['oversampling']).astype(int)
        p['max_support'] = np.array(p['max_support']).astype(int)
        for k in ('freq_chan', 'list_dish_diameters', 'list_blockage_diameters', 'unique_ant_indx', 'pol'):
            p[k] = np.array(p[k])
    return bool(ok)
