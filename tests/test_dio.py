"""vis.zarr reading and writing (zarr v2 directory stores, standard-library
codecs): round trips of a visibility master dataset, stores written by hand
to the zarr v2 layout (missing chunks, edge chunks, F order, '/' separator,
consolidated metadata), and the refusal of codecs that need numcodecs."""
import json
import os
import zlib

import numpy as np
import pytest


def _mxds(rng):
    from cngi_prototype_gb300 import xds
    T, B, C, P = 7, 5, 6, 2
    uvw = rng.standard_normal((T, B, 3)) * 100
    vis = (rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P))).astype(np.complex64)
    w = rng.uniform(0.5, 2, (T, B, C, P)).astype(np.float32)
    flag = rng.uniform(size=(T, B, C, P)) < 0.1
    ds = xds.vis_dataset(uvw, vis, w, 1e9 + 1e6 * np.arange(C), flag=flag, field_id=np.zeros((T, B), np.int32))
    ds.attrs['note'] = 'synthetic'
    ant = xds.Dataset({'NAME': (('antenna_id',), np.array(['A0', 'A1', 'A2'])),
                       'POSITION': (('antenna_id', 'xyz'), rng.standard_normal((3, 3)))},
                      coords={'antenna_id': ('antenna_id', np.arange(3))})
    return xds.mxds({'xds0': ds, 'ANTENNA': ant})


@pytest.mark.parametrize('compressor', [None, 'zlib', 'bz2'])
@pytest.mark.parametrize('consolidated', [True, False])
def test_round_trip(tmp_path, compressor, consolidated):
    from cngi_prototype_gb300 import dio
    rng = np.random.default_rng(3)
    m = _mxds(rng)
    out = tmp_path / 'obs.vis.zarr'
    dio.write_vis(m, out, chunks_on_disk={'time': 3, 'chan': 4}, compressor=compressor, consolidated=consolidated)
    assert os.path.isdir(out / 'xds0' / 'DATA') and os.path.isdir(out / 'global' / 'ANTENNA')
    r = dio.read_vis(out, consolidated=consolidated)
    a, b = m.attrs['xds0'], r.attrs['xds0']
    for name in ('DATA', 'UVW', 'DATA_WEIGHT', 'FLAG', 'FIELD_ID'):
        assert b[name].dims == a[name].dims
        assert b[name].values.dtype == a[name].values.dtype
        assert np.array_equal(b[name].values, a[name].values)
    assert np.array_equal(b.coords['chan'].values, a.coords['chan'].values)
    assert b.attrs['note'] == 'synthetic'
    assert b.attrs['data_groups'] == a.attrs['data_groups']   # what the imaging API selects by
    # partitions: every one by default; one by name; global tables by 'global'
    assert np.array_equal(r.attrs['ANTENNA']['NAME'].values, m.attrs['ANTENNA']['NAME'].values)
    assert np.array_equal(r.coords['antenna_ids'].values, np.arange(3))
    only = dio.read_vis(out, partition='xds0')
    assert 'xds0' in only.attrs and 'ANTENNA' not in only.attrs
    glob = dio.read_vis(out, partition=['global'])
    assert 'ANTENNA' in glob.attrs and 'xds0' not in glob.attrs


def _write_array(path, data, chunks, meta_extra=None, sep='.', order='C', compress=None, skip=()):
    os.makedirs(path, exist_ok=True)
    meta = {'zarr_format': 2, 'shape': list(data.shape), 'chunks': list(chunks), 'dtype': data.dtype.str,
            'compressor': {'id': 'zlib', 'level': 1} if compress else None, 'fill_value': 'NaN',
            'order': order, 'filters': None, 'dimension_separator': sep}
    meta.update(meta_extra or {})
    with open(os.path.join(path, '.zarray'), 'w') as fh:
        json.dump(meta, fh)
    grid = [-(-s // c) for s, c in zip(data.shape, chunks)]
    for idx in np.ndindex(*grid):
        if idx in skip:
            continue
        blk = np.zeros(chunks, dtype=data.dtype)
        sl = tuple(slice(i * c, min((i + 1) * c, s)) for i, c, s in zip(idx, chunks, data.shape))
        blk[tuple(slice(0, x.stop - x.start) for x in sl)] = data[sl]
        raw = blk.tobytes(order=order)
        raw = zlib.compress(raw) if compress else raw
        key = sep.join(str(i) for i in idx)
        os.makedirs(os.path.dirname(os.path.join(path, key)), exist_ok=True)
        with open(os.path.join(path, key), 'wb') as fh:
            fh.write(raw)


def test_hand_written_zarr_v2_layout(tmp_path):
    """Edge chunks, a missing chunk (fill_value NaN), Fortran order, the '/'
    separator, zlib chunks and xarray's dimension attributes."""
    from cngi_prototype_gb300 import dio
    g = tmp_path / 'grp'
    a = np.arange(7 * 5, dtype=np.float64).reshape(7, 5)
    _write_array(g / 'A', a, (3, 2), order='F', sep='/', compress=True, skip={(1, 1)})
    with open(g / 'A' / '.zattrs', 'w') as fh:
        json.dump({'_ARRAY_DIMENSIONS': ['time', 'chan'], 'units': 'Jy'}, fh)
    _write_array(g / 'chan', np.linspace(1, 2, 5), (5,))
    with open(g / 'chan' / '.zattrs', 'w') as fh:
        json.dump({'_ARRAY_DIMENSIONS': ['chan']}, fh)
    with open(g / '.zgroup', 'w') as fh:
        json.dump({'zarr_format': 2}, fh)
    ds = dio.read_xds(str(g))
    got = ds['A'].values
    want = a.copy()
    want[3:6, 2:4] = np.nan                     # the chunk that was not written
    assert np.array_equal(got, want, equal_nan=True)
    assert ds['A'].dims == ('time', 'chan') and ds['A'].attrs['units'] == 'Jy'
    assert 'chan' in ds.coords and 'A' in ds.data_vars


def test_unsupported_codecs_and_filters_are_refused(tmp_path):
    from cngi_prototype_gb300 import dio
    g = tmp_path / 'grp'
    _write_array(g / 'B', np.ones((4,)), (4,), meta_extra={'compressor': {'id': 'snappy'}})
    with open(g / 'B' / '.zattrs', 'w') as fh:
        json.dump({'_ARRAY_DIMENSIONS': ['x']}, fh)
    with pytest.raises(NotImplementedError, match='snappy'):
        dio.read_xds(str(g))
    _write_array(g / 'B', np.ones((4,)), (4,), meta_extra={'filters': [{'id': 'delta', 'dtype': '<f8'}]})
    with pytest.raises(NotImplementedError, match='filters'):
        dio.read_xds(str(g))
    with pytest.raises(NotImplementedError, match='S3'):
        dio.read_vis('s3://bucket/obs.vis.zarr')


@pytest.mark.gpu
def test_make_image_from_a_store_equals_make_image_in_memory(ngg, tmp_path):
    """A master dataset written with write_vis and read back with read_vis
    images as the in-memory one (to the gridder's FP32 atomic order)."""
    from conftest import load_golden
    from cngi_prototype_gb300 import dio, xds
    from cngi_prototype_gb300.imaging import make_image
    d = load_golden('std_cube')
    m = xds.mxds({'xds0': xds.vis_dataset(d['uvw'], d['vis'], d['weight'], d['freq'])})
    dio.write_vis(m, tmp_path / 'o.vis.zarr', chunks_on_disk={'time': 8}, compressor='zlib')
    r = dio.read_vis(tmp_path / 'o.vis.zarr')
    gp = {'image_size': [int(x) for x in d['image_size']], 'cell_size': [float(x) for x in d['cell_arcsec']],
          'chan_mode': 'cube', 'phase_center': [0.0, 0.0]}
    a = make_image(m, xds.Dataset(), gp, {'xds': 'xds0'}, {})['IMAGE'].values
    b = make_image(r, xds.Dataset(), gp, {'xds': 'xds0'}, {})['IMAGE'].values
    assert a.shape == b.shape
    # the tile pass's FP32 shared-memory atomics land in a different order
    # each run; the correction image (1.3e-3 in the corners) amplifies that
    # rounding difference ~770x, to ~1e-6 of the peak
    assert np.abs(a - b).max() <= 2e-6 * np.abs(a).max()
