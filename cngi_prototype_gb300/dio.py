"""vis.zarr reading and writing (cngi/dio/read_vis.py, cngi/dio/write_vis.py)
for zarr version-2 directory stores, without the zarr package.

A store is a directory of partitions (xds0, xds1, ..., global/ANTENNA, ...);
each partition is a zarr group whose arrays are directories holding
`.zarray` (shape, chunks, dtype, compressor, fill_value, order, filters),
`.zattrs` (xarray's `_ARRAY_DIMENSIONS` and the variable's attributes) and one
file per chunk named by its chunk indices. A group may instead carry all of
that metadata in one consolidated `.zmetadata` file.

Supported chunk codecs: none, zlib, gzip, bz2 and lzma (the Python standard
library's), zstd, and Blosc with its zstd, zlib or lz4 compressors and byte
shuffle -- Blosc zstd being what the reference's writers use
(write_vis.py:62, Blosc(cname='zstd', clevel=2, shuffle=0)). Blosc and zstd
are decoded by this package's own readers of the published formats
(_blosc.py, _zstd.py: RFC 8878), since numcodecs is not available here.
Array filters are not supported (NotImplementedError naming them).
Values are returned as stored: no CF decoding (times keep their numeric
encoding and `units` attribute).
"""
import bz2
import gzip
import json
import lzma
import math
import os
import zlib

import numpy as np

from . import _blosc, _zstd
from . import xds as _xds

_DECODERS = {
    'zlib': zlib.decompress,
    'gzip': gzip.decompress,
    'bz2': bz2.decompress,
    'lzma': lzma.decompress,
    'zstd': _zstd.decompress,
    'blosc': _blosc.decompress,
}


_SPECIAL = {'NaN': np.nan, 'Infinity': np.inf, '-Infinity': -np.inf}


def _fill(meta, dtype):
    fv = meta.get('fill_value')
    if fv is None:
        return None
    if isinstance(fv, (list, tuple)) and dtype.kind == 'c':
        re, im = (_SPECIAL.get(x, x) if isinstance(x, str) else x for x in fv[:2])
        return np.array(complex(re, im)).astype(dtype)
    if isinstance(fv, str):
        fv = _SPECIAL.get(fv, fv)
    return np.array(fv).astype(dtype)


def _decode(raw, compressor, name):
    if compressor is None:
        return raw
    cid = compressor.get('id')
    if cid not in _DECODERS:
        raise NotImplementedError(f'{name}: chunk codec {cid!r} is not supported; '
                                  f'supported: none, ' + ', '.join(sorted(_DECODERS)))
    return _DECODERS[cid](raw)


def _read_array(path, meta, name):
    """One zarr v2 array: assemble its chunks (missing chunks take fill_value)."""
    if meta.get('zarr_format', 2) != 2:
        raise NotImplementedError(f'{name}: zarr_format {meta.get("zarr_format")} (only 2 is supported)')
    if meta.get('filters'):
        raise NotImplementedError(f'{name}: array filters {meta["filters"]} need numcodecs (not available)')
    dtype = np.dtype(meta['dtype'])
    if dtype.kind == 'O':
        raise NotImplementedError(f'{name}: object dtype needs numcodecs filters (not available)')
    shape = tuple(int(x) for x in meta['shape'])
    chunks = tuple(int(x) for x in meta['chunks'])
    order = meta.get('order', 'C')
    sep = meta.get('dimension_separator', '.')
    fill = _fill(meta, dtype)
    out = np.empty(shape, dtype=dtype)
    if fill is not None:
        out[...] = fill
    else:
        out[...] = np.zeros((), dtype=dtype)
    if len(shape) == 0:
        f = os.path.join(path, '0')
        if os.path.exists(f):
            with open(f, 'rb') as fh:
                out[...] = np.frombuffer(_decode(fh.read(), meta.get('compressor'), name), dtype=dtype)[0]
        return out
    grid = [int(math.ceil(s / c)) if c else 0 for s, c in zip(shape, chunks)]
    for idx in np.ndindex(*grid):
        f = os.path.join(path, sep.join(str(i) for i in idx))
        if not os.path.exists(f):
            continue
        with open(f, 'rb') as fh:
            buf = _decode(fh.read(), meta.get('compressor'), name)
        block = np.frombuffer(buf, dtype=dtype).reshape(chunks, order=order)
        sl = tuple(slice(i * c, min((i + 1) * c, s)) for i, c, s in zip(idx, chunks, shape))
        out[sl] = block[tuple(slice(0, x.stop - x.start) for x in sl)]
    return out


def _group_metadata(path, consolidated):
    """{array name: (.zarray, .zattrs)} and the group attributes."""
    zm = os.path.join(path, '.zmetadata')
    if consolidated and os.path.exists(zm):
        with open(zm) as fh:
            md = json.load(fh)['metadata']
        names = sorted({k.rsplit('/', 1)[0] for k in md if k.endswith('/.zarray')})
        arrays = {n: (md[n + '/.zarray'], md.get(n + '/.zattrs', {})) for n in names}
        return arrays, md.get('.zattrs', {})
    arrays = {}
    for n in sorted(os.listdir(path)):
        za = os.path.join(path, n, '.zarray')
        if os.path.isfile(za):
            with open(za) as fh:
                meta = json.load(fh)
            attrs = {}
            zt = os.path.join(path, n, '.zattrs')
            if os.path.isfile(zt):
                with open(zt) as fh:
                    attrs = json.load(fh)
            arrays[n] = (meta, attrs)
    gattrs = {}
    gz = os.path.join(path, '.zattrs')
    if os.path.isfile(gz):
        with open(gz) as fh:
            gattrs = json.load(fh)
    return arrays, gattrs


def read_xds(path, consolidated=True):
    """One zarr group as a Dataset: dims from `_ARRAY_DIMENSIONS`; arrays named
    after their own (single) dimension, and those listed in a variable's
    `coordinates` attribute, become coordinates (xarray's conventions)."""
    arrays, gattrs = _group_metadata(path, consolidated)
    values, dims, attrs = {}, {}, {}
    coord_names = set()
    for n, (meta, a) in arrays.items():
        a = dict(a)
        d = a.pop('_ARRAY_DIMENSIONS', None)
        if d is None:
            d = [f'{n}_dim_{i}' for i in range(len(meta['shape']))]
        coord_names.update(str(a.pop('coordinates', '')).split())
        values[n] = _read_array(os.path.join(path, n), meta, n)
        dims[n], attrs[n] = tuple(d), a
    coords, data_vars = {}, {}
    for n in arrays:
        is_coord = (len(dims[n]) == 1 and dims[n][0] == n) or n in coord_names
        (coords if is_coord else data_vars)[n] = _xds.DataArray(values[n], dims[n], attrs[n])
    return _xds.Dataset(data_vars, coords, gattrs)


def read_vis(infile, partition=None, chunks=None, consolidated=True, overwrite_encoded_chunks=True, **kwargs):
    """Read a vis.zarr store into a master dataset whose attrs map partition
    names (xds0, ..., and the global tables ANTENNA, FIELD, ...) to Datasets,
    as the reference's read_vis (read_vis.py:178-200, local-filesystem
    branch). partition: a name or list of names (None: every partition;
    'global' adds every global/<table>). chunks and overwrite_encoded_chunks
    are accepted for signature compatibility: arrays are read whole (dask
    chunking does not apply). S3 URLs are not supported."""
    if str(infile).lower().startswith('s3'):
        raise NotImplementedError('S3 stores are not supported (local directory stores only)')
    infile = os.path.expanduser(str(infile))
    if not os.path.isdir(infile):
        raise FileNotFoundError(infile)
    if partition is None:
        partition = sorted(p for p in os.listdir(infile) if not p.startswith('.'))
    partition = [str(p) for p in np.atleast_1d(partition)]
    if 'global' in partition and os.path.isdir(os.path.join(infile, 'global')):
        partition += sorted('global/' + t for t in os.listdir(os.path.join(infile, 'global'))
                            if not t.startswith('.'))
    parts = {}
    for p in partition:
        if p == 'global':
            continue
        path = os.path.join(infile, p)
        if os.path.isdir(path):
            parts[p.replace('global/', '')] = read_xds(path, consolidated)
    return _package(parts)


def _package(parts):
    """The master dataset with the id coordinates of the global tables
    (cngi/_utils/_io.py:37-64, the tables present)."""
    m = _xds.mxds(parts)
    ids = {'ANTENNA': ('antenna_ids', 'antenna_id'), 'FIELD': ('field_ids', 'field_id'),
           'FEED': ('feed_ids', 'feed_id'), 'OBSERVATION': ('observation_ids', 'observation_id'),
           'SOURCE': ('source_ids', 'source_id'), 'SPECTRAL_WINDOW': ('spw_ids', 'spectral_window_id'),
           'STATE': ('state_ids', 'state_id')}
    for table, (cname, var) in ids.items():
        t = parts.get(table)
        if t is not None and var in t:
            m.coords[cname] = _xds.DataArray(np.asarray(t[var].values), (cname,))
    return m


_ENCODERS = {'zlib': lambda b, lvl: zlib.compress(b, lvl), 'gzip': lambda b, lvl: gzip.compress(b, lvl),
             'bz2': lambda b, lvl: bz2.compress(b, max(1, lvl)), 'lzma': lambda b, lvl: lzma.compress(b)}


def _json_attrs(attrs):
    out = {}
    for k, v in attrs.items():
        if isinstance(v, np.ndarray):
            v = v.tolist()
        elif isinstance(v, np.generic):
            v = v.item()
        try:
            json.dumps(v)
        except TypeError:
            continue   # not representable in .zattrs (e.g. a dataset): left out
        out[k] = v
    return out


def _fill_json(dtype):
    if dtype.kind == 'f':
        return 'NaN'
    if dtype.kind == 'c':
        return ['NaN', 'NaN']
    if dtype.kind in 'iub':
        return 0 if dtype.kind != 'b' else False
    return None


def write_xds(ds, path, chunks_on_disk=None, compressor=None, level=2, consolidated=True):
    """One Dataset as a zarr v2 group (see write_vis)."""
    os.makedirs(path, exist_ok=True)
    comp = None if compressor is None else {'id': compressor, 'level': level}
    if compressor is not None and compressor not in _ENCODERS:
        raise NotImplementedError(f'codec {compressor!r} is not available; supported: none, '
                                  + ', '.join(sorted(_ENCODERS)))
    consolidated_md = {'.zgroup': {'zarr_format': 2}, '.zattrs': _json_attrs(getattr(ds, 'attrs', {}))}
    coords = dict(ds.coords)
    non_dim = [n for n, da in coords.items() if not (len(da.dims) == 1 and da.dims[0] == n)]
    items = list(coords.items()) + list(ds.data_vars.items())
    for n, da in items:
        a = np.ascontiguousarray(np.asarray(da.values))
        if a.dtype.kind in 'OU':
            a = a.astype('U') if a.dtype.kind == 'O' else a
        ch = [int(min(a.shape[i], (chunks_on_disk or {}).get(d, a.shape[i])) or 1) for i, d in enumerate(da.dims)]
        meta = {'zarr_format': 2, 'shape': list(a.shape), 'chunks': ch, 'dtype': a.dtype.str,
                'compressor': comp, 'fill_value': _fill_json(a.dtype), 'order': 'C', 'filters': None}
        attrs = dict(_json_attrs(getattr(da, 'attrs', {})), _ARRAY_DIMENSIONS=list(da.dims))
        if n in ds.data_vars and non_dim:
            attrs['coordinates'] = ' '.join(non_dim)
        ap = os.path.join(path, n)
        os.makedirs(ap, exist_ok=True)
        with open(os.path.join(ap, '.zarray'), 'w') as fh:
            json.dump(meta, fh)
        with open(os.path.join(ap, '.zattrs'), 'w') as fh:
            json.dump(attrs, fh)
        consolidated_md[n + '/.zarray'], consolidated_md[n + '/.zattrs'] = meta, attrs
        if a.ndim == 0:
            blocks = [((0,), a.reshape(()))]
        else:
            grid = [int(math.ceil(s / c)) for s, c in zip(a.shape, ch)]
            blocks = []
            for idx in np.ndindex(*grid):
                sl = tuple(slice(i * c, min((i + 1) * c, s)) for i, c, s in zip(idx, ch, a.shape))
                blk = np.zeros(ch, dtype=a.dtype)
                blk[tuple(slice(0, x.stop - x.start) for x in sl)] = a[sl]
                blocks.append((idx, blk))
        for idx, blk in blocks:
            raw = np.ascontiguousarray(blk).tobytes()
            if compressor is not None:
                raw = _ENCODERS[compressor](raw, level)
            with open(os.path.join(ap, '.'.join(str(i) for i in idx)), 'wb') as fh:
                fh.write(raw)
    with open(os.path.join(path, '.zgroup'), 'w') as fh:
        json.dump({'zarr_format': 2}, fh)
    with open(os.path.join(path, '.zattrs'), 'w') as fh:
        json.dump(consolidated_md['.zattrs'], fh)
    if consolidated:
        with open(os.path.join(path, '.zmetadata'), 'w') as fh:
            json.dump({'metadata': consolidated_md, 'zarr_consolidated_format': 1}, fh)


def write_vis(mxds, outfile, chunks_on_disk=None, partition=None, consolidated=True, compressor=None,
              graph_name='write_zarr'):
    """Write the master dataset's partitions (attrs holding Datasets) as a
    vis.zarr store (write_vis.py:26-90). The global tables (ANTENNA, FIELD,
    ...) go under global/. compressor: None (uncompressed; the reference's
    default is Blosc, which needs numcodecs) or 'zlib' / 'gzip' / 'bz2' /
    'lzma'. chunks_on_disk: {dim: chunk size}."""
    parts = partition if partition is not None else [k for k, v in mxds.attrs.items() if hasattr(v, 'data_vars')]
    for p in np.atleast_1d(parts):
        p = str(p)
        ds = mxds.attrs[p]
        sub = p if p.startswith('xds') else os.path.join('global', p)
        write_xds(ds, os.path.join(os.path.expanduser(str(outfile)), sub), chunks_on_disk, compressor,
                  consolidated=consolidated)
