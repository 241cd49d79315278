"""A minimal stand-in for the xarray objects the imaging API exchanges.

The reference's API passes xarray Datasets (a multi-dataset `mxds` whose
attrs hold visibility datasets, and image datasets). xarray is not available
on every machine this library runs on, so the API works on any object that
offers the small interface used here -- `ds[name]` returning an object with
`.data`/`.values`/`.dims`, `ds.coords[name]`, `ds.attrs`, `ds.dims` (name ->
size), item assignment and `copy(deep=True)` -- and ships this container for
when xarray is absent. Real xarray Datasets work unchanged.
"""
import copy

import numpy as np


class DataArray:
    def __init__(self, data, dims, attrs=None):
        self.data = data
        self.dims = tuple(dims)
        self.attrs = dict(attrs or {})
        if getattr(data, 'ndim', len(self.dims)) != len(self.dims):
            raise ValueError(f'data has {np.ndim(data)} dims, got names {self.dims}')

    @property
    def values(self):
        d = self.data
        if hasattr(d, 'detach'):
            d = d.detach().cpu().numpy()
        return np.asarray(d)

    @property
    def shape(self):
        return tuple(self.data.shape)

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def ndim(self):
        return len(self.dims)

    def __array__(self, dtype=None):
        return self.values if dtype is None else self.values.astype(dtype)

    def __getitem__(self, k):
        return self.values[k]

    def __len__(self):
        return self.shape[0]

    def mean(self):
        return DataArray(np.asarray(np.mean(self.values)), ())

    def __repr__(self):
        return f'<DataArray {self.dims} {self.shape} {self.dtype}>'


class Dataset:
    def __init__(self, data_vars=None, coords=None, attrs=None):
        object.__setattr__(self, '_vars', {})
        object.__setattr__(self, 'coords', {})
        object.__setattr__(self, 'attrs', dict(attrs or {}))
        for k, v in (coords or {}).items():
            self.coords[k] = _as_da(v, k)
        for k, v in (data_vars or {}).items():
            self[k] = v

    # mapping interface
    def __getitem__(self, name):
        if name in self._vars:
            return self._vars[name]
        if name in self.coords:
            return self.coords[name]
        raise KeyError(name)

    def __setitem__(self, name, value):
        self._vars[name] = _as_da(value, name)

    def __contains__(self, name):
        return name in self._vars or name in self.coords

    def __getattr__(self, name):
        if name.startswith('__'):
            raise AttributeError(name)
        v = self.__dict__.get('_vars', {})
        if name in v:
            return v[name]
        c = self.__dict__.get('coords', {})
        if name in c:
            return c[name]
        a = self.__dict__.get('attrs', {})
        if name in a:
            return a[name]
        raise AttributeError(name)

    @property
    def data_vars(self):
        return dict(self._vars)

    @property
    def dims(self):
        out = {}
        for da in list(self._vars.values()) + list(self.coords.values()):
            for n, s in zip(da.dims, da.shape):
                out.setdefault(n, s)
        return out

    def assign_coords(self, coords):
        ds = self.copy(deep=False)
        for k, v in coords.items():
            ds.coords[k] = _as_da(v, k)
        return ds

    def copy(self, deep=True):
        ds = Dataset()
        f = copy.deepcopy if deep else copy.copy
        for k, v in self._vars.items():
            ds._vars[k] = DataArray(f(v.data) if deep else v.data, v.dims, v.attrs)
        for k, v in self.coords.items():
            ds.coords[k] = DataArray(f(v.data) if deep else v.data, v.dims, v.attrs)
        object.__setattr__(ds, 'attrs', f(self.attrs))
        return ds

    def __repr__(self):
        lines = ['<Dataset>', '  coords: ' + ', '.join(self.coords), '  data_vars:']
        lines += [f'    {k}: {v.dims} {v.shape} {v.dtype}' for k, v in self._vars.items()]
        return '\n'.join(lines)


def _as_da(v, name):
    if isinstance(v, DataArray):
        return v
    if hasattr(v, 'dims') and hasattr(v, 'data'):   # an xarray DataArray
        return DataArray(v.data, v.dims, getattr(v, 'attrs', None))
    if isinstance(v, tuple) and len(v) == 2:
        dims, data = v
        dims = (dims,) if isinstance(dims, str) else dims
        return DataArray(np.asarray(data) if not hasattr(data, 'shape') else data, dims)
    arr = np.asarray(v)
    return DataArray(arr, (name,) if arr.ndim == 1 else tuple(f'{name}_{i}' for i in range(arr.ndim)))


def set_var(ds, name, data, dims):
    """Assign a data variable on either this container or an xarray Dataset."""
    if isinstance(ds, Dataset):
        ds[name] = DataArray(data, dims)
    else:
        import xarray as xr
        ds[name] = xr.DataArray(data, dims=dims)


def vis_dataset(uvw, vis, weight, freq, pol=(5, 8), chan_width=None, time=None, flag=None, field_id=None,
                antenna1=None, antenna2=None):
    """Build a visibility dataset with the variable names of a converted MS
    (DATA, UVW, DATA_WEIGHT, FLAG) and one data group."""
    T, B, C, P = np.shape(weight)
    coords = {'chan': ('chan', np.asarray(freq, dtype=np.float64)), 'pol': ('pol', np.asarray(pol)[:P]),
              'time': ('time', np.arange(T, dtype=np.float64) if time is None else np.asarray(time)),
              'baseline': ('baseline', np.arange(B))}
    dv = {'UVW': (('time', 'baseline', 'uvw_index'), uvw),
          'DATA_WEIGHT': (('time', 'baseline', 'chan', 'pol'), weight),
          'chan_width': (('chan',), np.full(C, 1.0) if chan_width is None else np.asarray(chan_width))}
    if vis is not None:
        dv['DATA'] = (('time', 'baseline', 'chan', 'pol'), vis)
    if flag is not None:
        dv['FLAG'] = (('time', 'baseline', 'chan', 'pol'), flag)
    if field_id is not None:
        dv['FIELD_ID'] = (('time', 'baseline'), field_id)
    if antenna1 is not None:
        dv['ANTENNA1'] = (('baseline',), antenna1)
        dv['ANTENNA2'] = (('baseline',), antenna2)
    ds = Dataset(dv, coords)
    grp = {'id': '0', 'uvw': 'UVW', 'weight': 'DATA_WEIGHT'}
    if vis is not None:
        grp['data'] = 'DATA'
    if flag is not None:
        grp['flag'] = 'FLAG'
    ds.attrs['data_groups'] = [{'0': grp}]
    return ds


def mxds(vis_datasets, **attrs):
    """A multi-dataset whose attrs map names ('xds0', ...) to visibility datasets."""
    m = Dataset(attrs=dict(attrs))
    for k, v in vis_datasets.items():
        m.attrs[k] = v
    return m
