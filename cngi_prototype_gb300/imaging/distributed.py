"""Multi-process imaging: one process per GPU, one host-side sum.

The reference runs make_imaging_weight / make_psf / make_image as dask graphs
of per-chunk gridders over (time, baseline, chan) blocks whose partial grids
merge by a tree sum (_graph_standard_grid, ngcasa/imaging/_imaging_utils/
_standard_grid.py:23-120). Here each process owns one GPU and one shard of
the visibilities, and the graph reduces to at most one sum per call:

* cube mode -- channels are independent (one density grid per channel,
  make_imaging_weight.py:22-23; one grid per channel, _standard_grid.py:
  45-47): a rank holds a contiguous channel range and images it with no
  exchange at all;
* continuum mode -- every row lands on the one grid, so a rank holds a
  contiguous range of time rows and the ranks add their partial results
  once. The FFT is linear, so the sum is taken after it, on the cropped and
  corrected but not yet weight-normalised image (N0*N1 per pol instead of the
  padded complex grid), together with sum_weight; uniform and Briggs
  weighting first add up the weight-density grid (unpadded, N0*N1 per pol)
  and its weight sum, between the density pass and the lookup pass.

The sums run over torch.distributed. With a gloo group they add host
tensors (TCP between boxes of one GPU each; nothing waits on the device).
With an NCCL group (the GPUs of one node) the weight-density grid, which is
already on the device, is added on the device with no host copy; the
continuum image is added on the host either way, since the API returns it
as a host dataset. A rank that fails can mark itself in a store shared by the group
(ShardGroup.fail); the others see the mark before their next sum
(ShardGroup.check) instead of waiting out the process-group timeout, and
every sum that does not complete raises ShardError.
"""
import datetime

import numpy as np

from ..xds import Dataset, DataArray
from ._imaging_utils import _pipeline
from .make_image import _make
from .make_imaging_weight import _make_imaging_weight

__all__ = ['ShardError', 'ShardGroup', 'shard_range', 'shard_vis', 'make_imaging_weight_sharded',
           'make_psf_sharded', 'make_image_sharded']


class ShardError(RuntimeError):
    """A sum over the ranks did not complete, or a rank reported a failure."""


def shard_range(n, rank, world):
    """Contiguous [lo, hi) of n items for this rank; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f'rank {rank} outside world of {world}')
    base, extra = divmod(int(n), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _slice_ds(ds, axis, lo, hi):
    if not isinstance(ds, Dataset):       # an xarray Dataset
        return ds.isel({axis: slice(lo, hi)})
    out = Dataset(attrs=dict(ds.attrs))
    for name, da in list(ds.data_vars.items()) + [(k, v) for k, v in ds.coords.items()]:
        d = da.data
        if axis in da.dims:
            idx = [slice(None)] * len(da.dims)
            idx[da.dims.index(axis)] = slice(lo, hi)
            d = d[tuple(idx)]
        target = out.coords if name in ds.coords else out._vars
        target[name] = DataArray(d, da.dims, da.attrs)
    return out


def shard_vis(vis_mxds, sel_parms, chan_mode, rank, world):
    """This rank's shard of sel_parms['xds']: a channel range in cube mode, a
    time range in continuum mode. Other attrs of the mxds are shared."""
    axis = 'time' if chan_mode == 'continuum' else 'chan'
    name = sel_parms['xds']
    xds = vis_mxds.attrs[name]
    lo, hi = shard_range(xds.dims[axis], rank, world)
    out = vis_mxds.copy(deep=False)
    out.attrs[name] = _slice_ds(xds, axis, lo, hi)
    return out


class ShardGroup:
    """The ranks that image one observation together.

    group: a torch.distributed process group (default: the world group, or a
    single rank when torch.distributed is not initialised); its timeout bounds
    every sum. store: an optional torch.distributed Store shared by the ranks,
    used for failure marks.
    """

    def __init__(self, group=None, store=None, timeout_s=None):
        import torch.distributed as dist
        self._dist = dist if dist.is_available() and dist.is_initialized() else None
        self.group = group
        self.store = store
        self.timeout = datetime.timedelta(seconds=timeout_s) if timeout_s else None
        self.rank = self._dist.get_rank(group) if self._dist else 0
        self.world = self._dist.get_world_size(group) if self._dist else 1

    def fail(self, message):
        """Mark this rank failed, so the others stop before their next sum."""
        if self.store is not None:
            self.store.set(f'ngg_failed/{self.rank}', str(message)[:1000])

    def check(self):
        """Raise ShardError if any rank of the group has marked itself failed."""
        if self.store is None:
            return
        for r in range(self.world):
            key = f'ngg_failed/{r}'
            if self.store.check([key]):
                raise ShardError(f'rank {r} failed: {self.store.get(key).decode(errors="replace")}')

    def _nccl(self):
        if self.world == 1:
            return False
        try:
            return str(self._dist.get_backend(self.group)).lower() == 'nccl'
        except (RuntimeError, ValueError):
            return False

    def sum(self, arrays):
        """Element-wise sum over the ranks of a list of arrays (numpy or torch,
        any device); returns float64 numpy arrays of the same shapes, or, in
        an NCCL group when every array is a CUDA tensor, float64 CUDA tensors
        (summed on the device)."""
        if self._nccl() and all(getattr(a, 'is_cuda', False) for a in arrays):
            return self._sum_device(arrays)
        vals = [np.asarray(a.detach().cpu().numpy() if hasattr(a, 'detach') else a, dtype=np.float64)
                for a in arrays]
        self.check()
        if self.world == 1:
            return vals
        import torch
        flat = torch.from_numpy(np.concatenate([v.ravel() for v in vals]))
        try:
            work = self._dist.all_reduce(flat, op=self._dist.ReduceOp.SUM, group=self.group, async_op=True)
            if self.timeout is not None:
                work.wait(timeout=self.timeout)
            else:
                work.wait()
        except RuntimeError as e:
            raise ShardError(f'sum over {self.world} ranks failed on rank {self.rank}: {e}') from e
        self.check()
        out, k = [], 0
        flat = flat.numpy()
        for v in vals:
            out.append(flat[k:k + v.size].reshape(v.shape).copy())
            k += v.size
        return out

    def _sum_device(self, arrays):
        import torch
        self.check()
        flat = torch.cat([a.detach().reshape(-1).to(torch.float64) for a in arrays])
        try:
            work = self._dist.all_reduce(flat, op=self._dist.ReduceOp.SUM, group=self.group, async_op=True)
            if self.timeout is not None:
                work.wait(timeout=self.timeout)
            else:
                work.wait()
            torch.cuda.current_stream(flat.device).synchronize()
        except RuntimeError as e:
            raise ShardError(f'sum over {self.world} ranks failed on rank {self.rank}: {e}') from e
        self.check()
        out, k = [], 0
        for a in arrays:
            n = a.numel()
            out.append(flat[k:k + n].reshape(a.shape))
            k += n
        return out


def _chan_mode(grid_parms):
    return grid_parms.get('chan_mode', 'cube')


def make_imaging_weight_sharded(vis_mxds, imaging_weights_parms, grid_parms, sel_parms, group=None):
    """make_imaging_weight on this rank's shard (shard_vis). Continuum uniform
    or Briggs weighting sums the weight-density grid over the ranks; every
    other case is local."""
    g = group or ShardGroup()
    if _chan_mode(grid_parms) == 'cube' or imaging_weights_parms.get('weighting') == 'natural' or g.world == 1:
        return _make_imaging_weight(vis_mxds, imaging_weights_parms, grid_parms, sel_parms)

    def reduce(dens, dsw):
        import torch
        d, s = g.sum([dens, dsw])
        return (torch.as_tensor(d, dtype=dens.dtype, device=dens.device),
                torch.as_tensor(s, dtype=dsw.dtype, device=dsw.device))
    return _make_imaging_weight(vis_mxds, imaging_weights_parms, grid_parms, sel_parms, density_reduce=reduce)


def _make_sharded(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, do_psf, group):
    g = group or ShardGroup()
    if _chan_mode(grid_parms) == 'cube' or g.world == 1:
        return _make(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, do_psf)

    def cube_fn(vis, uvw, iw, freq, gp, psf):
        part, sw = _pipeline.image_cube(vis, uvw, iw, freq, gp, psf, normalize=False)
        tot, sw = g.sum([part, sw])
        return tot / np.where(sw == 0, 1.0, sw)[None, None], sw
    out = _make(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, do_psf, cube_fn=cube_fn)
    # the image's time coordinate is the mean over all ranks' rows
    t = np.asarray(vis_mxds.attrs[vis_sel_parms['xds']].coords['time'].values, dtype=np.float64)
    s, n = g.sum([np.array([t.sum()]), np.array([float(t.size)])])
    return out.assign_coords({'time': ('time', np.array([s[0] / max(n[0], 1.0)]))})


def make_psf_sharded(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, group=None):
    """make_psf on this rank's shard; continuum mode sums over the ranks and
    every rank returns the full PSF."""
    return _make_sharded(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, True, group)


def make_image_sharded(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, group=None):
    """make_image on this rank's shard; cube mode returns this rank's channels,
    continuum mode sums over the ranks and every rank returns the full image."""
    return _make_sharded(vis_mxds, img_xds, grid_parms, vis_sel_parms, img_sel_parms, False, group)
