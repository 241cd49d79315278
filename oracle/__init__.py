"""CPU oracle for the ngcasa standard-gridder imaging path.

This package is TEST INFRASTRUCTURE. It restates, on the CPU in FP64, the
algorithm of the reference's hot path (ngcasa/imaging/_imaging_utils/
_standard_grid.py, _gridding_convolutional_kernels.py, _aperture_grid.py,
make_imaging_weight.py, make_image.py, make_psf.py, _normalize.py) so that the
CUDA path of ``cngi_prototype_gb300`` can be checked against it.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import or execute anything in
this package, and only as the checker or as the timed CPU baseline. The
product path (``cngi_prototype_gb300``) never imports it.

Two restatements live here:

* ``oracle.imaging`` -- numpy, summation order identical to the reference's
  loop nest (time, baseline, chan, pol, v-tap, u-tap), so that small cases are
  bit-identical to the reference run through a numba shim (the golden
  fixtures under ``tests/golden`` pin this).
* ``oracle/ngg_oracle.c`` -- the same loop nests in C (FP64, complex128
  grid), OpenMP-parallel over channels in cube mode, used for the large
  configurations and as the timed CPU baseline.
"""
