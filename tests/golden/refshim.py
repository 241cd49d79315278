"""Load the reference's hot-path modules without numba, dask or xarray.

Used only by ``make_golden.py`` in a container where the reference checkout is
present; it is never imported by the tests. It installs an identity
``numba.jit`` shim and the removed numpy aliases (np.int/np.bool/np.complex)
and registers stub parent packages whose ``__path__`` points into the
reference tree, so that the leaf modules (pure numpy once ``jit`` is the
identity) import without running the package ``__init__`` files that need
xarray.
"""
import contextlib
import os
import sys
import types

def _reference_root():
    root = os.environ.get('CNGI_REFERENCE_ROOT')
    if not root:
        raise RuntimeError('set CNGI_REFERENCE_ROOT to the root of a cngi_prototype checkout '
                           '(the directory holding ngcasa/ and cngi/)')
    if not os.path.isdir(os.path.join(root, 'ngcasa')):
        raise RuntimeError(f'CNGI_REFERENCE_ROOT={root!r} holds no ngcasa/ package')
    return root


def install():
    import scipy.special  # noqa: F401  (import before the numpy aliases)
    import numpy as np
    if 'numba' not in sys.modules:
        nb = types.ModuleType('numba')

        def jit(*args, **kwargs):
            if len(args) == 1 and callable(args[0]) and not kwargs:
                return args[0]
            return lambda f: f

        nb.jit = jit
        nb.njit = jit
        nb.objmode = lambda *a, **k: contextlib.nullcontext()
        nb.f8 = float
        nb.double = float
        sys.modules['numba'] = nb
    np.int = int
    np.bool = np.bool_
    np.complex = complex
    for name, rel in [('ngcasa', 'ngcasa'), ('ngcasa.imaging', 'ngcasa/imaging'),
                      ('ngcasa.imaging._imaging_utils', 'ngcasa/imaging/_imaging_utils'),
                      ('cngi', 'cngi'), ('cngi._utils', 'cngi/_utils'), ('cngi.image', 'cngi/image')]:
        if name not in sys.modules:
            m = types.ModuleType(name)
            m.__path__ = [os.path.join(_reference_root(), rel)]
            sys.modules[name] = m


def modules():
    install()
    import importlib
    names = {
        'sg': 'ngcasa.imaging._imaging_utils._standard_grid',
        'gck': 'ngcasa.imaging._imaging_utils._gridding_convolutional_kernels',
        'ag': 'ngcasa.imaging._imaging_utils._aperture_grid',
        'pb': 'ngcasa.imaging._imaging_utils._make_pb_symmetric',
        'rp': 'ngcasa.imaging._imaging_utils._remove_padding',
        'cp': 'ngcasa.imaging._imaging_utils._check_imaging_parms',
        'gcf': 'ngcasa.imaging.make_gridding_convolution_function',
        'sic': 'ngcasa.imaging.synthesis_imaging_cube',
    }
    return types.SimpleNamespace(**{k: importlib.import_module(v) for k, v in names.items()})
