"""GB300 implementation of the ngcasa.imaging hot path (same function names and parameters)."""
from .make_image import make_image, make_psf
from .make_imaging_weight import make_imaging_weight
