"""GB300 implementation of ngcasa.deconvolution's point-source CLEAN."""
from .deconvolve_point_clean import deconvolve_point_clean
