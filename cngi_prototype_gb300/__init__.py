"""GB300-native (sm_103a) ngcasa imaging hot path: convolutional gridding with the
prolate-spheroidal kernel, imaging weights, FFT and gridding correction, behind
the ngcasa.imaging API. Kernels live in libngg.so (C ABI: include/ngg.h)."""
__version__ = '0.1.0'
