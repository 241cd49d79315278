"""GB300 implementation of the ngcasa.imaging hot path (same function names and parameters)."""
from .direction_rotate import direction_rotate
from .make_gridding_convolution_function import make_gridding_convolution_function
from .make_grid import make_grid
from .make_image import make_image, make_psf
from .make_image_with_gcf import make_image_with_gcf, make_psf_with_gcf
from .make_imaging_weight import make_imaging_weight
from .make_mosaic_pb import make_mosaic_pb
from .distributed import make_image_sharded, make_imaging_weight_sharded, make_psf_sharded, shard_vis, ShardGroup
from .predict_modelvis_image import predict_modelvis_image
from .synthesis_imaging_cube import synthesis_imaging_cube
