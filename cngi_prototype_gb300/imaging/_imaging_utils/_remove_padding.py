"""Centre crop of a padded image (ngcasa/imaging/_imaging_utils/_remove_padding.py:20-31)."""
import numpy as np


def _remove_padding(image, image_size):
    image_size = np.asarray(image_size)
    padded = np.array(image.shape[0:2])
    start = padded // 2 - image_size // 2
    end = start + image_size
    return image[start[0]:end[0], start[1]:end[1]]
