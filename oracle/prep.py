"""ORACLE — CPU restatement of the reference's image preparation (test
infrastructure only; nothing in the product imports it).

CropAndDownscale (Python/openSSS/Utils.py:212-267) crops or zero-pads a
window about the volume centre, then calls skimage.transform.resize with
order=3, mode='edge', clip=True, preserve_range=True, anti_aliasing=True.
scikit-image is not installed here, so resize is restated from its published
algorithm (scikit-image 0.19 and later, skimage/transform/_warps.py):
  * factors = input shape / output shape;
  * anti-aliasing: scipy.ndimage.gaussian_filter with sigma = max(0,
    (factors - 1) / 2) and mode 'nearest' (skimage's 'edge');
  * scipy.ndimage.zoom(order=3, mode='nearest', grid_mode=True) by 1 / factors;
  * clip to the [min, max] of resize's input.
The crop window is pinned against the reference's own CropAndDownscale run with
an identity resize (tests/golden/prep.npz); the resize glue above is not pinned
against scikit-image itself ("parity unpinned" for that part), only against the
scipy.ndimage routines it calls, which are the installed SciPy.
"""

from __future__ import annotations

import numpy as np
from scipy import ndimage as ndi


def crop(image, voxel_size, crop_size):
    """The window of Utils.py:238-260: numpy slicing (negative starts follow
    Python's rules) or a symmetric zero pad when the window overhangs both ends."""
    half = np.ceil(np.array(crop_size) / np.array(voxel_size) / 2).astype(int)
    center = np.array(image.shape) // 2
    out = image
    for dim in range(3):
        lo, hi = center[dim] - half[dim], center[dim] + half[dim]
        if lo < 0 and hi > image.shape[dim]:
            widths = [(0, 0)] * 3
            p = int(half[dim] - center[dim])
            widths[dim] = (p, p)
            out = np.pad(out, widths, mode="constant", constant_values=0)
        else:
            sl = [slice(None)] * 3
            sl[dim] = slice(int(lo), int(hi))
            out = out[tuple(sl)]
    return out


def resize(image, output_shape, order=3, mode="edge", clip=True, preserve_range=True, anti_aliasing=True):
    """skimage.transform.resize for the options CropAndDownscale uses."""
    assert order == 3 and mode == "edge" and preserve_range
    image = np.asarray(image)
    if image.dtype not in (np.float32, np.float64):
        image = image.astype(np.float64)
    factors = np.asarray(image.shape, dtype=float) / np.asarray(output_shape, dtype=float)
    filtered = image
    if anti_aliasing:
        sigma = np.maximum(0.0, (factors - 1.0) / 2.0)
        filtered = ndi.gaussian_filter(image, sigma, cval=0.0, mode="nearest")
    out = ndi.zoom(filtered, 1.0 / factors, order=order, mode="nearest", cval=0.0, grid_mode=True)
    if clip:
        np.clip(out, image.min(), image.max(), out=out)
    return out


def crop_and_downscale(image, voxel_size, crop_size, dims, anti_aliasing=True, clip=True):
    return resize(crop(image, voxel_size, crop_size), tuple(int(d) for d in dims), anti_aliasing=anti_aliasing,
                  clip=clip)
