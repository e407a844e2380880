"""Drop-in image preparation: ``PrepareImages`` / ``CropAndDownscale`` with the
reference's arguments and results, the resize running on the GPU.

Reference: ``Python/openSSS/Utils.py`` — ``PrepareImages`` (:30-74),
``ComputePhisicalDimensions`` (:76-109), ``LoadImage`` (:111-145) and
``CropAndDownscale`` (:212-267).  ``CropAndDownscale`` crops (or zero-pads)
a window about the volume centre with numpy's slicing rules, then calls
``skimage.transform.resize(order=3, mode='edge', anti_aliasing=True,
preserve_range=True, clip=True)``.  Here the window is worked out on the host
(``crop_window``) and the whole resize — anti-aliasing Gaussian, cubic B-spline
coefficients and their sampling, clipping — is one ``sss_crop_downscale`` call.
Only the reference's default resize options are built; others raise
``NotImplementedError`` (there is no CPU fallback).
"""

from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import torch

from . import _lib


def crop_window(shape, voxel_size, crop_size):
    """Per axis (start, before, length) of CropAndDownscale's window
    (Utils.py:238-260): the window holds image[i - before + start] for
    i < length, zeros outside the image.  An axis whose window would start
    before 0 and end past the image is zero-padded symmetrically; otherwise it
    is sliced with Python's rules for a possibly negative start."""
    half = np.ceil(np.array(crop_size) / np.array(voxel_size) / 2).astype(int)
    center = np.array(shape) // 2
    win = []
    for d in range(3):
        lo = int(center[d] - half[d])
        hi = int(center[d] + half[d])
        n = int(shape[d])
        if lo < 0 and hi > n:
            pad = int(half[d] - center[d])
            win.append((0, pad, n + 2 * pad))
        else:
            s, e, _ = slice(lo, hi).indices(n)
            win.append((s, 0, max(0, e - s)))
    return win


def antialias_sigma(crop_dims, out_dims):
    """resize's anti-aliasing sigma per axis: max(0, (in/out - 1) / 2)."""
    f = np.asarray(crop_dims, dtype=np.float64) / np.asarray(out_dims, dtype=np.float64)
    return np.maximum(0.0, (f - 1.0) / 2.0)


def crop_downscale_device(image: torch.Tensor, window, out_dims, anti_aliasing: bool = True,
                          clip: bool = True, zero_below: float = -np.inf) -> torch.Tensor:
    """The GPU call: image float32 [n0][n1][n2] on the device, window from
    ``crop_window``; returns float32 ``out_dims`` on the same device."""
    if not image.is_cuda:
        raise ValueError("crop_downscale_device needs a CUDA tensor")
    dev = image.device
    img = image.to(torch.float32).contiguous()
    dims = np.array(img.shape, dtype=np.int32)
    start = np.array([w[0] for w in window], dtype=np.int32)
    before = np.array([w[1] for w in window], dtype=np.int32)
    cdims = np.array([w[2] for w in window], dtype=np.int32)
    odims = np.array([int(v) for v in out_dims], dtype=np.int32)
    if np.any(cdims < 1):
        raise ValueError(f"empty crop window {tuple(cdims)}")
    if np.any(odims < 1):
        raise ValueError(f"output shape {tuple(odims)} has an empty axis")
    sigma = antialias_sigma(cdims, odims) if anti_aliasing else np.zeros(3)
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    L = _lib.lib()
    wsb = L.sss_crop_downscale_workspace_size(cdims.ctypes.data_as(C.c_void_p))
    ws = torch.empty(int(wsb), dtype=torch.uint8, device=dev)
    out = torch.empty(tuple(int(v) for v in odims), dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)

    def p(a):
        return a.ctypes.data_as(C.c_void_p)

    _lib.check(L.sss_crop_downscale(C.c_void_p(img.data_ptr()), p(dims), p(start), p(before), p(cdims), p(odims),
                                    p(sigma), int(bool(clip)), C.c_float(zero_below), C.c_void_p(out.data_ptr()),
                                    C.c_void_p(ws.data_ptr()), wsb, C.c_void_p(st.cuda_stream)))
    return out


def CropAndDownscale(image, voxel_size, crop_size, downscaled_dimensions, clip: bool = True, mode: str = "edge",
                     preserve_range: bool = True, anti_aliasing: bool = True, order: int = 3):
    """Utils.py:212-267 on the GPU.  A numpy image gives a numpy float32
    result; a CUDA tensor gives a CUDA tensor."""
    if mode != "edge" or order != 3 or not preserve_range:
        raise NotImplementedError("only resize(order=3, mode='edge', preserve_range=True) is built on the GPU")
    as_numpy = not isinstance(image, torch.Tensor)
    if not as_numpy and not image.is_cuda:
        raise ValueError("CropAndDownscale takes a numpy array or a CUDA tensor")
    t = torch.from_numpy(np.ascontiguousarray(image, dtype=np.float32)).cuda() if as_numpy else image
    if t.dim() != 3:
        raise ValueError("CropAndDownscale expects a 3-D volume")
    win = crop_window(tuple(t.shape), voxel_size, crop_size)
    out = crop_downscale_device(t, win, downscaled_dimensions, anti_aliasing=anti_aliasing, clip=clip)
    return out.cpu().numpy() if as_numpy else out


def LoadImage(Filename: str):
    """Utils.py:111-145: an interfile header (matrix size and mm/pixel per axis,
    name of the float32 data file beside it) -> (image [x][y][z], size, scale)."""
    with open(Filename) as f:
        header = f.read()
    scale = np.zeros(3, dtype=float)
    size = np.zeros(3, dtype=int)
    for i in range(3):
        size[i] = int(re.findall(rf".*matrix size \[{i + 1}\] := (\d*).*", header)[0])
        scale[i] = float(re.findall(rf".*scaling factor \(mm/pixel\) \[{i + 1}\] := (\d*\.*\d+).*", header)[0])
    datafile = re.findall(r".*name of data file := (\S*).*", header)[0]
    raw = np.fromfile(os.path.dirname(Filename) + f"/{datafile}", dtype=np.float32)
    image = raw.reshape(size[2], size[1], size[0]).transpose((2, 1, 0))
    return image, size, scale


def desired_size(SizeDesired, ScaleDesired, dims, scale):
    """PrepareImages' target (Utils.py:56-62): None entries of SizeDesired (mm)
    become the map's extent, written into the caller's list; the voxel counts
    are SizeDesired // ScaleDesired and the size is rounded down to them.
    Returns (SizeDesired, DimsDesired)."""
    for i, dim in enumerate(SizeDesired):
        if dim is None:
            SizeDesired[i] = dims[i] * scale[i]
    DimsDesired = (SizeDesired // ScaleDesired).astype(int)
    return DimsDesired * ScaleDesired, DimsDesired


def PrepareImages(ActivityFilename: str, AttenuationFilename: str, SizeDesired, ScaleDesired):
    """Utils.py:30-74: both maps cropped to SizeDesired (mm; None entries take
    the activity map's extent, filled into the caller's list as the reference
    does) and resized to SizeDesired // ScaleDesired voxels; attenuation below
    0.001 set to 0.  Returns (activity, attenuation, SizeDesired, DimsDesired)."""
    activity, dims_act, size_act = LoadImage(ActivityFilename)
    attenuation, _, size_atn = LoadImage(AttenuationFilename)
    SizeDesired, DimsDesired = desired_size(SizeDesired, ScaleDesired, dims_act, size_act)
    act = CropAndDownscale(activity, size_act, SizeDesired, DimsDesired)
    t = torch.from_numpy(np.ascontiguousarray(attenuation, dtype=np.float32)).cuda()
    win = crop_window(tuple(t.shape), size_atn, SizeDesired)
    atn = crop_downscale_device(t, win, DimsDesired, zero_below=0.001).cpu().numpy()
    return act, atn, SizeDesired, DimsDesired


def ComputePhisicalDimensions(DesiredSize, DeviceSize):
    """Utils.py:76-109: image and fitting bounds [x0, y0, z0, x1, y1, z1] in cm
    from the desired map size and the scanner size (mm)."""
    image_size = np.array([-DesiredSize[0] / 2, -DesiredSize[1] / 2, -DesiredSize[2] / 2,
                           DesiredSize[0] / 2, DesiredSize[1] / 2, DesiredSize[2] / 2]) / 10
    fitting_size = np.array([-DesiredSize[0] / 2, -DesiredSize[1] / 2, -DeviceSize[2] / 2,
                             DesiredSize[0] / 2, DesiredSize[1] / 2, DeviceSize[2] / 2]) / 10
    return image_size, fitting_size
