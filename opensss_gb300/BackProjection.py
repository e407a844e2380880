"""Drop-in ``BackProjectionScatterRandFit``: the tail-fit scale factor on the GPU.

Same arguments and result as the reference (``Python/openSSS/BackProjection.py:115-215``):
a float32 array of shape (1,).  ``fit_device`` is the engine form: it reads
the scatter value of every LOR through gather tables, so the upsampled
scatter sinogram never has to exist.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import DataReduction, _lib
from .engine import as_device


def _ptr(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def fit_device(prompts, randoms, mask, scatters, scat_cell, scat_ring, GridSize, ImageSize, Geometry,
               SinogramCoordinates, SinogramOrder, AccelerationFactor, scat_clamp=False,
               device="cuda", span: bool = False):
    """All sinogram arguments are CUDA tensors [cell, slice] (float32; mask
    float32, or uint8 meaning mask >= 1).  Returns the scale as a float.
    With ``span``, ``Geometry`` is the expanded geometry, ``SinogramOrder`` the
    mashed SinogramIndex (float [n, 2]) and the back-projection is
    length-weighted (BackProjection.py:217-393)."""
    _lib.require_cuda(prompts=prompts, randoms=randoms, mask=mask, scatters=scatters)
    geom = np.asarray(Geometry, dtype=np.float64)
    nr, nd = geom.shape[:2]
    grid = np.ascontiguousarray(np.asarray(GridSize).reshape(-1)[:3], dtype=np.int32)
    bounds = np.ascontiguousarray(np.asarray(ImageSize, dtype=np.float64).reshape(-1)[:6])
    g = as_device(geom, torch.float64, device)
    lor = as_device(np.asarray(SinogramCoordinates, dtype=np.int16), torch.int16, device)
    if span:
        pairs_np = DataReduction.span_ring_pairs(SinogramOrder)
        pairs = as_device(pairs_np, torch.int32, device)
    else:
        order = as_device(np.asarray(SinogramOrder, dtype=np.int16)[:nr, :nr], torch.int16, device)
    cs = as_device(scat_cell, torch.int64, device)
    rs = as_device(scat_ring, torch.int64, device)
    nvox = int(np.prod(grid))
    images = torch.empty(8 * nvox, dtype=torch.float32, device=device)
    sums = torch.empty(2, dtype=torch.float64, device=device)
    scale = torch.empty(1, dtype=torch.float32, device=device)
    status = torch.zeros(1, dtype=torch.int32, device=device)
    m_u8 = mask if mask.dtype == torch.uint8 else None
    m_f = None if m_u8 is not None else mask
    st = torch.cuda.current_stream(device)
    if span:
        n = pairs_np.shape[0]
        _lib.check(_lib.lib().sss_backproject_fit_pairs(
            grid.ctypes.data_as(C.c_void_p), bounds.ctypes.data_as(C.c_void_p), nr, nd, _ptr(g), _ptr(lor),
            _ptr(pairs), n, n, 1, int(AccelerationFactor or 1), _ptr(prompts), _ptr(randoms), _ptr(m_f),
            _ptr(m_u8), _ptr(scatters), _ptr(cs), _ptr(rs), int(bool(scat_clamp)), _ptr(images), _ptr(sums),
            _ptr(scale), _ptr(status), C.c_void_p(st.cuda_stream)))
    else:
        _lib.check(_lib.lib().sss_backproject_fit(
            grid.ctypes.data_as(C.c_void_p), bounds.ctypes.data_as(C.c_void_p), nr, nd, _ptr(g), _ptr(lor),
            _ptr(order), int(AccelerationFactor or 1), _ptr(prompts), _ptr(randoms), _ptr(m_f), _ptr(m_u8),
            _ptr(scatters), _ptr(cs), _ptr(rs), int(bool(scat_clamp)), _ptr(images), _ptr(sums),
            _ptr(scale), _ptr(status), C.c_void_p(st.cuda_stream)))
    st.synchronize()
    _lib.check_status(int(status.item()))
    return float(scale.item())


def fit_bins_device(prompts, randoms, mask, scatters, scat_stride: int, scat_cell, scat_ring, GridSize,
                    ImageSize, Geometry, SinogramCoordinates, SinogramOrder, AccelerationFactor,
                    scat_clamp=False, device="cuda", span: bool = False) -> np.ndarray:
    """Scales of all TOF bins in one pass (``sss_backproject_fit_bins``).
    prompts: CUDA float32 [bins, cell, slice]; scatters: CUDA float32 with
    bin b's values from ``b * scat_stride`` (through the gather tables);
    randoms / mask as in ``fit_device``.  Returns float32 [bins]."""
    _lib.require_cuda(prompts=prompts, randoms=randoms, mask=mask, scatters=scatters)
    geom = np.asarray(Geometry, dtype=np.float64)
    nr, nd = geom.shape[:2]
    nbins = int(prompts.shape[0])
    grid = np.ascontiguousarray(np.asarray(GridSize).reshape(-1)[:3], dtype=np.int32)
    bounds = np.ascontiguousarray(np.asarray(ImageSize, dtype=np.float64).reshape(-1)[:6])
    g = as_device(geom, torch.float64, device)
    lor = as_device(np.asarray(SinogramCoordinates, dtype=np.int16), torch.int16, device)
    order = pairs = None
    npairs = nslices = 0
    if span:
        pairs_np = DataReduction.span_ring_pairs(SinogramOrder)
        pairs = as_device(pairs_np, torch.int32, device)
        npairs = nslices = pairs_np.shape[0]
    else:
        order = as_device(np.asarray(SinogramOrder, dtype=np.int16)[:nr, :nr], torch.int16, device)
    cs = as_device(scat_cell, torch.int64, device)
    rs = as_device(scat_ring, torch.int64, device)
    nvox = int(np.prod(grid))
    images = torch.empty((nbins + 1) * 4 * nvox, dtype=torch.float32, device=device)
    sums = torch.empty(2 * nbins, dtype=torch.float64, device=device)
    scales = torch.empty(nbins, dtype=torch.float32, device=device)
    status = torch.zeros(1, dtype=torch.int32, device=device)
    m_u8 = mask if mask.dtype == torch.uint8 else None
    m_f = None if m_u8 is not None else mask
    st = torch.cuda.current_stream(device)
    stride = int(prompts[0].numel())
    _lib.check(_lib.lib().sss_backproject_fit_bins(
        grid.ctypes.data_as(C.c_void_p), bounds.ctypes.data_as(C.c_void_p), nr, nd, _ptr(g), _ptr(lor),
        _ptr(order), _ptr(pairs), npairs, nslices, int(bool(span)), int(AccelerationFactor or 1), nbins,
        _ptr(prompts), stride, _ptr(randoms), _ptr(m_f), _ptr(m_u8), _ptr(scatters), int(scat_stride), _ptr(cs),
        _ptr(rs), int(bool(scat_clamp)), _ptr(images), _ptr(sums), _ptr(scales), _ptr(status),
        C.c_void_p(st.cuda_stream)))
    st.synchronize()
    _lib.check_status(int(status.item()))
    return scales.cpu().numpy()


def BackProjectionScatterRandFit(PromptSinogram, ScatterSinogram, RandomSinogram, MaskSinogram,
                                 GridSize, ImageSize, Geometry, SinogramCoordinates, SinogramOrder,
                                 AccelerationFactor, device="cuda"):
    if not torch.cuda.is_available():
        raise _lib.EngineUnavailable("no CUDA device: the engine has no CPU path")
    geom = np.asarray(Geometry)
    nr, nd = geom.shape[:2]
    shp = ((nd + 1) * (nd // 2), nr * nr)

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(shp))
                                ).to(device)

    ncell = shp[0]
    cell = np.arange(ncell, dtype=np.int64) * (nr * nr)
    ring = np.arange(nr * nr, dtype=np.int64)
    s = fit_device(dev(PromptSinogram), dev(RandomSinogram), dev(MaskSinogram), dev(ScatterSinogram),
                   cell, ring, GridSize, ImageSize, Geometry, SinogramCoordinates, SinogramOrder,
                   AccelerationFactor, device=device)
    return np.array([s], dtype=np.float32)


def BackProjectionScatterRandFitMashing(PromptSinogram, ScatterSinogram, RandomSinogram, MaskSinogram,
                                        GridSize, ImageSize, Geometry, SinogramCoordinates, AccelerationFactor,
                                        MashedSinogramIndices, device="cuda"):
    """Scale fit with span (``BackProjection.py:302-393``): ``Geometry`` is
    the expanded geometry; sinograms are (ND+1, ND//2, mashed sinograms)."""
    if not torch.cuda.is_available():
        raise _lib.EngineUnavailable("no CUDA device: the engine has no CPU path")
    geom = np.asarray(Geometry)
    nd = geom.shape[1]
    nsl = np.asarray(MashedSinogramIndices).shape[0]
    shp = ((nd + 1) * (nd // 2), nsl)

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(shp))
                                ).to(device)

    cell = np.arange(shp[0], dtype=np.int64) * nsl
    ring = np.arange(nsl, dtype=np.int64)
    s = fit_device(dev(PromptSinogram), dev(RandomSinogram), dev(MaskSinogram), dev(ScatterSinogram),
                   cell, ring, GridSize, ImageSize, Geometry, SinogramCoordinates, MashedSinogramIndices,
                   AccelerationFactor, device=device, span=True)
    return np.array([s], dtype=np.float32)
