"""Drop-in ``GenerateTailsMask`` / ``MaskGenerator``: the tail mask on the GPU.

Same arguments and result as the reference (``Python/openSSS/TailsMask.py:28-82,165-228``):
uint8 ``(ND+1, ND//2, NR**2)``, 1 where the LOR's attenuation correction
factor is exactly 1 (or, with ``UseAttenuation=False``, where it sees no
activity), for the LORs on the AccelerationFactor lattice.  With span
(``MaskGeneratorMashing``, :230-377) the slices are the mashed sinograms,
each traced once at its mean ring pair on the expanded geometry.
"""

from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np
import torch

from . import DataReduction, _lib, geometry
from .engine import as_device, fortran_flat


def _ptr(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def tail_mask_device(volume, ImageSize, Geometry, SinogramCoordinates, SinogramIndex,
                     AccelerationFactor=1, use_activity=False, device="cuda", span: bool = False,
                     acf_below: float | None = None) -> torch.Tensor:
    """uint8 CUDA tensor [(ND+1)*(ND//2), slices]: NR*NR slices, or with
    ``span`` the mashed sinograms of ``SinogramIndex`` (float [n, 2], from
    SinogramLUT) on the expanded ``Geometry``.  ``acf_below`` None keeps the
    reference's rule (attenuation factor exactly 1); a bound above 1 marks the
    LORs whose factor 1/exp(-sum mu*len) is below it instead."""
    acf = 0.0 if acf_below is None else float(acf_below)
    if not (acf == 0.0 or acf > 1.0):
        raise ValueError("acf_below must be None or above 1")
    if not torch.cuda.is_available():
        raise _lib.EngineUnavailable("no CUDA device: the engine has no CPU path")
    geom = np.asarray(Geometry, dtype=np.float64)
    nr, nd = geom.shape[:2]
    shape = tuple(int(s) for s in volume.shape)
    vol = fortran_flat(volume, device)
    g = as_device(geom, torch.float64, device)
    lor = as_device(np.asarray(SinogramCoordinates, dtype=np.int16), torch.int16, device)
    status = torch.zeros(1, dtype=torch.int32, device=device)
    grid = np.array(shape, dtype=np.int32)
    bounds = np.ascontiguousarray(np.asarray(ImageSize, dtype=np.float64).reshape(-1)[:6])
    st = torch.cuda.current_stream(device)
    if span:
        pairs_np = DataReduction.span_ring_pairs(SinogramIndex)
        nslices = pairs_np.shape[0]
        pairs = as_device(pairs_np, torch.int32, device)
        out = torch.zeros(((nd + 1) * (nd // 2), nslices), dtype=torch.uint8, device=device)
        _lib.check(_lib.lib().sss_tail_mask_pairs(
            grid.ctypes.data_as(C.c_void_p), bounds.ctypes.data_as(C.c_void_p), _ptr(vol),
            int(bool(use_activity)), nr, nd, _ptr(g), _ptr(lor), _ptr(pairs), nslices, nslices,
            int(AccelerationFactor or 1), acf, _ptr(out), _ptr(status), C.c_void_p(st.cuda_stream)))
    else:
        si = as_device(geometry.check_slice_table(SinogramIndex, nr).astype(np.int16), torch.int16, device)
        out = torch.zeros(((nd + 1) * (nd // 2), nr * nr), dtype=torch.uint8, device=device)
        _lib.check(_lib.lib().sss_tail_mask(grid.ctypes.data_as(C.c_void_p),
                                            bounds.ctypes.data_as(C.c_void_p), _ptr(vol),
                                            int(bool(use_activity)), nr, nd, _ptr(g), _ptr(lor), _ptr(si),
                                            int(AccelerationFactor or 1), acf, _ptr(out), _ptr(status),
                                            C.c_void_p(st.cuda_stream)))
    st.synchronize()
    _lib.check_status(int(status.item()))
    return out


def MaskGenerator(ActivityMap, AttenuationMap, ImageSize, Geometry, SinogramCoordinates,
                  SinogramIndex, UseAttenuation, AccelerationFactor=1, device="cuda", AttenuationThreshold=None):
    """``AttenuationThreshold`` (no reference counterpart): None keeps the
    reference's tails (attenuation factor exactly 1); a value above 1 marks
    the LORs whose attenuation factor lies below it, e.g. 1.03."""
    t0 = time.time()
    geom = np.asarray(Geometry)
    nr, nd = geom.shape[:2]
    vol = AttenuationMap if UseAttenuation else ActivityMap
    m = tail_mask_device(vol, ImageSize, geom, SinogramCoordinates, SinogramIndex,
                         AccelerationFactor, use_activity=not UseAttenuation, device=device,
                         acf_below=AttenuationThreshold)
    print("Time for Generate Tail Mask:", time.time() - t0, "seconds")
    return m.cpu().numpy().reshape(nd + 1, nd // 2, nr * nr)


def MaskGeneratorMashing(ActivityMap, AttenuationMap, ImageSize, Geometry, SinogramCoordinates,
                         MashedSinogramIndices, UseAttenuation, AccelerationFactor=1, device="cuda",
                         AttenuationThreshold=None):
    """Tail mask with span (``TailsMask.py:311-377``): ``Geometry`` is the
    expanded geometry and ``MashedSinogramIndices`` the mashed SinogramIndex
    of SinogramLUT.  uint8 (ND+1, ND//2, mashed sinograms)."""
    t0 = time.time()
    geom = np.asarray(Geometry)
    nd = geom.shape[1]
    vol = AttenuationMap if UseAttenuation else ActivityMap
    m = tail_mask_device(vol, ImageSize, geom, SinogramCoordinates, MashedSinogramIndices,
                         AccelerationFactor, use_activity=not UseAttenuation, device=device, span=True,
                         acf_below=AttenuationThreshold)
    print("Time for Generate Tail Mask:", time.time() - t0, "seconds")
    return m.cpu().numpy().reshape(nd + 1, nd // 2, -1)


def GenerateTailsMask(SavePath, ActivityMapDownscaled, AttenuationMapDownscaled, ImageSize, Geometry,
                      extendedGeometry, LORCoordinates, SinogramIndex, AccelerationFactor,
                      UseAttenuation=True, Overwrite=False, device="cuda", AttenuationThreshold=None):
    path = os.path.join(SavePath, "AttenuationMask.npy")
    if os.path.isfile(path) and not Overwrite:
        return np.load(path)
    if np.asarray(extendedGeometry).shape[0] != 0:  # span (TailsMask.py:70-74)
        mask = MaskGeneratorMashing(ActivityMapDownscaled, AttenuationMapDownscaled, ImageSize,
                                    extendedGeometry, LORCoordinates, SinogramIndex, UseAttenuation,
                                    AccelerationFactor, device, AttenuationThreshold)
    else:
        mask = MaskGenerator(ActivityMapDownscaled, AttenuationMapDownscaled, ImageSize, Geometry,
                             LORCoordinates, SinogramIndex, UseAttenuation, AccelerationFactor, device,
                             AttenuationThreshold)
    np.save(path, mask)
    return mask
