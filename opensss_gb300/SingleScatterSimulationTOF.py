"""Drop-in ``SingleScatterSimulationTOF`` / ``SingleScatterSimulation``.

Same names, arguments, units and output as the reference
(``Python/openSSS/SingleScatterSimulationTOF.py:36-208``): NumPy in, a fresh
float32 array ``(NrBins, ND+1, ND//2, NrRingsUsed**2)`` out, and the
``Scatters_SSS.npz`` side file when ``SavePath`` is given.  The work runs on
the GPU through ``libsss300.so``; there is no CPU path.
"""

from __future__ import annotations

import collections
import hashlib
import os
import threading
import time

import numpy as np
import torch

from . import geometry
from .engine import TofSSS, as_device

# Engines of recent calls.  An outer reconstruction loop calls the SSS once
# per iteration with the same scanner, tables and sampling and a new activity
# map; the engine (device tables, launch state) and the reference-layout
# device buffer are kept for such calls, keyed by a SHA-1 of every input but
# the two maps.
_CACHE_SIZE = 2
_cache: "collections.OrderedDict[bytes, _DropIn]" = collections.OrderedDict()
_lock = threading.Lock()


class _DropIn:
    def __init__(self, eng: TofSSS, lor):
        self.engine = eng
        self.full = (eng.nru * eng.nru) % 4 == 0
        if self.full:
            # the result is page-locked host memory: the host clears it during
            # the simulation, then the GPU writes the sampled cells into it
            self.cells = as_device(geometry.dense_cell_pairs(lor, eng.dets_np, eng.nd), torch.int32, eng.device)
        else:
            lor = geometry.check_dense_lor(lor, eng.dets_np, eng.nd)
            self.lor = as_device(np.asarray(lor, dtype=np.int16), torch.int16, eng.device)
            # the reference layout; cells of unsampled pairs stay 0 across calls
            self.dense = torch.zeros((eng.nbins, eng.nd + 1, eng.nd // 2, eng.nru * eng.nru),
                                     dtype=torch.float32, device=eng.device)


def _key(arrays, scalars, device) -> bytes:
    h = hashlib.sha1(usedforsecurity=False)
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(f"{a.dtype.str}{a.shape}".encode())
        h.update(a.reshape(-1).view(np.uint8))
    h.update(repr((scalars, str(device))).encode())
    return h.digest()


def _drop_in(Geometry, SinogramCoordinates, NormalVectors, DetectorSize, AttenuationTable, EnergyResolution,
             EnergyThreshold, NrRingsUsed, NrDetectorsUsed, SampleStep, TOFResolution, TOFRange, NrBins,
             device) -> _DropIn:
    key = _key([Geometry, SinogramCoordinates, NormalVectors, DetectorSize, AttenuationTable, SampleStep],
               (float(EnergyResolution), float(EnergyThreshold), int(NrRingsUsed), int(NrDetectorsUsed),
                float(TOFResolution), float(TOFRange), int(NrBins)), device)
    with _lock:
        d = _cache.get(key)
        if d is not None:
            _cache.move_to_end(key)
            return d
    eng = TofSSS(Geometry, NormalVectors, DetectorSize, AttenuationTable, EnergyResolution, EnergyThreshold,
                 NrRingsUsed, NrDetectorsUsed, SampleStep, TOFResolution, TOFRange, NrBins, device=device)
    d = _DropIn(eng, SinogramCoordinates)
    with _lock:
        _cache[key] = d
        while len(_cache) > _CACHE_SIZE:
            _cache.popitem(last=False)
    return d


def SingleScatterSimulationTOF(ActivityMap, AttenuationMap, ImageSize, Geometry, SinogramCoordinates,
                               NormalVectors, DetectorSize, AttenuationTable, EnergyResolution,
                               EnergyThreshold, NrRingsUsed, NrDetectorsUsed, SampleStep, TOFResolution,
                               TOFRange, NrBins, SavePath, device="cuda"):
    """3D TOF single scatter simulation (Watson); see the module docstring.

    The result is a fresh float32 array the caller owns.  Its memory is
    page-locked host memory from torch's pinned-memory cache, which the GPU
    writes directly over the host link (when NRU^2 is a multiple of 4; else
    the dense array is built on the device and copied): the host clears it
    while the simulation runs, and the GPU writes the sampled cells.  The
    memory returns to the cache when the array is dropped."""
    t0 = time.time()
    d = _drop_in(Geometry, SinogramCoordinates, NormalVectors, DetectorSize, AttenuationTable,
                 EnergyResolution, EnergyThreshold, NrRingsUsed, NrDetectorsUsed, SampleStep, TOFResolution,
                 TOFRange, NrBins, device)
    eng = d.engine
    shape = (eng.nbins, eng.nd + 1, eng.nd // 2, eng.nru * eng.nru)
    host = torch.empty(shape, dtype=torch.float32, pin_memory=True)
    if d.full:
        # Over 99% of the dense layout is zero: the host's cores clear the
        # result (torch's parallel fill, in a thread of its own) while the GPU
        # simulates, and the GPU then writes the sampled cells alone over the
        # host link instead of the whole array.
        clearing = threading.Thread(target=host.zero_)
        clearing.start()
        try:
            compact = eng.run(ActivityMap, AttenuationMap, ImageSize)
        finally:
            clearing.join()
        eng.densify_full(compact, d.cells, host, sampled_only=True)
    else:
        compact = eng.run(ActivityMap, AttenuationMap, ImageSize)
        eng.densify(compact, d.lor, out=d.dense)
        host.copy_(d.dense)
    eng.check_status()
    dense = host.numpy()
    print("Time for SSS: {:.2f} seconds".format(time.time() - t0))
    if SavePath:
        np.savez_compressed(os.path.join(SavePath, "Scatters_SSS.npz"), dense)
    return dense


def SingleScatterSimulation(ActivityMap, AttenuationMap, ImageSize, Geometry, SinogramCoordinates,
                            NormalVectors, DetectorSize, AttenuationTable, EnergyResolution,
                            EnergyThreshold, NrRingsUsed, NrDetectorsUsed, SampleStep, SavePath=None,
                            device="cuda"):
    """Non-TOF SSS: one TOF bin with a timing kernel so wide that every TOF
    weight is exactly 1 (the MATLAB name, ``Matlab/SingleScatterSimulation.m:44``,
    with the Python v1.0 numerics).  Returns ``(ND+1, ND//2, NrRingsUsed**2)``."""
    out = SingleScatterSimulationTOF(ActivityMap, AttenuationMap, ImageSize, Geometry,
                                     SinogramCoordinates, NormalVectors, DetectorSize,
                                     AttenuationTable, EnergyResolution, EnergyThreshold,
                                     NrRingsUsed, NrDetectorsUsed, SampleStep, 1.0e6, 1000.0, 1,
                                     SavePath, device=device)
    return out[0]
