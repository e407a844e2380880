"""Drop-in ``SingleScatterSimulationTOF`` / ``SingleScatterSimulation``.

Same names, arguments, units and output as the reference
(``Python/openSSS/SingleScatterSimulationTOF.py:36-208``): NumPy in, a fresh
float32 array ``(NrBins, ND+1, ND//2, NrRingsUsed**2)`` out, and the
``Scatters_SSS.npz`` side file when ``SavePath`` is given.  The work runs on
the GPU through ``libsss300.so``; there is no CPU path.
"""

from __future__ import annotations

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
# device buffer are kept for such calls, found by comparing every input but
# the two maps with copies kept from the call that built them.
_CACHE_SIZE = 2
# Host threads below which the GPU writes the whole result rather than the
# host clearing it during the simulation: 16 threads clear the 13-bin
# workload's 3.85 GB in 13 ms, against 52 ms of simulation and 20 ms for the
# GPU to write the zeros over the host link.
_MIN_CLEAR_THREADS = 4
_cache: "list[tuple[_Inputs, _DropIn]]" = []
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


class _Inputs:
    """The inputs an engine is built from, kept as contiguous copies: a later
    call reuses the engine when its inputs are the same bytes (compared in
    full; a few MB, a fraction of a millisecond)."""

    def __init__(self, arrays, scalars, device):
        self.arrays = [np.array(a, copy=True, order="C") for a in arrays]
        self.scalars = (scalars, str(device))

    def same(self, arrays, scalars, device) -> bool:
        if self.scalars != (scalars, str(device)):
            return False
        for mine, a in zip(self.arrays, arrays):
            a = np.ascontiguousarray(a)
            if a.dtype != mine.dtype or a.shape != mine.shape:
                return False
            words = np.uint64 if a.nbytes % 8 == 0 else np.uint8  # the bytes, compared 8 at a time
            if not np.array_equal(a.reshape(-1).view(words), mine.reshape(-1).view(words)):
                return False
        return True


def _drop_in(Geometry, SinogramCoordinates, NormalVectors, DetectorSize, AttenuationTable, EnergyResolution,
             EnergyThreshold, NrRingsUsed, NrDetectorsUsed, SampleStep, TOFResolution, TOFRange, NrBins,
             device) -> _DropIn:
    arrays = [Geometry, SinogramCoordinates, NormalVectors, DetectorSize, AttenuationTable, SampleStep]
    scalars = (float(EnergyResolution), float(EnergyThreshold), int(NrRingsUsed), int(NrDetectorsUsed),
               float(TOFResolution), float(TOFRange), int(NrBins))
    with _lock:
        for i, (inputs, d) in enumerate(_cache):
            if inputs.same(arrays, scalars, device):
                _cache.append(_cache.pop(i))  # most recent last
                return d
    eng = TofSSS(Geometry, NormalVectors, DetectorSize, AttenuationTable, EnergyResolution, EnergyThreshold,
                 NrRingsUsed, NrDetectorsUsed, SampleStep, TOFResolution, TOFRange, NrBins, device=device)
    d = _DropIn(eng, SinogramCoordinates)
    with _lock:
        _cache.append((_Inputs(arrays, scalars, device), d))
        while len(_cache) > _CACHE_SIZE:
            _cache.pop(0)
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
    if d.full and torch.get_num_threads() < _MIN_CLEAR_THREADS:
        # too few host threads to clear 3.85 GB within the simulation: the GPU
        # writes every element, zeros included, over the host link
        compact = eng.run(ActivityMap, AttenuationMap, ImageSize)
        eng.densify_full(compact, d.cells, host)
    elif d.full:
        # Over 99% of the dense layout is zero: the host's cores clear the
        # result (torch's parallel fill, in a thread of its own) while the GPU
        # simulates, and the GPU then writes the sampled cells alone over the
        # host link instead of the whole array.
        failed = []

        def clear():
            try:
                host.zero_()
            except BaseException as e:  # noqa: BLE001 - re-raised in the calling thread
                failed.append(e)

        clearing = threading.Thread(target=clear)
        clearing.start()
        try:
            compact = eng.run(ActivityMap, AttenuationMap, ImageSize)
        finally:
            clearing.join()
        if failed:
            raise failed[0]
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
