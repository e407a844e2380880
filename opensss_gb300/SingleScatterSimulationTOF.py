"""Drop-in ``SingleScatterSimulationTOF`` / ``SingleScatterSimulation``.

Same names, arguments, units and output as the reference
(``Python/openSSS/SingleScatterSimulationTOF.py:36-208``): NumPy in, a fresh
float32 array ``(NrBins, ND+1, ND//2, NrRingsUsed**2)`` out, and the
``Scatters_SSS.npz`` side file when ``SavePath`` is given.  The work runs on
the GPU through ``libsss300.so``; there is no CPU path.
"""

from __future__ import annotations

import os
import time

import numpy as np

from .engine import TofSSS


def SingleScatterSimulationTOF(ActivityMap, AttenuationMap, ImageSize, Geometry, SinogramCoordinates,
                               NormalVectors, DetectorSize, AttenuationTable, EnergyResolution,
                               EnergyThreshold, NrRingsUsed, NrDetectorsUsed, SampleStep, TOFResolution,
                               TOFRange, NrBins, SavePath, device="cuda"):
    """3D TOF single scatter simulation (Watson); see the module docstring."""
    t0 = time.time()
    eng = TofSSS(Geometry, NormalVectors, DetectorSize, AttenuationTable, EnergyResolution,
                 EnergyThreshold, NrRingsUsed, NrDetectorsUsed, SampleStep, TOFResolution, TOFRange,
                 NrBins, device=device)
    compact = eng.run(ActivityMap, AttenuationMap, ImageSize)
    dense = eng.densify(compact, SinogramCoordinates).cpu().numpy()
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
