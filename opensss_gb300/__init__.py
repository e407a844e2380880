"""opensss_gb300 — GB300-native (sm_103a) TOF single scatter simulation.

Drop-in replacements for openSSS's scatter-estimation entry points; the
compute runs in hand-written CUDA kernels in ``libsss300.so`` behind the C ABI
of ``include/sss300.h``.  PyTorch provides device buffers and streams only.
"""

from .geometry import SinogramCoordinates, sampled_detectors, sampled_rings  # noqa: F401
from .RayTracing3DTOF import (RayTracing3D, RayTracing3DBatch, RayTracing3DTOF,  # noqa: F401
                              RayTracing3DTOFBatch)
from .SingleScatterSimulationTOF import SingleScatterSimulation, SingleScatterSimulationTOF  # noqa: F401
from .engine import TofSSS  # noqa: F401

__version__ = "0.1.0"
