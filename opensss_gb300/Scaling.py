"""Drop-in ``openSSS.Scaling.ScaleScattersToPrompts``: the scale factors of all
TOF bins from the saved prompts, randoms, normalisation, tail mask and
upsampled scatter bins (``Python/openSSS/Scaling.py:27-130``).

The reference fits the bins one after another, walking every LOR once per
bin; here one GPU pass walks each LOR once and back-projects into all bins'
images (``sss_backproject_fit_bins``), which gives each bin the scale its
own fit gives.
"""

from __future__ import annotations

import os
import time

import numpy as np
import torch

from . import _lib
from .BackProjection import fit_bins_device


def ScaleScattersToPrompts(SinogramIndex, SinogramCoordinates, SavePath, DesiredDimensions, FittingSize,
                           Geometry, ExtendedGeometry, AccelerationFactor, SpanFlag, LORCounts, device="cuda"):
    if not torch.cuda.is_available():
        raise _lib.EngineUnavailable("no CUDA device: the engine has no CPU path")
    name = "PromptsSinogramMashed.npz" if SpanFlag else "PromptsSinogram.npz"
    prompts = np.load(os.path.join(SavePath, name))["arr_0"]
    bins = prompts.shape[-1]
    size = prompts.shape[:-1]
    try:
        norm = np.load(os.path.join(SavePath, "NormSinogram.npz"))["arr_0"]
    except Exception:
        norm = np.ones(size, np.single)
    try:
        randoms = np.load(os.path.join(SavePath, "RandomsSinogram.npz"))["arr_0"] * norm
    except Exception:
        randoms = np.zeros(size, np.single)
    mask = np.float32(np.load(os.path.join(SavePath, "AttenuationMask.npy")) >= 1)
    t0 = time.time()
    ncell, nsl = size[0] * size[1], size[2]

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(ncell, nsl))).to(device)

    p = torch.stack([dev(prompts[..., b] / LORCounts) for b in range(bins)])
    s = torch.stack([dev(np.load(os.path.join(SavePath, f"SSS_mashed_bin{b}.npz"))["arr_0"])
                     for b in range(bins)])
    cell = np.arange(ncell, dtype=np.int64) * nsl
    ring = np.arange(nsl, dtype=np.int64)
    if SpanFlag:
        scales = fit_bins_device(p, dev(randoms), dev(mask), s, ncell * nsl, cell, ring, DesiredDimensions,
                                 FittingSize, ExtendedGeometry, SinogramCoordinates, SinogramIndex,
                                 AccelerationFactor, device=device, span=True)
    else:
        nr = np.asarray(SinogramIndex).shape[0]
        order = np.asarray(SinogramIndex)[0:nr, 0:nr].T
        scales = fit_bins_device(p, dev(randoms), dev(mask), s, ncell * nsl, cell, ring, DesiredDimensions,
                                 FittingSize, Geometry, SinogramCoordinates, order, AccelerationFactor,
                                 device=device)
    print("Time for Scaling: {:.2f} seconds".format(time.time() - t0))
    scales = scales.astype(np.float32)
    np.save(os.path.join(SavePath, "ScaleFactors.npy"), scales)
    return scales
