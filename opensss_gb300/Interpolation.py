"""Drop-in ``InterpolateScatters``: the scatter sinogram upsampled from the
sampled crystals/rings to the full sinogram, on the GPU.

Same arguments and result as the reference (``Python/openSSS/Interpolation.py:32-93``):
the sum over TOF bins, float32 ``(ND+1, ND//2, NR**2)``, plus the per-bin
``SSS_mashed_bin{b}.npz`` side files when ``SavePath`` is given.  The
nearest-neighbour choices are resolved once per geometry
(``geometry.upsample_tables``); the upsampling itself is one gather kernel.
"""

from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np
import torch

from . import _lib, geometry


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def upsample_device(sampled: torch.Tensor, tables, nbins: int, ncell: int, nslices: int,
                    bin_index: int | None = None, out: torch.Tensor | None = None) -> torch.Tensor:
    """Gather on the device.  ``tables``: geometry.upsample_tables(...).
    bin_index None sums all bins (in bin order)."""
    _lib.require_cuda(sampled=sampled, out=out)
    if not isinstance(tables, geometry.UpsampleTables):
        tables = geometry.UpsampleTables(*(t.cpu().numpy() if isinstance(t, torch.Tensor) else t
                                           for t in tables[:2]), int(tables[2]))
    stride = tables[2]
    dev = sampled.device
    cs, ro, ri = tables.on(dev)
    if out is None:
        out = torch.empty((ncell, nslices), dtype=torch.float32, device=dev)
    base = sampled if bin_index is None else sampled.reshape(-1)[bin_index * stride:]
    st = torch.cuda.current_stream(dev)
    _lib.check(_lib.lib().sss_upsample(_ptr(base), stride, nbins if bin_index is None else 1,
                                       _ptr(cs), ncell, _ptr(ro), int(ro.numel()), _ptr(ri), nslices,
                                       _ptr(out), C.c_void_p(st.cuda_stream)))
    return out


def InterpolateScatters(Scatters, NrRings, NrRingsUsed, NrDetectors, NrDetectorsUsed,
                        SinogramCoordinates, SinogramIndex, SavePath, SpanFlag, device="cuda"):
    """Upsample the sampled scatter sinogram (see the module docstring).
    With ``SpanFlag`` the slices are the mashed sinograms of SinogramIndex
    (float [n, 2], mean rings, from SinogramLUT), as InterpolateAllBinsSpan
    (Interpolation.py:321-399) evaluates them."""
    if not torch.cuda.is_available():
        raise _lib.EngineUnavailable("no CUDA device: the engine has no CPU path")
    t0 = time.time()
    nd, nr = int(NrDetectors), int(NrRings)
    nbins = Scatters.shape[0]
    dense = torch.from_numpy(np.ascontiguousarray(Scatters, dtype=np.float32)).to(device)
    if SpanFlag:
        tables = geometry.span_upsample_tables(SinogramCoordinates, SinogramIndex, nr, int(NrRingsUsed),
                                               int(NrDetectorsUsed), "dense")
        nslices = int(np.asarray(SinogramIndex).shape[0])
    else:
        tables = geometry.upsample_tables(SinogramCoordinates, np.asarray(SinogramIndex)[:nr, :nr],
                                          int(NrRingsUsed), int(NrDetectorsUsed), "dense")
        nslices = nr * nr
    ncell = (nd + 1) * (nd // 2)
    if SavePath:
        buf = torch.empty((ncell, nslices), dtype=torch.float32, device=device)
        for b in range(nbins):
            upsample_device(dense, tables, nbins, ncell, nslices, bin_index=b, out=buf)
            np.savez_compressed(os.path.join(SavePath, f"SSS_mashed_bin{b}"),
                                buf.cpu().numpy().reshape(nd + 1, nd // 2, nslices))
    total = upsample_device(dense, tables, nbins, ncell, nslices)
    out = total.cpu().numpy().reshape(nd + 1, nd // 2, nslices)
    elapsed = time.time() - t0
    print("Time for Interpolation: {:.2f} seconds".format(elapsed))
    if SavePath:
        with open(os.path.join(SavePath, "Simulation_time.txt"), "w") as f:
            f.write("Time for Interpolation: {:.2f} seconds\n".format(elapsed))
    return out
