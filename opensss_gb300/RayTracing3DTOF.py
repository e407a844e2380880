"""Drop-in ``RayTracing3DTOF`` / ``RayTracing3D`` and their batched forms.

``RayTracing3DTOF(GridSize, GridBounds, LineCoordinates)`` returns the
reference's triple (``Python/openSSS/RayTracing3DTOF.py:29-180``): FP64
lengths, int32 1-based linear indices (``X + (Y-1)*Ny + (Z-1)*Ny*Nx``) and
FP64 running half-length samples; empty arrays on a miss; ``IndexError``
where the reference's traversal overruns its Nx+Ny+Nz storage.
``RayTracing3D`` mirrors the non-TOF MEX tracer (``Matlab/RayTracing3D.cpp``):
float32 lengths and int32 indices.  The ``*Batch`` forms trace many rays in
one GPU launch and return padded ``[n, Nx+Ny+Nz]`` arrays plus counts.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib


def _trace(GridSize, GridBounds, lines, variant, device="cuda", as_numpy=True):
    if not torch.cuda.is_available():
        raise _lib.EngineUnavailable("no CUDA device: the engine has no CPU path")
    L = _lib.lib()
    grid = np.ascontiguousarray(np.asarray(GridSize).reshape(-1)[:3], dtype=np.int32)
    bounds = np.ascontiguousarray(np.asarray(GridBounds, dtype=np.float64).reshape(-1)[:6])
    if isinstance(lines, torch.Tensor):
        d_lines = lines.to(device=device, dtype=torch.float64).reshape(-1, 6).contiguous()
    else:
        d_lines = torch.from_numpy(np.ascontiguousarray(np.asarray(lines, dtype=np.float64).reshape(-1, 6))
                                   ).to(device)
    n = d_lines.shape[0]
    cap = int(grid.astype(np.int64).sum())
    dev = d_lines.device
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    idx = torch.zeros((n, cap), dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    if variant == 0:
        len64 = torch.zeros((n, cap), dtype=torch.float64, device=dev)
        samp = torch.zeros((n, cap), dtype=torch.float64, device=dev)
        len32 = None
    else:
        len64 = samp = None
        len32 = torch.zeros((n, cap), dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    p = lambda t: C.c_void_p(0 if t is None else t.data_ptr())  # noqa: E731
    _lib.check(L.sss_raytrace(grid.ctypes.data_as(C.c_void_p), bounds.ctypes.data_as(C.c_void_p),
                              p(d_lines), n, variant, cap, p(counts), p(len64), p(len32), p(idx),
                              p(samp), p(status), C.c_void_p(st.cuda_stream)))
    st.synchronize()
    out = (counts, len64 if variant == 0 else len32, idx, samp)
    if as_numpy:
        out = tuple(None if t is None else t.cpu().numpy() for t in out)
    return out


def RayTracing3DTOFBatch(GridSize, GridBounds, Lines, device="cuda", as_numpy=True):
    """(counts [n], lengths f64 [n, cap], indices int32 [n, cap], samples f64 [n, cap]);
    counts = -1 marks rays on which the reference would raise IndexError."""
    return _trace(GridSize, GridBounds, Lines, 0, device, as_numpy)


def RayTracing3DBatch(GridSize, GridBounds, Lines, device="cuda", as_numpy=True):
    """(counts [n], lengths f32 [n, cap], indices int32 [n, cap])."""
    c, ln, ix, _ = _trace(GridSize, GridBounds, Lines, 1, device, as_numpy)
    return c, ln, ix


def RayTracing3DTOF(GridSize, GridBounds, LineCoordinates):
    c, ln, ix, sm = RayTracing3DTOFBatch(GridSize, GridBounds, LineCoordinates)
    n = int(c[0])
    if n < 0:
        raise IndexError("ray traversal overran its Nx+Ny+Nz storage (as the reference does)")
    return ln[0, :n].copy(), ix[0, :n].copy(), sm[0, :n].copy()


def RayTracing3D(GridSize, GridBounds, LineCoordinates):
    c, ln, ix = RayTracing3DBatch(GridSize, GridBounds, LineCoordinates)
    n = int(c[0])
    if n < 0:
        raise IndexError("ray traversal overran its Nx+Ny+Nz storage")
    return ln[0, :n].copy(), ix[0, :n].copy()
