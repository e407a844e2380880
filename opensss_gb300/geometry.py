"""Geometry-time lookup tables (host, computed once per scanner / sampling).

These are the reference's set-up tables, not per-call work: sinogram
coordinates of every crystal pair, the ring-pair slice order, the sampled
rings/crystals of the SSS, and the nearest-neighbour source tables the
upsampling gathers through.  The hot paths that consume them run on the GPU.
"""

from __future__ import annotations

import functools

import numpy as np


def SinogramCoordinates(NrSectorsTrans: int, NrSectorsAxial: int, NrModulesAxial: int,
                        NrModulesTrans: int, NrCrystalsTrans: int, NrCrystalsAxial: int,
                        MinSectorDifference: int = 0, ID_Shidt: bool = True):
    """Sinogram coordinates of every crystal pair and slice index of every
    ring pair; same arguments and outputs as the reference
    (``Python/openSSS/Sinogram.py:27-141``), evaluated with array operations.

    Returns ``(LORCoordinates int16 [N, N, 2] (angular, radial),
    SinogramIndex int16 [NR, NR], DetectorShift int)``.
    """
    nr = NrSectorsAxial * NrModulesAxial * NrCrystalsAxial
    n = NrSectorsTrans * NrModulesTrans * NrCrystalsTrans
    min_diff = MinSectorDifference * NrModulesTrans * NrCrystalsTrans
    radial_size = n - 2 * (min_diff - 1) - 1
    shift = (NrModulesTrans * NrCrystalsTrans) // 2 if ID_Shidt else 0

    cid = np.arange(n, dtype=np.int64) % n - shift
    cid[cid < 0] += n
    c1 = cid[:, None]
    c2 = cid[None, :]
    ida = np.where(c1 < c2, c1, c2)
    idb = np.where(c1 < c2, c2, c1)
    s = ida + idb
    diff = idb - ida
    outer = (s >= (3 * n) // 2) | (s < n // 2)
    rad_outer = np.where(ida == idb, (-n) // 2, ((diff - 1) // 2) - ((n - (diff + 1)) // 2))
    rad_inner = np.where(ida == idb, n // 2, ((n - (diff + 1)) // 2) - ((diff - 1) // 2))
    radial = np.where(outer, rad_outer, rad_inner)
    angular = np.where(s < n // 2, (2 * ida + n + radial) // 2,
                       np.where(s >= (3 * n) // 2, (2 * ida - n + radial) // 2,
                                (2 * ida - radial) // 2))
    lor = np.full((n, n, 2), -1, dtype=np.int64)
    ok = diff >= min_diff
    lor[..., 0] = np.where(ok, angular, -1)
    lor[..., 1] = np.where(ok, radial + radial_size // 2, -1)

    r1 = np.arange(nr)[:, None]
    r2 = np.arange(nr)[None, :]
    d = np.abs(r1 - r2)
    below = (2 * d - 1) * nr - d * (d - 1) + r2
    above = (2 * d - 1) * nr - d * (d - 1) + (nr - d) + r1
    sino = np.where(r1 == r2, r1, np.where(r2 < r1, below, above))
    return lor.astype(np.int16), sino.astype(np.int16), int(shift)


def check_dense_lor(lor, detectors, nd: int) -> np.ndarray:
    """The LORCoordinates table ``sss_tof_densify`` reads, checked on the
    host: shape [nd, nd, 2], and for every pair of sampled crystals (di1 <=
    di2) an angle in 0..nd/2-1 and a radius in 0..nd, the bounds of the
    dense [B, nd+1, nd/2, NRU^2] output.  Raises IndexError otherwise (the
    reference's numpy indexing raises for entries past the array)."""
    lor = np.asarray(lor)
    if lor.shape != (nd, nd, 2):
        raise ValueError(f"SinogramCoordinates must be [{nd}, {nd}, 2], got {lor.shape}")
    d = np.asarray(detectors, dtype=np.int64)
    i1, i2 = np.triu_indices(len(d))
    pairs = lor[d[i1], d[i2]]
    ang, rad = pairs[:, 0], pairs[:, 1]
    if len(pairs) and (ang.min() < 0 or ang.max() >= nd // 2 or rad.min() < 0 or rad.max() > nd):
        raise IndexError(f"SinogramCoordinates of a sampled crystal pair lie outside the "
                         f"{nd + 1} x {nd // 2} sinogram")
    return lor


def dense_cell_pairs(lor, detectors, nd: int) -> np.ndarray:
    """int32 [(nd+1)*(nd/2)]: for each sinogram cell rad*(nd/2) + ang of the
    dense layout, the sampled crystal pair di1*ndu + di2 (di1 <= di2) whose
    LOR lies there, or -1 (the table sss_tof_densify_full reads).  The LOR
    table is checked as for sss_tof_densify; two sampled pairs in one cell
    (which the reference would add together) raise ValueError."""
    lor = check_dense_lor(lor, detectors, nd)
    d = np.asarray(detectors, dtype=np.int64)
    ndu = len(d)
    i1, i2 = np.triu_indices(ndu)
    cells = lor[d[i1], d[i2], 1].astype(np.int64) * (nd // 2) + lor[d[i1], d[i2], 0]
    if len(np.unique(cells)) != len(cells):
        raise ValueError("two sampled crystal pairs share a sinogram cell")
    out = np.full((nd + 1) * (nd // 2), -1, dtype=np.int32)
    out[cells] = (i1 * ndu + i2).astype(np.int32)
    return out


def check_slice_table(SinogramIndex, nr: int) -> np.ndarray:
    """SinogramIndex[:nr, :nr] as the tail mask reads it on the device: every
    ring pair's slice in 0..nr^2-1, the mask's slice axis.  Raises IndexError
    otherwise (the reference's numpy indexing raises past the axis)."""
    si = np.asarray(SinogramIndex)[:nr, :nr]
    if si.shape != (nr, nr):
        raise ValueError(f"SinogramIndex must cover {nr} x {nr} ring pairs, got {si.shape}")
    if si.size and (si.min() < 0 or si.max() >= nr * nr):
        raise IndexError(f"SinogramIndex holds slices outside 0..{nr * nr - 1}")
    return si


def sampled_rings(nr_rings: int, nr_rings_used: int) -> np.ndarray:
    """Rings the SSS simulates (``SingleScatterSimulationTOF.py:153``)."""
    return np.floor(np.linspace(0, nr_rings - 1, nr_rings_used) + 0.5).astype(np.int64)


def sampled_detectors(nr_detectors: int, nr_detectors_used: int) -> np.ndarray:
    """Crystals the SSS simulates per ring (``SingleScatterSimulationTOF.py:159-167``):
    accumulated floor with step ND/NDU starting at crystal 0."""
    step = nr_detectors / nr_detectors_used
    det = np.zeros(nr_detectors_used, dtype=np.int64)
    for d in range(1, nr_detectors_used):
        det[d] = int(np.floor(det[d - 1] + step))
    return det


@functools.lru_cache(maxsize=16)
def _upsample_source_cached(lor_bytes: bytes, nd: int, det_key: tuple):
    lor = np.frombuffer(lor_bytes, dtype=np.int16).reshape(nd, nd, 2)
    return _upsample_source(lor, nd, np.array(det_key, dtype=np.int64))


def _upsample_source(lor, nd, det):
    # The reference fills each full sinogram from the sampled crystal pairs
    # with scipy's nearest-neighbour griddata (Interpolation.py:122-131); the
    # point set is the same for every ring pair because every ring uses the
    # same crystals.  Asking the same interpolator for point numbers instead of
    # values reproduces its choices, including its tie-breaking.
    from scipy.interpolate import NearestNDInterpolator

    ndu = len(det)
    rad = lor[np.ix_(det, det, [1])][:, :, 0]
    ang = lor[np.ix_(det, det, [0])][:, :, 0]
    points = np.array([(y, x) for y, x in zip(rad.flatten(), ang.flatten())])
    gx, gy = np.mgrid[0:nd + 1, 0:nd // 2]
    src = NearestNDInterpolator(points, np.arange(ndu * ndu))((gx, gy))
    return np.ascontiguousarray(src.astype(np.int32))


def upsample_source(lor: np.ndarray, detectors: np.ndarray) -> np.ndarray:
    """int32 [ND+1, ND/2]: griddata point number p = a*NDU + b (a, b = sampled
    crystal indices of the two rings) whose value fills each full-sinogram bin."""
    lor = np.ascontiguousarray(lor, dtype=np.int16)
    nd = lor.shape[0]
    return _upsample_source_cached(lor.tobytes(), nd, tuple(int(d) for d in detectors))


def nearest_grid_index(x, grid: np.ndarray) -> np.ndarray:
    """RegularGridInterpolator 'nearest' along one axis (SciPy's published
    rule): interval i with grid[i] <= x < grid[i+1] (clamped to the first and
    last interval), then i if (x - grid[i]) / (grid[i+1] - grid[i]) <= 0.5
    else i + 1; -1 where x lies outside [grid[0], grid[-1]] (the reference's
    fill_value=0)."""
    g = np.asarray(grid, dtype=np.float64)
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    if len(g) == 1:
        return np.where(x == g[0], 0, -1).astype(np.int32)
    i = np.clip(np.searchsorted(g, x, side="right") - 1, 0, len(g) - 2)
    frac = (x - g[i]) / (g[i + 1] - g[i])
    out = np.where(frac <= 0.5, i, i + 1)
    out[(x < g[0]) | (x > g[-1])] = -1
    return out.astype(np.int32)


def ring_nearest(nr_rings: int, rings: np.ndarray) -> np.ndarray:
    """Index of the sampled ring each ring copies from: RegularGridInterpolator
    'nearest' over the sampled ring numbers, ties to the lower ring
    (Interpolation.py:256)."""
    return nearest_grid_index(np.arange(nr_rings), rings)


def slice_rings(sino_index: np.ndarray) -> np.ndarray:
    """Inverse of SinogramIndex: int64 [NR*NR, 2] ring pair (Ring1, Ring2) of each slice."""
    si = np.asarray(sino_index, dtype=np.int64)
    nr = si.shape[0]
    inv = np.full((nr * nr, 2), -1, dtype=np.int64)
    r1, r2 = np.meshgrid(np.arange(nr), np.arange(nr), indexing="ij")
    inv[si.reshape(-1), 0] = r1.reshape(-1)
    inv[si.reshape(-1), 1] = r2.reshape(-1)
    if (inv < 0).any():
        raise ValueError("SinogramIndex is not a permutation of the slices")
    return inv


class UpsampleTables(tuple):
    """``(cell_src, ring_src, bin_stride)`` plus ``ring_off`` (the distinct
    values of ring_src, int64) and ``ring_idx`` (int32, ring_src =
    ring_off[ring_idx]): the upsampling kernel stages one cell's distinct
    ring pairs in shared memory."""

    def __new__(cls, cell_src, ring_src, stride):
        self = super().__new__(cls, (cell_src, ring_src, stride))
        off, inv = np.unique(np.asarray(ring_src), return_inverse=True)
        self.ring_off = np.ascontiguousarray(off, dtype=np.int64)
        self.ring_idx = np.ascontiguousarray(inv.reshape(-1), dtype=np.int32)
        self.device_copies = {}
        return self

    def on(self, device):
        """(cell_src, ring_off, ring_idx) as device tensors, cached per device."""
        import torch

        key = str(device)
        if key not in self.device_copies:
            self.device_copies[key] = tuple(torch.from_numpy(a).to(device)
                                            for a in (self[0], self.ring_off, self.ring_idx))
        return self.device_copies[key]


def upsample_tables(lor, sino_index, nru: int, ndu: int, layout: str = "dense"):
    """Gather tables of the upsampling (Interpolation.py:197-319):
    full-sinogram value (cell, slice) = sampled[cell_src[cell] + ring_src[slice]]
    (per TOF bin, plus bin * bin_stride).

    layout 'dense'  : the reference's sampled array [bins][ND+1][ND/2][NRU^2]
    layout 'legpair': the engine's [bins][NL][NL], leg = crystal_index*NRU + ring_index
    Returns UpsampleTables (cell_src int64 [(ND+1)*(ND/2)], ring_src int64
    [NR*NR], bin_stride)."""
    lor = np.asarray(lor)
    nd = lor.shape[0]
    nr = np.asarray(sino_index).shape[0]
    det = sampled_detectors(nd, ndu)
    rings = sampled_rings(nr, nru)
    src = upsample_source(lor, det).astype(np.int64)
    a, b = np.divmod(src, ndu)
    rmap = ring_nearest(nr, rings).astype(np.int64)
    inv = slice_rings(sino_index)
    # slice (r1, r2) copies the sampled pair (nearest(r1), nearest(r2)) (:251-310)
    ri1, ri2 = rmap[inv[:, 0]], rmap[inv[:, 1]]
    if layout == "dense":
        rad = lor[det[a], det[b], 1].astype(np.int64)
        ang = lor[det[a], det[b], 0].astype(np.int64)
        cell_src = (rad * (nd // 2) + ang) * (nru * nru)
        ring_src = ri1 * nru + ri2
        stride = (nd + 1) * (nd // 2) * nru * nru
    elif layout == "legpair":
        nl = nru * ndu
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        cell_src = lo * nru * nl + hi * nru
        ring_src = ri1 * nl + ri2
        stride = nl * nl
    else:
        raise ValueError(layout)
    return UpsampleTables(np.ascontiguousarray(cell_src.reshape(-1), dtype=np.int64),
                          np.ascontiguousarray(ring_src, dtype=np.int64), int(stride))


# ---------------------------------------------------------------- span / mash


def expandRings(Geometry, NormalVectors):
    """Geometry with a virtual ring half-way between neighbouring rings (2NR-1
    rings), and every ring's normals set to ring 0's, as the reference does
    (``Python/openSSS/Geometry.py:161-197``)."""
    g = np.asarray(Geometry, dtype=np.float64)
    nv = np.asarray(NormalVectors, dtype=np.float64)
    out = np.zeros((2 * g.shape[0] - 1,) + g.shape[1:])
    out[0::2] = g
    out[1::2] = (g[:-1] + g[1:]) / 2
    normals = np.broadcast_to(nv[0], out.shape).copy()
    return out, normals


def mashDetectors(Geometry, NormalVectors, combineSize: int):
    """Angular mashing: groups of ``combineSize`` neighbouring crystals become
    one at their mean position and mean normal
    (``Python/openSSS/Geometry.py:200-235``)."""
    g = np.asarray(Geometry, dtype=np.float64)
    nv = np.asarray(NormalVectors, dtype=np.float64)
    nd = g.shape[1]
    if nd % combineSize != 0:
        raise Exception("Number of detectors not divisible by combineSize: ", nd, combineSize)
    shape = (g.shape[0], nd // combineSize, combineSize, 3)
    return np.nanmean(g.reshape(shape), axis=2), np.nanmean(nv.reshape(shape), axis=2)


def span_upsample_tables(lor, SinogramIndex, nr_rings: int, nru: int, ndu: int,
                         layout: str = "dense") -> UpsampleTables:
    """Gather tables of the span upsampling (``Interpolation.py:321-399``):
    the (radial, angular) sources are those of the plain upsampling; mashed
    sinogram i copies the sampled ring pair (nearest(mean Ring1), nearest(mean
    Ring2)) of the RegularGridInterpolator over the sampled ring numbers."""
    lor = np.asarray(lor)
    nd = lor.shape[0]
    det = sampled_detectors(nd, ndu)
    rings = sampled_rings(nr_rings, nru)
    si = np.asarray(SinogramIndex, dtype=np.float32)
    ri2 = nearest_grid_index(si[:, 0].astype(np.float64), rings).astype(np.int64)
    ri1 = nearest_grid_index(si[:, 1].astype(np.float64), rings).astype(np.int64)
    if (ri1 < 0).any() or (ri2 < 0).any():
        raise ValueError("a mashed sinogram lies outside the sampled rings")
    src = upsample_source(lor, det).astype(np.int64)
    a, b = np.divmod(src, ndu)
    if layout == "dense":
        rad = lor[det[a], det[b], 1].astype(np.int64)
        ang = lor[det[a], det[b], 0].astype(np.int64)
        cell_src = (rad * (nd // 2) + ang) * (nru * nru)
        ring_src = ri1 * nru + ri2
        stride = (nd + 1) * (nd // 2) * nru * nru
    elif layout == "legpair":
        nl = nru * ndu
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        cell_src = lo * nru * nl + hi * nru
        ring_src = ri1 * nl + ri2
        stride = nl * nl
    else:
        raise ValueError(layout)
    return UpsampleTables(np.ascontiguousarray(cell_src.reshape(-1), dtype=np.int64),
                          np.ascontiguousarray(ring_src, dtype=np.int64), int(stride))
