"""Drop-in ``openSSS.DataReduction``: the span (axial mashing) tables.

``SinogramLUT`` (``Python/openSSS/DataReduction.py:102-172``) maps every ring
pair to its mashed sinogram; ``SumLORsCounts`` (:174-215) counts the LORs
mashed into each sinogram bin; ``span_ring_pairs`` gives each mashed
sinogram's ring pair on the expanded geometry, the form the tail-mask and
fit kernels take.  All three are geometry-time host tables (NumPy).  The
ring expansion and angular mashing of the scanner geometry
(``expandRings``, ``mashDetectors``) are ``openSSS.Geometry`` functions and
live in ``opensss_gb300.geometry``.
"""

from __future__ import annotations

import numpy as np

__all__ = ["SinogramLUT", "SumLORsCounts", "span_ring_pairs"]


def SinogramLUT(NrRings: int, AxialMashing: int, MaxRingDifference: int | None = None):
    """Axial mashing (span) tables, same outputs as the reference
    (``Python/openSSS/DataReduction.py:102-172``): ``(SinogramIndex float32
    [n, 2] = mean (Ring2, Ring1) of each mashed sinogram, RingLUT bool
    [2NR-1, 2NR-1], LookUpTable int16 [NR, NR] = mashed sinogram of each ring
    pair or -1, SinogramCounts float32 = ring pairs per mashed sinogram)``.

    A ring pair closer than (span+1)/2 goes to sinogram Ring1 + Ring2 - 1 (the
    sinograms of ring sum); farther pairs go to the segment of their ring
    difference, segments of `span` differences each, alternating positive
    and negative.  The reference's own sinogram count is kept, so ring counts
    it cannot place raise IndexError here too."""
    nr, span = int(NrRings), int(AxialMashing)
    half = (span + 1) / 2
    nseg = int(np.round(nr / span))
    n = int(nr * 2 - 1 + np.sum(4 * (nr - half - span * (np.arange(1, nseg + 1) - 1)) - 2))
    index = np.zeros((n, 2), dtype=np.float32)
    counts = np.zeros(n, dtype=np.float32)
    lut = np.full((nr, nr), -1, dtype=np.int16)
    for r1 in range(1, nr + 1):
        for r2 in range(1, nr + 1):
            diff = r2 - r1
            if MaxRingDifference is not None and abs(diff) > MaxRingDifference:
                continue
            if abs(diff) < half:
                sino = r1 + r2 - 1
            else:
                seg = int(np.floor((abs(diff) - half) / span)) + 1
                # first sinogram of the segment: all lower segments, both signs,
                # and the negative half of this one for a positive difference
                pos = 2 * nr - 1
                last = seg + 1 if diff > 0 else seg
                for k in range(1, last):
                    width = (nr - half - span * (k - 1)) * 2 - 1
                    pos += width * (1 if (k == last - 1 and diff > 0) else 2)
                sino = (r1 + r2 - 1) - seg * span + (span - 1) / 2 + pos
            j = int(sino - 1)
            if j >= n:
                raise IndexError(f"index {j} is out of bounds for axis 0 with size {n}")
            index[j, 0] += r2 - 1
            index[j, 1] += r1 - 1
            counts[j] += 1
            lut[r1 - 1, r2 - 1] = j
    index[:, 0] /= counts + np.float32(1e-8)
    index[:, 1] /= counts + np.float32(1e-8)
    index = index[counts != 0, :]
    ring_lut = np.zeros((nr * 2 - 1, nr * 2 - 1), dtype=bool)
    for a, b in span_ring_pairs(index)[:, :2]:
        ring_lut[a, b] = True
    return index, ring_lut, lut, counts


def span_ring_pairs(SinogramIndex) -> np.ndarray:
    """int32 [n, 3] = (Ring1, Ring2, slice) of each mashed sinogram on the
    expanded (2NR-1)-ring geometry: int(2 * mean ring) as the reference
    computes it in float32 (TailsMask.py:370, BackProjection.py:373)."""
    si = np.asarray(SinogramIndex, dtype=np.float32)
    two = np.float32(2)
    out = np.zeros((si.shape[0], 3), dtype=np.int32)
    out[:, 0] = (si[:, 0] * two).astype(np.int64)
    out[:, 1] = (si[:, 1] * two).astype(np.int64)
    out[:, 2] = np.arange(si.shape[0])
    return out


def SumLORsCounts(Geometry, LookUpTable, SinogramIndex, Mash: int, Span: int, NrSinograms: int):
    """LORs mashed into each sinogram bin: Mash^2 per ring pair, summed over
    the ring pairs of each slice (``Python/openSSS/DataReduction.py:174-215``).
    A ring pair that the span table leaves out (-1) lands on the last slice,
    as numpy's negative index does in the reference."""
    g = np.asarray(Geometry)
    nr, nd = g.shape[0], g.shape[1]
    nslices = NrSinograms if Span > 1 else nr * nr
    table = np.asarray(LookUpTable if Span > 1 else SinogramIndex)[:nr, :nr].astype(np.int64)
    per_slice = np.bincount(np.mod(table.reshape(-1), nslices), minlength=nslices).astype(np.float32)
    ring = np.float32(Mash ** 2)
    return np.broadcast_to(per_slice * ring, (nd + 1, nd // 2, nslices)).astype(np.float32)
