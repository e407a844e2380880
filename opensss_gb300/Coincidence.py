"""CASToR list-mode event records (drop-in for ``Timber.Coincidence``).

An event is a packed little-endian record: uint32 time (ms), one float32 per
correction present (attenuation, scatter, random, normalisation, TOF in that
order), a uint32 line count when an event may hold several lines, then the
uint32 crystal IDs of each line (``Python/Timber/Coincidence.py:47-95``).
The record layout is CASToR's file format, so the field order and the
positions returned are the reference's.  ``ParseCASToRIDs`` is the host form
of the ID decoding that ``csrc/listmode.cu`` runs per event on the GPU.
"""

from __future__ import annotations

import struct


def GenerateListEventInfo(AttenuationFlag: bool, ScatterFlag: bool, RandomFlag: bool,
                          NormalizationFlag: bool, TOFFlag: bool, MaxNbLines: int):
    """(struct format, positions): positions are the field indices of the
    scatter, random, normalisation and TOF values (None when absent) and of
    the first crystal ID."""
    nlines = MaxNbLines > 1
    ncorr = int(AttenuationFlag) + int(ScatterFlag) + int(RandomFlag) + int(NormalizationFlag) + int(TOFFlag)
    fmt = "<1L" + (f"{ncorr}f" if ncorr > 0 else "") + ("1I" if nlines else "") + f"{2 * MaxNbLines}L"
    a, s, r, n, t = (int(AttenuationFlag), int(ScatterFlag), int(RandomFlag), int(NormalizationFlag),
                     int(TOFFlag))
    pos = (1 + a if ScatterFlag else None,
           1 + a + s if RandomFlag else None,
           1 + a + s + r if NormalizationFlag else None,
           1 + a + s + r + n if TOFFlag else None,
           1 + a + s + r + n + t + int(nlines))
    return fmt, pos


def GenerateEventClass(DataHeader: dict):
    if "list" not in DataHeader["data_mode"]:
        raise NotImplementedError("Handling of histogram data is not yet implemented")
    return GenerateListEventInfo(DataHeader["attenuation_flag"], DataHeader["scatter_flag"],
                                 DataHeader["random_flag"], DataHeader["normalization_flag"],
                                 DataHeader["tof_flag"], DataHeader["nb_max_lines"])


def record_bytes(fmt: str) -> int:
    return struct.calcsize(fmt)


def ParseCASToRIDs(event, field_pos, NrCrystalsPerRing: int, Shift: int = 0):
    """(detector1, ring1, detector2, ring2, TOF) of one unpacked event: the
    two crystals ordered by crystal number, the rings ordered by the shifted
    crystal numbers, and the TOF sign following the ring order
    (``Python/Timber/Coincidence.py:97-159``)."""
    a, b = event[field_pos[4]], event[field_pos[4] + 1]
    tof = event[field_pos[3]]
    id1, id2 = (a, b) if a < b else (b, a)
    tof_t = tof if a < b else -tof
    c1, c2 = id1 % NrCrystalsPerRing, id2 % NrCrystalsPerRing
    d1, d2 = (c1, c2) if c1 < c2 else (c2, c1)
    s1, s2 = c1 - Shift, c2 - Shift
    s1 += NrCrystalsPerRing if s1 < 0 else 0
    s2 += NrCrystalsPerRing if s2 < 0 else 0
    if s1 < s2:
        return d1, id1 // NrCrystalsPerRing, d2, id2 // NrCrystalsPerRing, tof_t
    return d1, id2 // NrCrystalsPerRing, d2, id1 // NrCrystalsPerRing, -tof_t
