"""CASToR data-file headers (drop-in for ``Timber.Headerfile``).

The header is CASToR's text format: one ``Key: value`` line per field.  The
fields, their defaults and the flag rule follow the reference reader
(``Python/Timber/Headerfile.py:22-105``): a correction flag counts as set when
its line is present with any digit, ``0`` included.
"""

from __future__ import annotations

import re

_NUM = r"(\d*[.]?\d*)"


def _first(pattern: str, text: str):
    m = re.search(pattern, text)
    return m.group(1) if m else None


def ReadHeaderFile(HeaderFilePath: str) -> dict:
    with open(HeaderFilePath) as f:
        text = f.read()

    def req(pattern):
        v = _first(pattern, text)
        if v is None:
            raise IndexError(f"header field missing: {pattern}")
        return v

    mode = req(r"Data mode: (\w*[-]?\w*)")
    max_lines = _first(r"Maximum number of lines per event: (\d*)", text)
    flags = {}
    for key, label in (("attenuation_flag", "Attenuation correction flag"),
                       ("normalization_flag", "Normalization correction flag"),
                       ("scatter_flag", "Scatter correction flag"),
                       ("random_flag", "Random correction flag"),
                       ("tof_flag", "TOF information flag")):
        flags[key] = _first(label + r": (\d)", text) is not None
    tof_resolution = tof_size = tof_bins = tof_range = None
    if flags["tof_flag"]:
        tof_resolution = float(req(r"TOF resolution \(ps\): " + _NUM))
        if "histo" in mode:
            tof_bins = int(req(r"Histo TOF number of bins: (\d*)"))
            tof_size = float(req(r"Histo TOF bin size \(ps\): " + _NUM))
        elif "list" in mode:
            tof_range = float(req(r"List TOF measurement range \(ps\): " + _NUM))
    return {
        "data_filename": req(r"Data filename: (\S*)"),
        "nb_events": int(req(r"Number of events: (\d*)")),
        "data_mode": mode,
        "data_type": req(r"Data type: (\w*)"),
        "start_time": float(req(r"Start time \(s\): " + _NUM)),
        "duration": float(req(r"Duration \(s\): " + _NUM)),
        "scanner_name": req(r"Scanner name: (\S*)"),
        "isotope": req(r"Isotope: (\S*)"),
        "calibration_factor": float(req(r"Calibration factor: " + _NUM)),
        "nb_max_lines": int(max_lines) if max_lines else 1,
        "attenuation_flag": flags["attenuation_flag"],
        "normalization_flag": flags["normalization_flag"],
        "scatter_flag": flags["scatter_flag"],
        "random_flag": flags["random_flag"],
        "tof_flag": flags["tof_flag"],
        "tof_resolution": tof_resolution,
        "tof_bin_size": tof_size,
        "tof_nb_bins": tof_bins,
        "tof_range": tof_range,
    }


def WriteHeaderFile(Header: dict, HeaderFilePath: str):
    """Writes the fields ReadHeaderFile reads, in CASToR's order
    (``Python/Timber/Headerfile.py:107-143``)."""
    lines = [f"Data filename: {Header['data_filename']}",
             f"Number of events: {Header['nb_events']}",
             f"Data mode: {Header['data_mode']}",
             f"Data type: {Header['data_type']}",
             f"Start time (s): {Header['start_time']}",
             f"Duration (s): {Header['duration']}",
             f"Scanner name: {Header['scanner_name']}",
             f"Isotope: {Header['isotope']}",
             f"Calibration factor: {Header['calibration_factor']}"]
    if Header["nb_max_lines"] > 1:
        lines.append(f"Maximum number of lines per event: {Header['nb_max_lines']}")
    for key, label in (("attenuation_flag", "Attenuation correction flag"),
                       ("normalization_flag", "Normalization correction flag"),
                       ("scatter_flag", "Scatter correction flag"),
                       ("random_flag", "Random correction flag")):
        if Header[key]:
            lines.append(f"{label}: 1")
    if Header["tof_flag"]:
        lines.append("TOF information flag: 1")
        lines.append(f"TOF resolution (ps): {Header['tof_resolution']}")
        if "histo" in Header["data_mode"]:
            lines.append(f"Histo TOF number of bins: {Header['tof_nb_bins']}")
            lines.append(f"Histo TOF bin size (ps): {Header['tof_bin_size']}")
        elif "list" in Header["data_mode"]:
            lines.append(f"List TOF measurement range (ps): {Header['tof_range']}")
    with open(HeaderFilePath, "w") as f:
        f.write("\n".join(lines) + "\n")
