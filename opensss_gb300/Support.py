"""Drop-in ``ReadParameters`` and ``NormalizeArray`` (Python/openSSS/Support.py:103-220).

``ReadParameters`` reads the ``key = value`` parameter file that the
reference's pipeline starts from (Python/parameters_Demo.txt,
ExampleScript.py:44), with the reference's value typing:
- one level of matching quotes is removed;
- ``(a, b, c)`` becomes a tuple of the first three items, all int or all
  float;
- ``[a, b, ...]`` becomes a list, all int or all float;
- ``True`` / ``False`` become bools;
- a lone value becomes an int, else a float, else it stays a string.

Items are separated by ", " exactly.  A group that converts neither way
stays a string without its brackets.  The errors are the reference's: a line
without exactly one "=" raises ValueError, and a parenthesised group whose
first items convert but that has fewer than three raises IndexError.
Host code, no device work.
"""

from __future__ import annotations

import numpy as np


def _triple(items, kind):
    """The first three items as ``kind``; None if one does not convert (a
    missing item raises IndexError, as in the reference)."""
    try:
        return (kind(items[0]), kind(items[1]), kind(items[2]))
    except ValueError:
        return None


def _sequence(items, kind):
    try:
        return [kind(x) for x in items]
    except ValueError:
        return None


def _scalar(text):
    for kind in (int, float):
        try:
            return kind(text)
        except ValueError:
            pass
    return text


def _typed(value: str):
    if value[:1] in ("'", '"') and value.endswith(value[:1]):  # a lone quote becomes ""
        value = value[1:-1]
    if value.startswith("(") and value.endswith(")"):
        value = value[1:-1]
        items = value.split(", ")
        for kind in (int, float):
            got = _triple(items, kind)
            if got is not None:
                return got
    if value.startswith("[") and value.endswith("]"):
        value = value[1:-1]
        items = value.split(", ")
        for kind in (int, float):
            got = _sequence(items, kind)
            if got is not None:
                return got
    if value in ("True", "False"):
        return value == "True"
    return _scalar(value)


def ReadParameters(file_path: str) -> dict:
    """Every ``key = value`` line of the file (blank lines and lines starting
    with '#' skipped), typed as the module docstring says."""
    params = {}
    with open(file_path) as f:
        for raw in f:
            line = raw.strip()
            if not line or line.startswith("#"):
                continue
            parts = line.split("=")
            if len(parts) != 2:
                raise ValueError(f"parameter line needs exactly one '=': {line!r}")
            params[parts[0].strip()] = _typed(parts[1].strip())
    return params


def NormalizeArray(array, target_min: float = 0, target_max: float = 255):
    """Min-max scaling of ``array`` to [target_min, target_max]; a constant
    array is not rescaled first.  The default 0..255 range gives uint8."""
    lo, hi = np.min(array), np.max(array)
    unit = (array - lo) / (hi - lo) if hi > lo else array
    out = target_min + unit * (target_max - target_min)
    if target_min == 0 and target_max == 255:
        out = out.astype(np.uint8)
    return out
