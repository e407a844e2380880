"""Loader for the reference openSSS Python package (test infrastructure only).

ORACLE — this module is test infrastructure, never part of the product.  It imports
the unmodified reference modules from the reference checkout named by the
``OPENSSS_REFERENCE`` environment variable (its ``Python`` folder) with a
pass-through ``numba`` stub first on ``sys.path``.  It is used only by
``tests/golden/make_golden.py`` where the reference checkout exists, to produce
the golden fixtures committed under ``tests/golden``; nothing at run time imports it.
"""

import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_PY = os.environ.get("OPENSSS_REFERENCE", "")


def available() -> bool:
    return bool(REFERENCE_PY) and os.path.isdir(os.path.join(REFERENCE_PY, "openSSS"))


def load():
    """Import and return the reference modules as a namespace dict."""
    if not available():
        raise RuntimeError("set OPENSSS_REFERENCE to the reference checkout's Python folder "
                           f"(found: {REFERENCE_PY!r})")
    stub = os.path.join(_HERE, "numba_stub")
    for p in (stub, REFERENCE_PY):
        if p not in sys.path:
            sys.path.insert(0, p)
    # the stub must shadow any real numba
    sys.path.remove(stub)
    sys.path.insert(0, stub)
    import importlib

    mods = {}
    for name in (
        "RayTracing3DTOF",
        "SingleScatterSimulationTOF",
        "Interpolation",
        "TailsMask",
        "BackProjection",
        "Sinogram",
        "Support",
        "DataReduction",
        "Geometry",
    ):
        mods[name] = importlib.import_module(f"openSSS.{name}")
    return mods


def load_utils():
    """Import the reference's Utils module with the recording skimage stand-in
    (oracle/skimage_stub) first on sys.path; returns (Utils, stub transform)."""
    if not available():
        raise RuntimeError("set OPENSSS_REFERENCE to the reference checkout's Python folder "
                           f"(found: {REFERENCE_PY!r})")
    stub = os.path.join(_HERE, "skimage_stub")
    if stub in sys.path:
        sys.path.remove(stub)
    sys.path.insert(0, stub)
    if REFERENCE_PY not in sys.path:
        sys.path.insert(1, REFERENCE_PY)
    import importlib

    transform = importlib.import_module("skimage.transform")
    return importlib.import_module("openSSS.Utils"), transform
