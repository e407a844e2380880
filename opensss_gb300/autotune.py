"""Launch-shape tuner for the TOF-SSS kernels.

The pair kernel's block (warps per block, up to the size it is compiled for)
and the leg kernel's block (threads per block) are runtime choices
(``sss_tof_problem.pair_warps`` / ``leg_threads``).  ``tune`` times every
candidate on the first scatter points of a problem — the pair stage for each
pair-block size, then the leg stage for each leg-block size, with the stage
timers of ``sss_tof_run`` — and keeps the fastest of each.  Results are cached
per device and size class (TOF bins, sampled legs, volume size, compensated
sum), in memory and in a JSON file (``OPENSSS_GB300_TUNE_CACHE``, default
``~/.cache/opensss_gb300/launch_shapes.json``), so a class is timed once per
machine.  ``BatchSSS(..., autotune=True)`` tunes each TOF class of a batch on
its largest problem.
"""

from __future__ import annotations

import ctypes as C
import json
import os
import threading

import numpy as np
import torch

from . import _lib

LEG_THREADS = (64, 128, 256)
_lock = threading.Lock()
_memory: dict[str, dict] = {}


def cache_path() -> str:
    return os.environ.get("OPENSSS_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "opensss_gb300", "launch_shapes.json"))


def pair_warp_candidates(nbins: int, kahan: bool = False) -> list[int]:
    """Pair-block sizes to try: 4, 8, 12 warps up to the compiled bound."""
    bound = int(_lib.lib().sss_pair_warps_max(int(nbins), _lib.SSS_FLAG_KAHAN if kahan else 0))
    return [w for w in (4, 8, 12) if w <= bound] or [bound]


def size_class(device_name: str, nbins: int, nl: int, shape, kahan: bool = False) -> str:
    """Cache key: device, bin count, sampled legs and volume voxels rounded to
    powers of two (problems in one class share their best launch shape)."""
    def p2(x):
        return 1 << max(0, int(np.ceil(np.log2(max(1, int(x))))))
    return f"{device_name}|bins={int(nbins)}|legs={p2(nl)}|vox={p2(np.prod([int(s) for s in shape]))}|kahan={int(kahan)}"


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, value: dict) -> None:
    data = _load()
    data[key] = value
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home: the in-memory cache still holds the result


def lookup(key: str) -> dict | None:
    with _lock:
        if key in _memory:
            return _memory[key]
    v = _load().get(key)
    if v is not None:
        with _lock:
            _memory[key] = v
    return v


def _stage_ms(engine, act_f, mu_f, shape, image_size, points: int, reps: int, kahan: bool) -> tuple[float, float]:
    L = _lib.lib()
    st = np.zeros(6)
    legs, pairs = [], []
    L.sss_set_timing(1)
    try:
        for i in range(reps + 1):
            engine.run_flat(act_f, mu_f, shape, image_size, max_points=points, check=(i == 0), kahan=kahan)
            _lib.check(L.sss_get_timing(st.ctypes.data_as(C.c_void_p)))
            if i:  # the first run warms up
                legs.append(st[0])
                pairs.append(st[1])
    finally:
        L.sss_set_timing(0)
    return float(np.median(legs)), float(np.median(pairs))


def tune(engine, activity, attenuation, image_size, sample_points: int = 256, reps: int = 3,
         kahan: bool = False, use_cache: bool = True, shape=None) -> dict:
    """Times the launch-shape candidates on the problem's first
    ``sample_points`` scatter points, sets ``engine.pair_warps`` /
    ``engine.leg_threads`` to the fastest and returns
    ``{"pair_warps", "leg_threads", "pairs_ms", "legs_ms", "key", "cached"}``
    (the two ``_ms`` maps hold every candidate's stage time).  Maps are
    [Nx, Ny, Nz] volumes, or CUDA tensors flattened in Fortran order with
    ``shape`` given."""
    from .engine import fortran_flat

    dev = engine.device
    if shape is None:
        shape = tuple(int(s) for s in np.shape(activity))
        act_f, mu_f = fortran_flat(activity, dev), fortran_flat(attenuation, dev)
    else:
        shape = tuple(int(s) for s in shape)
        act_f, mu_f = activity, attenuation
    key = size_class(torch.cuda.get_device_name(dev), engine.nbins, engine.nl, shape, kahan)
    if use_cache:
        hit = lookup(key)
        if hit is not None:
            engine.pair_warps, engine.leg_threads = int(hit["pair_warps"]), int(hit["leg_threads"])
            return dict(hit, cached=True)
    pairs_ms, legs_ms = {}, {}
    engine.leg_threads = 0
    for w in pair_warp_candidates(engine.nbins, kahan):
        engine.pair_warps = w
        pairs_ms[w] = _stage_ms(engine, act_f, mu_f, shape, image_size, sample_points, reps, kahan)[1]
    best_w = min(pairs_ms, key=pairs_ms.get)
    engine.pair_warps = best_w
    for t in LEG_THREADS:
        engine.leg_threads = t
        legs_ms[t] = _stage_ms(engine, act_f, mu_f, shape, image_size, sample_points, reps, kahan)[0]
    best_t = min(legs_ms, key=legs_ms.get)
    engine.leg_threads = best_t
    result = {"pair_warps": best_w, "leg_threads": best_t, "key": key, "sample_points": sample_points,
              "pairs_ms": {str(k): v for k, v in pairs_ms.items()},
              "legs_ms": {str(k): v for k, v in legs_ms.items()}}
    with _lock:
        _memory[key] = result
    if use_cache:
        _store(key, result)
    return dict(result, cached=False)
