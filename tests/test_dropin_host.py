"""Host logic of the drop-in SingleScatterSimulationTOF: the engine cache
reuses an engine only for inputs that are the same bytes (no GPU needed)."""

import sys

import numpy as np


def _module():
    import opensss_gb300.SingleScatterSimulationTOF  # noqa: F401

    return sys.modules["opensss_gb300.SingleScatterSimulationTOF"]


def test_engine_cache_compares_inputs_byte_for_byte():
    M = _module()
    rng = np.random.default_rng(3)
    geom = rng.random((4, 6, 3))
    lor = np.arange(72, dtype=np.int16).reshape(6, 6, 2)
    scalars = (0.1, 450.0, 4, 8)
    keep = M._Inputs([geom, lor], scalars, "cuda:0")
    assert keep.same([geom.copy(), lor.copy()], scalars, "cuda:0")
    assert keep.same([np.asfortranarray(geom), lor], scalars, "cuda:0")  # same values, another memory order
    nudged = geom.copy()
    nudged[1, 2, 0] = np.nextafter(nudged[1, 2, 0], 2.0)
    assert not keep.same([nudged, lor], scalars, "cuda:0")
    assert not keep.same([geom, lor.astype(np.int32)], scalars, "cuda:0")
    assert not keep.same([geom[:3], lor], scalars, "cuda:0")
    assert not keep.same([geom, lor], (0.1, 450.0, 4, 16), "cuda:0")
    assert not keep.same([geom, lor], scalars, "cuda:1")
    # the copies are the cache's own: changing the caller's array afterwards is a change
    geom[0, 0, 0] += 1.0
    assert not keep.same([geom, lor], scalars, "cuda:0")


def test_engine_cache_matches_nan_inputs_bitwise():
    M = _module()
    a = np.array([1.0, np.nan, 3.0, 4.0, 5.0])  # 40 bytes: compared 8 at a time
    b = np.array([1, 2, 3], dtype=np.int8)      # 3 bytes: compared one at a time
    keep = M._Inputs([a, b], (), "cuda:0")
    assert keep.same([a.copy(), b.copy()], (), "cuda:0")
