"""GPU ray tracer (sss_raytrace) against the reference's outputs."""

import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _ulp_close(a, b, ulps=4):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.all(np.abs(a - b) <= ulps * np.spacing(np.maximum(np.abs(a), np.abs(b))))


@pytest.mark.parametrize("case", range(4))
def test_tof_tracer_matches_reference(cuda_ok, case):
    from opensss_gb300 import RayTracing3DTOFBatch

    g = golden("rays")
    grid, gb, lines = g[f"grid{case}"], g[f"bounds{case}"], g[f"lines{case}"]
    cnt, ln, ix, sm = RayTracing3DTOFBatch(grid, gb, lines)
    cref = g[f"count{case}"]
    assert np.array_equal(cnt, cref)  # including -1 where the reference overruns
    ocnt, oln, oix, osm = O.trace_batch(grid, gb, lines, allow_overrun=True)
    for i in np.where(cref > 0)[0]:
        n = cref[i]
        assert np.array_equal(ix[i, :n], g[f"idx{case}"][i, :n])  # bit-exact indices
        assert np.array_equal(ln[i, :n], oln[i, :n])  # same FP64 operations as the oracle
        assert np.array_equal(sm[i, :n], osm[i, :n])
        assert _ulp_close(ln[i, :n], g[f"len{case}"][i, :n])
        assert _ulp_close(sm[i, :n], g[f"samples{case}"][i, :n], ulps=16)


@pytest.mark.parametrize("case", range(4))
def test_nontof_tracer_matches_mex(cuda_ok, case):
    from opensss_gb300 import RayTracing3DBatch

    g = golden("rays")
    grid, gb, lines = g[f"grid{case}"], g[f"bounds{case}"], g[f"lines{case}"]
    cnt, ln, ix = RayTracing3DBatch(grid, gb, lines)
    cref = g[f"count_nontof{case}"]
    ok = cref >= 0
    assert np.array_equal(cnt[ok], cref[ok])
    for i in np.where(cref > 0)[0]:
        n = cref[i]
        assert np.array_equal(ix[i, :n], g[f"idx_nontof{case}"][i, :n])
        a, b = ln[i, :n], g[f"len_nontof{case}"][i, :n]
        assert np.all(np.abs(a - b) <= np.spacing(np.maximum(np.abs(a), np.abs(b))))


def test_single_ray_dropin(cuda_ok):
    from opensss_gb300 import RayTracing3DTOF

    g = golden("rays")
    grid, gb, lines = g["grid1"], g["bounds1"], g["lines1"]
    cref = g["count1"]
    for i in list(np.where(cref > 0)[0][:5]) + list(np.where(cref == 0)[0][:2]):
        ln, ix, sm = RayTracing3DTOF(grid, gb, lines[i])
        assert ix.dtype == np.int32 and ln.dtype == np.float64
        assert len(ln) == cref[i]
        assert np.array_equal(ix, g["idx1"][i, :cref[i]])
    bad = np.where(cref < 0)[0]
    if len(bad):
        with pytest.raises(IndexError):
            RayTracing3DTOF(grid, gb, lines[bad[0]])


def test_large_batch_property(cuda_ok):
    """1M random rays: indices and counts identical to the oracle, lengths sum
    to the clipped segment length."""
    from opensss_gb300 import RayTracing3DTOFBatch

    rng = np.random.default_rng(3)
    grid = np.array([64, 64, 48])
    gb = np.array([-19.2, -19.2, -14.4, 19.2, 19.2, 14.4])
    n = 200_000
    lines = np.concatenate([rng.uniform(-25, 25, (n, 3)), rng.uniform(-25, 25, (n, 3))], axis=1)
    cnt, ln, ix, sm = RayTracing3DTOFBatch(grid, gb, lines)
    ocnt, oln, oix, osm = O.trace_batch(grid, gb, lines, allow_overrun=True)
    assert np.array_equal(cnt, ocnt)
    assert np.array_equal(ix, oix)
    assert np.array_equal(ln, oln)
