"""Span (axial mashing) and mash (angular) host tables against the reference's
own outputs (tests/golden/span.npz, made by tests/golden/make_golden.py)."""

import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O


@pytest.mark.parametrize("case", range(4))
def test_sinogram_lut_matches_reference(case):
    from opensss_gb300.DataReduction import SinogramLUT

    g = golden("span")
    nr, span, mrd = (int(v) for v in g[f"lut{case}_args"])
    si, ring_lut, lut, counts = SinogramLUT(nr, span, None if mrd < 0 else mrd)
    assert si.dtype == np.float32 and np.array_equal(si, g[f"lut{case}_index"])
    assert np.array_equal(ring_lut, g[f"lut{case}_ringlut"])
    assert lut.dtype == np.int16 and np.array_equal(lut, g[f"lut{case}_table"])
    assert np.array_equal(counts, g[f"lut{case}_counts"])


def test_sinogram_lut_keeps_the_reference_error():
    """Ring counts the reference's sinogram count cannot hold raise IndexError there too."""
    from opensss_gb300.DataReduction import SinogramLUT

    with pytest.raises(IndexError):
        SinogramLUT(8, 3, 7)


def test_expand_and_mash_geometry():
    from opensss_gb300.geometry import expandRings, mashDetectors

    g = golden("span")
    eg, en = expandRings(g["geom_in"], g["normals_in"])
    assert np.array_equal(eg, g["geom_expanded"]) and np.array_equal(en, g["normals_expanded"])
    mg, mn = mashDetectors(g["geom_in"], g["normals_in"], 2)
    assert np.allclose(mg, g["geom_mashed2"], rtol=0, atol=1e-13)
    assert np.allclose(mn, g["normals_mashed2"], rtol=0, atol=1e-13)
    with pytest.raises(Exception):
        mashDetectors(g["geom_in"], g["normals_in"], 5)


def test_sum_lor_counts():
    from opensss_gb300.DataReduction import SinogramLUT, SumLORsCounts

    g = golden("span")
    si, _, lut, counts = SinogramLUT(6, 3, 5)
    got = SumLORsCounts(g["geom_in"], lut, si, 2, 3, counts.shape[0])
    assert got.dtype == np.float32 and np.array_equal(got, g["lorcounts"])


def test_span_ring_pairs_use_float32_doubling():
    from opensss_gb300.DataReduction import SinogramLUT, span_ring_pairs

    si, ring_lut, _, _ = SinogramLUT(10, 3, 9)
    pairs = span_ring_pairs(si)
    assert pairs.shape == (si.shape[0], 3)
    assert np.array_equal(pairs[:, 2], np.arange(si.shape[0]))
    assert ring_lut[pairs[:, 0], pairs[:, 1]].all()
    assert pairs[:, :2].max() <= 2 * 10 - 2


@pytest.mark.parametrize("layout", ["dense", "legpair"])
def test_span_upsampling_tables_reproduce_reference(layout):
    """Gathering the sampled sinogram through the span tables gives the
    reference's InterpolateAllBinsSpan output bit for bit."""
    from opensss_gb300 import DataReduction as D, geometry as G
    from opensss_gb300.engine import compact_to_leg_pair

    g = golden("span")
    nd, nr, nru, ndu, nb, span, mrd = (int(v) for v in g["up_dims"])
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    si, _, _, _ = D.SinogramLUT(nr, span, mrd)
    cmp = g["up_compact"]
    if layout == "dense":
        src = O.densify(cmp.astype(np.float64), lor, nd, nru, ndu).astype(np.float32)
    else:
        src = compact_to_leg_pair(cmp, nru, ndu)
    t = G.span_upsample_tables(lor, si, nr, nru, ndu, layout)
    cell, ring, stride = t
    flat = src.reshape(-1)
    idx = cell[:, None] + ring[None, :]
    total = np.zeros(idx.shape, np.float32)
    for b in range(nb):
        vb = np.maximum(flat[b * stride + idx], 0)
        assert np.array_equal(vb.reshape(nd + 1, nd // 2, -1), g["up_bins"][b])
        total += vb
    assert np.array_equal(total.reshape(nd + 1, nd // 2, -1), g["up_sum"])


@pytest.mark.parametrize("ci", range(2))
def test_oracle_span_mask_and_fit_match_reference(ci):
    """The C oracle's span mask (bit-exact, both rules) and length-weighted
    fit (1e-5) against the reference's outputs."""
    from opensss_gb300 import DataReduction as D, geometry as G

    g = golden("span")
    nd, nr, span, af = (int(v) for v in g[f"case{ci}_dims"])
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    si, _, _, _ = D.SinogramLUT(nr, span, nr - 1)
    eg, _ = G.expandRings(g[f"case{ci}_geometry"], np.zeros_like(g[f"case{ci}_geometry"]))
    pairs = D.span_ring_pairs(si)
    m = O.mask_pairs(g[f"case{ci}_mu"], g[f"case{ci}_bounds"], eg, lor, pairs, si.shape[0], af)
    assert np.array_equal(m, g[f"case{ci}_mask"])
    ma = O.mask_pairs(g[f"case{ci}_act"], g[f"case{ci}_bounds"], eg, lor, pairs, si.shape[0], af,
                      use_activity=True)
    assert np.array_equal(ma, g[f"case{ci}_mask_activity"])
    s = O.fit_pairs(g[f"case{ci}_prompts"], g[f"case{ci}_scatter"], g[f"case{ci}_randoms"],
                    np.float32(g[f"case{ci}_mask"] >= 1), g[f"case{ci}_grid"], g[f"case{ci}_fit_bounds"], eg, lor,
                    pairs, af)
    ref = float(g[f"case{ci}_scale"][0])
    assert abs(float(s[0]) - ref) <= 1e-5 * abs(ref)
