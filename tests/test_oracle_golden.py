"""Pin the CPU oracle to the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the unmodified reference)."""

import numpy as np
import pytest

from conftest import golden, problem_from_golden, rel_l2
from oracle import oracle as O

# full-size slice: the reference's float32 sums over 218 points per cell against
# FP64 (measured 2.3e-7 relative L2 on the kept cells, 2.0e-7 on the bin totals)
SLICE_TOL = 1e-6


def _ulp_close(a, b, ulps=4):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    tol = ulps * np.spacing(np.maximum(np.abs(a), np.abs(b)))
    return np.all(np.abs(a - b) <= tol)


@pytest.mark.parametrize("case", range(4))
def test_oracle_rays_match_reference(case):
    g = golden("rays")
    grid, gb, lines = g[f"grid{case}"], g[f"bounds{case}"], g[f"lines{case}"]
    cnt_ref = g[f"count{case}"]
    cnt, ln, ix, sm = O.trace_batch(grid, gb, lines, allow_overrun=True)
    # overruns (reference IndexError) are flagged, everything else matches
    assert np.array_equal(cnt < 0, cnt_ref < 0)
    ok = cnt_ref >= 0
    assert np.array_equal(cnt[ok], cnt_ref[ok])
    for i in np.where(ok & (cnt_ref > 0))[0]:
        n = cnt_ref[i]
        assert np.array_equal(ix[i, :n], g[f"idx{case}"][i, :n]), i
        # the interpreted reference squares through libm pow(); the oracle
        # multiplies (as numba does): lengths agree to a few ulp
        assert _ulp_close(ln[i, :n], g[f"len{case}"][i, :n]), i
        assert _ulp_close(sm[i, :n], g[f"samples{case}"][i, :n], ulps=16), i


def test_rays_fixture_has_edge_cases():
    g = golden("rays")
    allc = np.concatenate([g[f"count{c}"] for c in range(int(g["ncases"]))])
    assert (allc == 0).sum() > 50          # misses
    assert (allc < 0).sum() > 0            # reference overruns
    assert (allc > 0).sum() > 1000


EDGE = ["sss_edge_empty_mu", "sss_edge_empty_act", "sss_edge_one_ring", "sss_edge_one_crystal",
        "sss_edge_step_past_volume"]


@pytest.mark.parametrize("name", ["sss_tiny_b1", "sss_tiny_b3", "sss_tiny_b5", "sss_tiny_nx14_ny10",
                                  "sss_tiny_wide", "sss_tiny_far", "sss_wide_body_tof13", "sss_tiny_even_aniso"]
                         + EDGE)
def test_oracle_sss_matches_reference(name, att_table):
    g = golden(name)
    pr = problem_from_golden(g)
    cmp = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                        pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                        pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                        pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                        pr.nr_bins)
    ref = g["compact"]
    assert np.array_equal(cmp != 0, ref != 0)
    # reference accumulates in float32, the oracle in FP64
    assert rel_l2(cmp, ref) < 1e-6


@pytest.mark.slow
def test_oracle_sss_nontof_40x40x20_matches_reference(att_table):
    g = golden("sss_nontof_40x40x20")
    pr = problem_from_golden(g)
    cmp = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                        pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                        pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                        pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                        pr.nr_bins)
    ref = g["compact"]
    assert np.array_equal(cmp != 0, ref != 0)
    assert rel_l2(cmp, ref) < 1e-6


@pytest.mark.parametrize("case", range(4))
def test_oracle_mask_matches_reference(case):
    from opensss_gb300.geometry import SinogramCoordinates

    g = golden("mask")
    nd, nr, af = (int(v) for v in g[f"case{case}_dims"])
    lor, si, _ = SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    m = O.mask(g[f"case{case}_mu"], g[f"case{case}_bounds"], g[f"case{case}_geometry"], lor, si, af)
    assert np.array_equal(m, g[f"case{case}_mask"])


@pytest.mark.parametrize("case", range(2))
def test_oracle_fit_matches_reference(case):
    from opensss_gb300.geometry import SinogramCoordinates

    g = golden("fit")
    nd, nr, af = (int(v) for v in g[f"case{case}_dims"])
    lor, si, _ = SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    s = O.fit(g[f"case{case}_prompts"], g[f"case{case}_scatter"], g[f"case{case}_randoms"],
              g[f"case{case}_mask"], g[f"case{case}_grid"], g[f"case{case}_bounds"],
              g[f"case{case}_geometry"], lor, si, af)
    ref = g[f"case{case}_scale"]
    assert abs(float(s[0]) - float(ref[0])) <= 1e-5 * abs(float(ref[0]))


@pytest.mark.parametrize("name", ["mask", "scatter", "trues"])
def test_oracle_fit_degenerate_inputs(name):
    """No masked LOR, no scatter, or prompts below the randoms everywhere:
    the reference's lstsq gives a scale of 0."""
    from opensss_gb300.geometry import SinogramCoordinates

    g = golden("fit")
    nd, nr, af = (int(v) for v in g["case0_dims"])
    lor, si, _ = SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    prm, scat, mask = g["case0_prompts"], g["case0_scatter"], g["case0_mask"]
    prm, scat, mask = {"mask": (prm, scat, 0 * mask), "scatter": (prm, 0 * scat, mask),
                       "trues": (0 * prm, scat, mask)}[name]
    s = O.fit(prm, scat, g["case0_randoms"], mask, g["case0_grid"], g["case0_bounds"], g["case0_geometry"], lor,
              si, af)
    assert float(g[f"edge_no_{name}_scale"][0]) == 0.0
    assert float(s[0]) == 0.0


@pytest.mark.parametrize("case", range(2))
def test_oracle_upsample_matches_reference(case):
    from opensss_gb300 import geometry as G

    g = golden("upsample")
    nd, nr, nru, ndu, nb = (int(v) for v in g[f"case{case}_dims"])
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    det = G.sampled_detectors(nd, ndu)
    lut = G.upsample_source(lor, det)
    rmap = G.ring_nearest(nr, G.sampled_rings(nr, nru))
    cmp = g[f"case{case}_compact"].astype(np.float64)
    bins = []
    for b in range(nb):
        bins.append(O.upsample_bin(cmp[b], nru, ndu, nr, nd, lut, rmap, si))
    assert np.array_equal(np.stack(bins), g[f"case{case}_bins"])
    assert np.allclose(np.sum(bins, axis=0), g[f"case{case}_sum"], rtol=1e-6, atol=0)


def test_oracle_rejects_tof_offsets_past_the_table_as_the_reference_does(att_table):
    """A 2 m wide body in a 1.5 m ring: the reference indexes its 8001-entry
    TOF table past the end and raises IndexError (recorded in the fixture);
    the oracle reports status -2 for the same problem (the engine:
    SSS_ERR_TOF_RANGE)."""
    g = golden("sss_tofrange")
    assert str(g["reference_error"]).startswith("IndexError")
    pr = problem_from_golden(g)
    with pytest.raises(RuntimeError, match="status -2"):
        O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                      pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                      pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                      pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                      pr.nr_bins)


@pytest.mark.slow
def test_oracle_sss_tof13_slice_matches_reference(att_table):
    """One sampled z-slice of the 13-bin, 64x64x48 @ 6 mm workload on the
    760 x 80 scanner (16 x 48 sampled): the reference's own driver restricted
    to that slice, against the oracle over the same scatter points.  The
    reference adds each term into float32, the oracle in FP64."""
    from opensss_gb300 import workloads as W

    g = golden("sss_tof13_slice")
    pr = W.tof13_64x64x48(seed=0)
    _, sl = O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)
    idx = np.flatnonzero(sl == int(g["z_index"]))
    assert len(idx) > 100 and np.all(np.diff(idx) == 1)
    cmp = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry, pr.scanner.normals,
                        pr.scanner.detector_size_mm, att_table, pr.energy_resolution, pr.energy_threshold,
                        pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step, pr.tof_resolution,
                        pr.tof_range, pr.nr_bins, sp_begin=int(idx[0]), sp_end=int(idx[-1]) + 1)
    assert tuple(cmp.shape) == tuple(g["shape"])
    flat = cmp.reshape(cmp.shape[0], -1)
    got, ref = flat[:, g["cells"]], g["values"]
    # the reference adds each term into float32, where terms below ~7e-46 round
    # to 0; FP64 keeps their sums (at most ~1e-45): zero-ness may differ there only
    tiny = 1e-25 * float(np.abs(ref).max())
    differ = (got != 0) != (ref != 0)
    assert not np.any(differ & ((np.abs(got) > tiny) | (np.abs(ref) > tiny)))
    assert int(np.count_nonzero(flat.any(axis=0))) == int(g["contributing"])
    assert rel_l2(got, ref) < SLICE_TOL
    np.testing.assert_allclose(flat.sum(axis=1), g["bin_totals"], rtol=SLICE_TOL)


def test_oracle_point_list_matches_ranges(att_table):
    """The oracle's explicit point list: all points equal the full run, the
    first ten equal the range cut, and a list that is not ascending is an
    error."""
    g = golden("sss_tiny_b5")
    pr = problem_from_golden(g)
    args = (pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry, pr.scanner.normals,
            pr.scanner.detector_size_mm, att_table, pr.energy_resolution, pr.energy_threshold,
            pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
            pr.nr_bins)
    n = len(O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)[0])
    assert np.array_equal(O.sss_compact(*args, points=np.arange(n)), O.sss_compact(*args))
    assert np.array_equal(O.sss_compact(*args, points=np.arange(10)), O.sss_compact(*args, sp_end=10))
    with pytest.raises(RuntimeError, match="status -5"):
        O.sss_compact(*args, points=np.array([3, 2]))


@pytest.mark.parametrize("case", range(4))
def test_oracle_mask_threshold_rule(case):
    """The oracle's bound on the attenuation factor: a bound just above 1
    gives exactly the reference's tails; a larger bound only adds LORs, and
    on a faint map it adds crossing LORs whose factor lies below it."""
    g = golden("mask")
    nd, nr, af = (int(v) for v in g[f"case{case}_dims"])
    from opensss_gb300 import geometry as G

    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    mu, b, geo = g[f"case{case}_mu"], g[f"case{case}_bounds"], g[f"case{case}_geometry"]
    ref = g[f"case{case}_mask"]
    assert np.array_equal(O.mask(mu, b, geo, lor, si, af), ref)
    tight = O.mask(mu, b, geo, lor, si, af, acf_below=1.0 + 1e-15)
    assert np.array_equal(tight, ref)
    assert np.all(O.mask(mu, b, geo, lor, si, af, acf_below=1.03) >= ref)
    # a faint map (2% of the values) puts many crossing LORs between 1 and 1.03
    faint = (mu * np.float32(0.02)).astype(np.float32)
    exact = O.mask(faint, b, geo, lor, si, af)
    loose = O.mask(faint, b, geo, lor, si, af, acf_below=1.03)
    assert np.all(loose >= exact)
    if mu.max() > 0:  # one fixture is the empty map, where every LOR is a tail either way
        assert loose.sum() > exact.sum()


def test_gpu_oracle_library_builds_and_exports_its_entry_point():
    """The FP64 GPU oracle (oracle/sss_oracle_gpu.cu) cross-compiles for
    sm_103a here and loads without a GPU; its runs are the -m gpu tests."""
    assert hasattr(O.gpu_lib(), "orc_sss_gpu")
