"""GPU upsampling, tail mask and back-projection fit against the reference's outputs."""

import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _sino(nd, nr):
    from opensss_gb300.geometry import SinogramCoordinates

    return SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)


@pytest.mark.parametrize("case", range(2))
def test_interpolate_scatters_matches_reference(cuda_ok, tmp_path, case):
    from opensss_gb300.Interpolation import InterpolateScatters

    g = golden("upsample")
    nd, nr, nru, ndu, nb = (int(v) for v in g[f"case{case}_dims"])
    lor, si, _ = _sino(nd, nr)
    dense = O.densify(g[f"case{case}_compact"].astype(np.float64), lor, nd, nru, ndu)
    out = InterpolateScatters(dense, nr, nru, nd, ndu, lor, si, str(tmp_path), False)
    assert out.dtype == np.float32
    assert np.array_equal(out, g[f"case{case}_sum"])  # bit-exact, bins summed in order
    for b in range(nb):
        saved = np.load(tmp_path / f"SSS_mashed_bin{b}.npz")["arr_0"]
        assert np.array_equal(saved, g[f"case{case}_bins"][b])


def test_upsample_from_engine_layout(cuda_ok):
    """The engine's leg-pair output upsamples to the same sinogram."""
    import torch

    from opensss_gb300 import geometry as G
    from opensss_gb300.Interpolation import upsample_device

    g = golden("upsample")
    nd, nr, nru, ndu, nb = (int(v) for v in g["case0_dims"])
    lor, si, _ = _sino(nd, nr)
    cmp = g["case0_compact"]
    lp = cmp.reshape(nb, nru, nru, ndu, ndu).transpose(0, 3, 1, 4, 2).reshape(nb, nru * ndu, nru * ndu)
    t = G.upsample_tables(lor, si, nru, ndu, "legpair")
    out = upsample_device(torch.from_numpy(np.ascontiguousarray(lp)).cuda(), t, nb,
                          (nd + 1) * (nd // 2), nr * nr)
    assert np.array_equal(out.cpu().numpy().reshape(nd + 1, nd // 2, nr * nr), g["case0_sum"])


@pytest.mark.parametrize("case", range(4))
def test_tail_mask_matches_reference_bit_exact(cuda_ok, case):
    from opensss_gb300.TailsMask import MaskGenerator

    g = golden("mask")
    nd, nr, af = (int(v) for v in g[f"case{case}_dims"])
    lor, si, _ = _sino(nd, nr)
    mu = g[f"case{case}_mu"]
    m = MaskGenerator(np.ones_like(mu), mu, g[f"case{case}_bounds"], g[f"case{case}_geometry"], lor,
                      si, True, af)
    assert m.dtype == np.uint8
    assert np.array_equal(m, g[f"case{case}_mask"])


def test_tail_mask_tables_out_of_range_are_an_error(cuda_ok):
    """A slice table entry past the nr^2 slices (sss_tail_mask), a ring-pair
    entry with a ring past the scanner or a slice past nslices
    (sss_tail_mask_pairs) and LOR coordinates past the sinogram set
    SSS_ERR_TABLE; those LORs are skipped, the others marked as before."""
    import ctypes as C

    import torch

    from opensss_gb300 import _lib
    from opensss_gb300.engine import fortran_flat

    def ptr(t):
        return C.c_void_p(t.data_ptr())

    g = golden("mask")
    nd, nr, af = (int(v) for v in g["case0_dims"])
    lor, si, _ = _sino(nd, nr)
    mu = fortran_flat(g["case0_mu"], torch.device("cuda"))
    grid = np.array(g["case0_mu"].shape, np.int32)
    bounds = np.ascontiguousarray(np.asarray(g["case0_bounds"], np.float64).reshape(-1)[:6])
    geom = torch.from_numpy(np.ascontiguousarray(g["case0_geometry"], np.float64)).cuda()
    lor_t = torch.from_numpy(np.ascontiguousarray(lor, np.int16)).cuda()
    L = _lib.lib()
    args = (grid.ctypes.data_as(C.c_void_p), bounds.ctypes.data_as(C.c_void_p), ptr(mu), 0, nr, nd, ptr(geom))
    ncell = (nd + 1) * (nd // 2)

    def mask(lor_dev, si_np):
        out = torch.zeros((ncell, nr * nr), dtype=torch.uint8, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        si_dev = torch.from_numpy(np.ascontiguousarray(si_np[:nr, :nr], np.int16)).cuda()
        assert L.sss_tail_mask(*args, ptr(lor_dev), ptr(si_dev), af, 0.0, ptr(out), ptr(st), None) == 0
        torch.cuda.synchronize()
        return out.cpu().numpy(), int(st.item())

    good, st = mask(lor_t, si)
    assert st == 0 and np.array_equal(good.reshape(g["case0_mask"].shape), g["case0_mask"])
    bad_si = np.array(si[:nr, :nr], np.int64)
    bad_si[0, 1] = nr * nr
    got, st = mask(lor_t, bad_si)
    assert L.sss_status_code(st) == 11
    keep = np.ones(nr * nr, bool)
    keep[int(si[0, 1])] = False  # the slice whose LORs were skipped
    assert np.array_equal(got[:, keep], good[:, keep]) and not got[:, ~keep].any()
    bad_lor = lor_t.clone()
    bad_lor[0, af, 1] = nd + 1  # one past the last radius
    _, st = mask(bad_lor, si)
    assert L.sss_status_code(st) == 11

    pairs = np.array([[0, 1, 0], [1, 0, 1], [nr, 0, 2], [0, 0, 7]], np.int32)  # a bad ring, a bad slice
    pairs_dev = torch.from_numpy(pairs).cuda()
    out = torch.zeros((ncell, 3), dtype=torch.uint8, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.sss_tail_mask_pairs(*args, ptr(lor_t), ptr(pairs_dev), len(pairs), 3, af, 0.0, ptr(out), ptr(st),
                                 None) == 0
    torch.cuda.synchronize()
    assert L.sss_status_code(int(st.item())) == 11
    assert not out[:, 2].any()


def test_activity_mask_matches_oracle(cuda_ok):
    """UseAttenuation=False marks LORs that see no activity (TailsMask.py:153-161)."""
    from opensss_gb300 import workloads as W
    from opensss_gb300.TailsMask import MaskGenerator

    g = golden("mask")
    nd, nr, af = (int(v) for v in g["case0_dims"])
    lor, si, _ = _sino(nd, nr)
    mu = g["case0_mu"]
    act, _, _ = W.cylinder_phantom(mu.shape, 2.0, seed=0, radius_cm=3.0)  # activity in a 3 cm core
    m_act = MaskGenerator(act, mu, g["case0_bounds"], g["case0_geometry"], lor, si, False, af)
    ref = O.mask(act, g["case0_bounds"], g["case0_geometry"], lor, si, af, use_activity=True)
    assert np.array_equal(m_act, ref)
    m_mu = MaskGenerator(act, mu, g["case0_bounds"], g["case0_geometry"], lor, si, True, af)
    assert np.all(m_act >= m_mu) and m_act.sum() > m_mu.sum()


@pytest.mark.parametrize("case", range(2))
def test_backprojection_fit_matches_reference(cuda_ok, case):
    from opensss_gb300.BackProjection import BackProjectionScatterRandFit

    g = golden("fit")
    nd, nr, af = (int(v) for v in g[f"case{case}_dims"])
    lor, si, _ = _sino(nd, nr)
    s = BackProjectionScatterRandFit(g[f"case{case}_prompts"], g[f"case{case}_scatter"],
                                     g[f"case{case}_randoms"], g[f"case{case}_mask"],
                                     g[f"case{case}_grid"], g[f"case{case}_bounds"],
                                     g[f"case{case}_geometry"], lor, si[:nr, :nr].T, af)
    ref = g[f"case{case}_scale"]
    assert s.dtype == np.float32 and s.shape == (1,)
    assert abs(float(s[0]) - float(ref[0])) <= 1e-5 * abs(float(ref[0]))


@pytest.mark.parametrize("name", ["mask", "scatter", "trues"])
def test_backprojection_fit_degenerate_inputs(cuda_ok, name):
    """No masked LOR, no scatter, or prompts below the randoms everywhere:
    a scale of 0, as the reference's lstsq gives."""
    from opensss_gb300.BackProjection import BackProjectionScatterRandFit

    g = golden("fit")
    nd, nr, af = (int(v) for v in g["case0_dims"])
    lor, si, _ = _sino(nd, nr)
    prm, scat, mask = g["case0_prompts"], g["case0_scatter"], g["case0_mask"]
    prm, scat, mask = {"mask": (prm, scat, 0 * mask), "scatter": (prm, 0 * scat, mask),
                       "trues": (0 * prm, scat, mask)}[name]
    s = BackProjectionScatterRandFit(prm, scat, g["case0_randoms"], mask, g["case0_grid"], g["case0_bounds"],
                                     g["case0_geometry"], lor, si[:nr, :nr].T, af)
    assert float(g[f"edge_no_{name}_scale"][0]) == 0.0
    assert s.dtype == np.float32 and s.shape == (1,) and float(s[0]) == 0.0


def test_fit_reads_upsampled_scatter_without_materialising(cuda_ok):
    """Fused path: the fit reads the sampled (leg-pair) sinogram through the
    upsampling tables; same scale as fitting the materialised upsampled
    sinogram with the FP64 oracle."""
    import torch

    from opensss_gb300 import geometry as G, workloads as W
    from opensss_gb300.BackProjection import fit_device

    g = golden("upsample")
    nd, nr, nru, ndu, nb = (int(v) for v in g["case1_dims"])
    lor, si, _ = _sino(nd, nr)
    cmp = g["case1_compact"]
    lp = cmp.reshape(nb, nru, nru, ndu, ndu).transpose(0, 3, 1, 4, 2).reshape(nb, nru * ndu, nru * ndu)
    up = g["case1_bins"][0]
    sc = W.ring_scanner(nd, nr, radius_cm=20.3, ring_pitch_cm=1.1)
    rng = np.random.default_rng(3)
    shp = up.shape
    prm = rng.poisson(3.0, size=shp).astype(np.float32)
    rnd = np.full(shp, 0.1, np.float32)
    mask = (rng.uniform(size=shp) < 0.5).astype(np.float32)
    grid = np.array([10, 10, 8])
    bounds = np.array([-8.0, -8.0, -6.0, 8.0, 8.0, 6.0])
    order = si[:nr, :nr].T
    ref = O.fit(prm, up, rnd, mask, grid, bounds, sc.geometry, lor, si, 1)  # the oracle transposes
    cell, ring, _ = G.upsample_tables(lor, si, nru, ndu, "legpair")
    dev = "cuda"
    flat = lambda a: torch.from_numpy(np.ascontiguousarray(a.reshape(-1, nr * nr))).to(dev)  # noqa: E731
    s = fit_device(flat(prm), flat(rnd), flat(mask),
                   torch.from_numpy(np.ascontiguousarray(lp[0])).to(dev), cell, ring, grid, bounds,
                   sc.geometry, lor, order, 1, scat_clamp=True)
    assert abs(s - float(ref[0])) <= 1e-5 * abs(float(ref[0]))


@pytest.mark.parametrize("case,nb", [(0, 3), (1, 3), (0, 4)])
def test_all_bins_in_one_pass_match_per_bin_fits(cuda_ok, case, nb):
    """sss_backproject_fit_bins gives every bin the scale of its own fit: bins
    paired into shared vector images, an odd last bin on its own, and bins of
    a pair that skip different LORs."""
    import torch

    from opensss_gb300.BackProjection import fit_bins_device, fit_device

    g = golden("fit")
    nd, nr, af = (int(v) for v in g[f"case{case}_dims"])
    lor, si, _ = _sino(nd, nr)
    shp = g[f"case{case}_scatter"].shape
    ncell, nsl = shp[0] * shp[1], shp[2]
    rng = np.random.default_rng(case)
    factors = (1.0, 0.5, 2.0, 0.8)[:nb]
    scat = np.stack([g[f"case{case}_scatter"] * f for f in factors])
    scat[1][rng.uniform(size=shp) < 0.2] = 0  # bins skip different LORs
    if nb > 3:
        scat[2][rng.uniform(size=shp) < 0.3] = 0
    prm = np.stack([rng.poisson(3.0 * f, size=shp).astype(np.float32) for f in (1.0, 0.7, 1.5, 1.2)[:nb]])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.reshape(-1, ncell, nsl))).cuda()  # noqa: E731
    cell = np.arange(ncell, dtype=np.int64) * nsl
    ring = np.arange(nsl, dtype=np.int64)
    rnd = dev(g[f"case{case}_randoms"])[0]
    mask = dev(g[f"case{case}_mask"])[0]
    order = si[:nr, :nr].T
    got = fit_bins_device(dev(prm), rnd, mask, dev(scat).reshape(-1), ncell * nsl, cell, ring,
                          g[f"case{case}_grid"], g[f"case{case}_bounds"], g[f"case{case}_geometry"], lor, order, af)
    for b in range(nb):
        ref = fit_device(dev(prm)[b], rnd, mask, dev(scat)[b], cell, ring, g[f"case{case}_grid"],
                         g[f"case{case}_bounds"], g[f"case{case}_geometry"], lor, order, af)
        assert abs(float(got[b]) - ref) <= 1e-5 * abs(ref)


def test_scale_scatters_to_prompts_dropin(cuda_ok, tmp_path):
    """Scaling.ScaleScattersToPrompts from the saved files equals the per-bin
    BackProjectionScatterRandFit calls of the reference's loop."""
    from opensss_gb300.BackProjection import BackProjectionScatterRandFit
    from opensss_gb300.Scaling import ScaleScattersToPrompts

    g = golden("fit")
    nd, nr, af = (int(v) for v in g["case1_dims"])
    lor, si, _ = _sino(nd, nr)
    shp = g["case1_scatter"].shape
    rng = np.random.default_rng(9)
    bins = 3
    prompts = rng.poisson(3.0, size=shp + (bins,)).astype(np.uint16)
    lorcounts = np.full(shp, 1.0, np.float32)
    np.savez_compressed(tmp_path / "PromptsSinogram.npz", prompts)
    np.savez_compressed(tmp_path / "RandomsSinogram.npz", g["case1_randoms"])
    np.save(tmp_path / "AttenuationMask.npy", (g["case1_mask"] >= 1).astype(np.uint8))
    for b in range(bins):
        np.savez_compressed(tmp_path / f"SSS_mashed_bin{b}", g["case1_scatter"] * (b + 1))
    s = ScaleScattersToPrompts(si, lor, str(tmp_path), g["case1_grid"], g["case1_bounds"], g["case1_geometry"],
                               np.array([]), af, False, lorcounts)
    assert s.dtype == np.float32 and s.shape == (bins,)
    order = si[:nr, :nr].T
    for b in range(bins):
        ref = BackProjectionScatterRandFit(prompts[..., b] / lorcounts, g["case1_scatter"] * (b + 1),
                                           g["case1_randoms"], np.float32(g["case1_mask"] >= 1), g["case1_grid"],
                                           g["case1_bounds"], g["case1_geometry"], lor, order, af)
        assert abs(float(s[b]) - float(ref[0])) <= 1e-5 * abs(float(ref[0]))
    assert np.array_equal(np.load(tmp_path / "ScaleFactors.npy"), s)


def test_tail_mask_with_signed_map_matches_oracle(cuda_ok):
    """A map with negative values disables the early decision (the line
    integral can shrink back); the mask still equals the FP64 oracle's."""
    from opensss_gb300.TailsMask import MaskGenerator

    g = golden("mask")
    nd, nr, af = (int(v) for v in g["case0_dims"])
    lor, si, _ = _sino(nd, nr)
    mu = g["case0_mu"].copy()
    rng = np.random.default_rng(4)
    flip = rng.uniform(size=mu.shape) < 0.3
    mu[flip] = -mu[flip]  # lines through both signs can cancel
    m = MaskGenerator(np.ones_like(mu), mu, g["case0_bounds"], g["case0_geometry"], lor, si, True, af)
    ref = O.mask(mu, g["case0_bounds"], g["case0_geometry"], lor, si, af)
    assert np.array_equal(m, ref)


@pytest.mark.parametrize("case", range(4))
@pytest.mark.parametrize("bound", [1.03, 1.5])
def test_tail_mask_threshold_matches_oracle(cuda_ok, case, bound):
    """A bound on the attenuation factor instead of the reference's ACF == 1
    (the benchmark's non-TOF workload masks where the factor is below 1.03):
    bit-exact against the FP64 oracle's restatement of the same rule, and a
    superset of the reference's mask."""
    from opensss_gb300.TailsMask import MaskGenerator

    g = golden("mask")
    nd, nr, af = (int(v) for v in g[f"case{case}_dims"])
    lor, si, _ = _sino(nd, nr)
    for scale in (1.0, 0.02):  # the golden map, and a faint one with many factors in (1, bound)
        mu = (g[f"case{case}_mu"] * np.float32(scale)).astype(np.float32)
        m = MaskGenerator(np.ones_like(mu), mu, g[f"case{case}_bounds"], g[f"case{case}_geometry"], lor, si, True,
                          af, AttenuationThreshold=bound)
        ref = O.mask(mu, g[f"case{case}_bounds"], g[f"case{case}_geometry"], lor, si, af, acf_below=bound)
        assert np.array_equal(m, ref), scale
        assert np.all(m >= O.mask(mu, g[f"case{case}_bounds"], g[f"case{case}_geometry"], lor, si, af))
