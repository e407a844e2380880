"""GPU TOF-SSS (sss_tof_run) against the reference's outputs and the FP64 oracle.

Tolerance: 1e-4 relative L2 over the whole sampled sinogram, the bar the
engine is built to; the zero / non-zero pattern (which pairs and slices
contribute) must match exactly."""

import numpy as np
import pytest

from conftest import golden, problem_from_golden, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _engine(pr, att):
    from opensss_gb300 import TofSSS

    return TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att,
                  pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                  pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                  pr.nr_bins)


def _gpu_compact(pr, att, **kw):
    from opensss_gb300.engine import leg_pair_to_compact

    eng = _engine(pr, att)
    lp = eng.run(pr.activity, pr.attenuation, pr.image_size, **kw).cpu().numpy()
    return leg_pair_to_compact(lp, pr.nr_rings_used, pr.nr_detectors_used)


def _oracle_compact(pr, att, sp_end=-1):
    return O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                         pr.scanner.normals, pr.scanner.detector_size_mm, att,
                         pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                         pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                         pr.nr_bins, sp_end=sp_end)


def assert_same_support(got, ref, floor=1e-25):
    """Same set of contributing cells.  FP32 flushes TOF weights that are
    below ~1e-38 in FP64 to zero, so cells whose reference value is that far
    below the sinogram's peak may differ in zero-ness only."""
    tiny = floor * float(np.abs(ref).max())
    diff = (got != 0) != (ref != 0)
    assert not np.any(diff & (np.abs(ref) > tiny)), int(np.sum(diff & (np.abs(ref) > tiny)))
    assert not np.any(diff & (np.abs(got) > tiny))


def _valid_mask(nru, ndu):
    ri1 = np.arange(nru)[:, None, None, None]
    ri2 = np.arange(nru)[None, :, None, None]
    d1 = np.arange(ndu)[None, None, :, None]
    d2 = np.arange(ndu)[None, None, None, :]
    return ((d1 < d2) | ((d1 == d2) & (ri1 != ri2))).reshape(nru * nru, ndu, ndu)


@pytest.mark.parametrize("name", ["sss_tiny_b1", "sss_tiny_b3", "sss_tiny_b5", "sss_nontof_40x40x20",
                                  "sss_tiny_nx14_ny10", "sss_tiny_wide", "sss_tiny_even_aniso"])
def test_sss_matches_reference(cuda_ok, att_table, name):
    """sss_tiny_wide has bins 1.56 x the timing FWHM wide, so its weights take
    the per-bin 2^x evaluation; the other TOF cases take the factored one."""
    g = golden(name)
    pr = problem_from_golden(g)
    got = _gpu_compact(pr, att_table)
    ref = g["compact"]
    assert_same_support(got, ref)
    assert rel_l2(got, ref) < TOL
    # nothing outside the valid detector pairs
    assert not got[:, ~_valid_mask(pr.nr_rings_used, pr.nr_detectors_used)].any()


@pytest.mark.parametrize("name", ["sss_edge_empty_mu", "sss_edge_empty_act", "sss_edge_one_ring",
                                  "sss_edge_one_crystal", "sss_edge_step_past_volume"])
def test_degenerate_inputs_match_reference(cuda_ok, att_table, name):
    """No scatter point (empty attenuation map, sampling step past the
    volume), no activity, one sampled ring, one sampled crystal per ring
    (backscatter pairs only, efficiency 0): the reference's sinogram, which
    is all zero in every case but the single ring."""
    g = golden(name)
    pr = problem_from_golden(g)
    got = _gpu_compact(pr, att_table)
    ref = g["compact"]
    assert got.shape == ref.shape
    assert np.isfinite(got).all()
    if not ref.any():
        assert not got.any()
    else:
        assert_same_support(got, ref)
        assert rel_l2(got, ref) < TOL


def test_scatter_points_match_oracle(cuda_ok, att_table):
    from opensss_gb300 import workloads as W

    pr = W.tof13_64x64x48()
    eng = _engine(pr, att_table)
    from opensss_gb300.engine import fortran_flat

    act = fortran_flat(pr.activity, eng.device)
    mu = fortran_flat(pr.attenuation, eng.device)
    p = eng.problem(act, mu, pr.grid, pr.image_size)
    pts, counts = eng.scatter_points(p)
    xyz, sl = O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)
    pts = pts.cpu().numpy()
    assert len(pts) == len(xyz) == counts.sum()
    assert np.array_equal(pts[:, :3], xyz)
    assert np.array_equal(pts[:, 3].astype(np.int64), sl)


def test_tof13_whole_workload_against_fp64_oracle(cuda_ok, att_table):
    """The 13-bin benchmark workload (64x64x48 @ 6 mm, 760 x 80 scanner,
    16 x 48 sampled) over all 3,270 scatter points and 24 sampled z-slices:
    every slice's normalisation (:555-557) and the sum over slices (:201)
    enter, against the FP64 oracle on the host cores."""
    from opensss_gb300 import workloads as W

    pr = W.tof13_64x64x48()
    got = _gpu_compact(pr, att_table)
    ref = _oracle_compact(pr, att_table)
    assert_same_support(got, ref)
    assert rel_l2(got, ref) < TOL
    np.testing.assert_allclose(got.astype(np.float64).sum(axis=(1, 2, 3)), ref.sum(axis=(1, 2, 3)), rtol=TOL)


def test_tof33_stratified_sample_against_fp64_oracle(cuda_ok, att_table):
    """The 33-bin precision workload (128x128x96 @ 4 mm, 32 x 96 sampled): 48
    scatter points spread evenly over its 11,362 in lattice order (one or two
    in most of its 48 sampled z-slices); engine and oracle run the same point
    subset and normalise each slice over its kept points."""
    from opensss_gb300 import workloads as W

    pr = W.tof33_128x128x96()
    xyz, _ = O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)
    idx = W.stratified_points(len(xyz), 48)
    got = _gpu_compact(pr, att_table, points=idx)
    ref = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                        pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                        pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                        pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                        pr.nr_bins, points=idx)
    assert_same_support(got, ref)
    assert rel_l2(got, ref) < TOL


def test_point_subset_matches_oracle_subset(cuda_ok, att_table):
    """An uneven subset of points (some slices emptied, others thinned) is
    normalised per slice over the kept points, on the GPU as in the oracle."""
    g = golden("sss_tiny_b5")
    pr = problem_from_golden(g)
    xyz, sl = O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)
    idx = np.array([i for i in range(len(xyz)) if (i % 3 != 1) and sl[i] != sl[len(xyz) // 2]])
    got = _gpu_compact(pr, att_table, points=idx)
    ref = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                        pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                        pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                        pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                        pr.nr_bins, points=idx)
    assert_same_support(got, ref)
    assert rel_l2(got, ref) < TOL


def test_waves_do_not_change_the_result(cuda_ok, att_table):
    """Splitting the run into many waves of whole slices gives the same sums."""
    g = golden("sss_tiny_b5")
    pr = problem_from_golden(g)
    a = _gpu_compact(pr, att_table)
    b = _gpu_compact(pr, att_table, wave_points=1)  # one slice per wave
    assert rel_l2(b, a) < 1e-6


def test_run_on_a_side_stream(cuda_ok, att_table):
    """run(stream=s) with s not the current stream: the maps' copies, the
    buffers and the status reset are ordered on s, so the result is the
    default-stream run's."""
    import torch

    from opensss_gb300.engine import leg_pair_to_compact

    g = golden("sss_tiny_b3")
    pr = problem_from_golden(g)
    eng = _engine(pr, att_table)
    ref = eng.run(pr.activity, pr.attenuation, pr.image_size).cpu().numpy()
    side = torch.cuda.Stream(eng.device)
    got = eng.run(pr.activity, pr.attenuation, pr.image_size, stream=side).cpu().numpy()  # side synchronised
    assert rel_l2(got, ref) < 1e-6
    assert rel_l2(leg_pair_to_compact(got, pr.nr_rings_used, pr.nr_detectors_used), g["compact"]) < TOL


def test_dropin_dense_output(cuda_ok, att_table, tmp_path):
    from opensss_gb300 import SingleScatterSimulationTOF
    from opensss_gb300.geometry import SinogramCoordinates

    g = golden("sss_tiny_b3")
    pr = problem_from_golden(g)
    lor, _, _ = SinogramCoordinates(1, 1, 1, 1, pr.scanner.nr_detectors, pr.scanner.nr_rings,
                                    ID_Shidt=False)
    out = SingleScatterSimulationTOF(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                                     lor, pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                                     pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                                     pr.nr_detectors_used, pr.sample_step, pr.tof_resolution,
                                     pr.tof_range, pr.nr_bins, str(tmp_path))
    ref = O.densify(g["compact"].astype(np.float64), lor, pr.scanner.nr_detectors,
                    pr.nr_rings_used, pr.nr_detectors_used)
    assert out.dtype == np.float32
    assert out.shape == (pr.nr_bins, pr.scanner.nr_detectors + 1, pr.scanner.nr_detectors // 2,
                         pr.nr_rings_used ** 2)
    assert_same_support(out, ref)
    assert rel_l2(out, ref) < TOL
    assert (tmp_path / "Scatters_SSS.npz").exists()
    # a second call (the cached engine and device buffer) with twice the
    # activity: a fresh array, twice the first (the SSS is linear in the
    # activity), and the first result left as it was
    first = out.copy()
    out2 = SingleScatterSimulationTOF(2 * pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                                      lor, pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                                      pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                                      pr.nr_detectors_used, pr.sample_step, pr.tof_resolution,
                                      pr.tof_range, pr.nr_bins, None)
    assert out2 is not out and not np.shares_memory(out2, out)
    assert np.array_equal(out, first)
    assert rel_l2(out2, 2 * first) < 1e-6


def test_tof_bins_sum_to_nontof(cuda_ok, att_table):
    """TOF weights are normalised over bins: summing the TOF bins gives the
    non-TOF estimate of the same problem (size-independent property)."""
    from opensss_gb300 import workloads as W

    pr = W.tiny_problem(5, seed=9)
    tof = _gpu_compact(pr, att_table)
    pr1 = W.tiny_problem(5, seed=9)
    pr1.nr_bins, pr1.tof_resolution = 1, 1.0e6
    non = _gpu_compact(pr1, att_table)
    # weights only sum to one away from the table edges; the tiny scanner stays inside
    assert rel_l2(tof.sum(axis=0), non[0]) < 1e-4


@pytest.mark.parametrize("name", ["sss_tiny_b1", "sss_tiny_b5", "sss_tiny_wide", "sss_tiny_far",
                                  "sss_nontof_40x40x20"])
def test_kahan_reduction_matches_reference(cuda_ok, att_table, name):
    """The precision launch (SSS_FLAG_KAHAN: compensated sum over the scatter
    points, float-pair TOF offsets) stays within the same 1e-4 bar and is at
    least as close to the reference's own result as the plain launch."""
    g = golden(name)
    pr = problem_from_golden(g)
    plain = _gpu_compact(pr, att_table)
    kahan = _gpu_compact(pr, att_table, kahan=True)
    ref = g["compact"]
    assert_same_support(kahan, ref)
    assert rel_l2(kahan, ref) < TOL
    assert rel_l2(kahan, ref) <= 1.05 * rel_l2(plain, ref) + 1e-8


def test_precision_launch_against_fp64_oracle(cuda_ok, att_table):
    """96 scatter points spread over the 13-bin workload against the FP64
    oracle: the plain launch's error (~4e-6 relative L2, ~4e-5 on the worst
    bin) comes mostly from FP32 TOF offsets that take the neighbouring 1-ps
    column near a boundary; the precision launch forms them from float pairs
    and lands an order of magnitude closer (measured 4.0e-7 and 7.4e-7)."""
    from opensss_gb300 import workloads as W

    pr = W.tof13_64x64x48()
    xyz, _ = O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)
    idx = W.stratified_points(len(xyz), 96)
    ref = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                        pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                        pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                        pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                        pr.nr_bins, points=idx)
    plain = _gpu_compact(pr, att_table, points=idx)
    precise = _gpu_compact(pr, att_table, points=idx, kahan=True)
    assert_same_support(precise, ref)
    e_plain, e_precise = rel_l2(plain, ref), rel_l2(precise, ref)
    worst = float(np.abs(precise.astype(np.float64) - ref).max() / np.abs(ref).max())
    assert e_precise < 1e-6 and e_precise < 0.25 * e_plain
    assert worst < 5e-6


def test_kahan_on_33bin_sample(cuda_ok, att_table):
    from opensss_gb300 import workloads as W

    pr = W.tof33_128x128x96()
    got = _gpu_compact(pr, att_table, max_points=6, kahan=True)
    ref = _oracle_compact(pr, att_table, sp_end=6)
    assert_same_support(got, ref)
    assert rel_l2(got, ref) < TOL


@pytest.mark.parametrize("name", ["sss_tiny_b1", "sss_nontof_40x40x20"])
def test_unit_tof_fast_path_matches_voxel_walk(cuda_ok, att_table, name):
    """With one bin of unit weights the pairs take the legs' activity
    integrals instead of walking the voxels: same sinogram to FP32 rounding."""
    g = golden(name)
    pr = problem_from_golden(g)
    eng = _engine(pr, att_table)
    assert eng.unit_tof
    fast = eng.run(pr.activity, pr.attenuation, pr.image_size).cpu().numpy()
    walk = eng.run(pr.activity, pr.attenuation, pr.image_size, unit_tof=False).cpu().numpy()
    assert rel_l2(fast, walk) < 1e-6
    assert_same_support(fast, walk)


def test_slice_shards_add_up_to_the_full_run(cuda_ok, att_table):
    """Two shards of whole z-slices (the multi-GPU split) sum to the full run."""
    from opensss_gb300 import workloads as W
    from opensss_gb300.engine import fortran_flat
    from opensss_gb300.replicas import partition_slices

    pr = W.tiny_problem(5, seed=3)
    eng = _engine(pr, att_table)
    full = eng.run(pr.activity, pr.attenuation, pr.image_size).cpu().numpy()
    act, mu = fortran_flat(pr.activity, eng.device), fortran_flat(pr.attenuation, eng.device)
    _, counts = eng.scatter_points(eng.problem(act, mu, pr.grid, pr.image_size))
    parts = [eng.run(pr.activity, pr.attenuation, pr.image_size,
                     slice_range=partition_slices(counts, r, 2)).cpu().numpy() for r in range(2)]
    assert all(np.abs(p).max() > 0 for p in parts)
    assert rel_l2(parts[0] + parts[1], full) < 1e-6


@pytest.mark.parametrize("bins", [63, 64])
def test_widest_bin_counts_launch_and_match_oracle(cuda_ok, att_table, bins):
    """The largest bin counts: a 64-row Gaussian table in shared memory, and
    with Kahan's partial sums also there (the densest layout).  The plain,
    compensated and batched runs all match the FP64 oracle."""
    from opensss_gb300 import workloads as W
    from opensss_gb300.batch import BatchSSS
    from opensss_gb300.engine import leg_pair_to_compact

    scanner = W.ring_scanner(48, 6, radius_cm=20.0, ring_pitch_cm=1.0)
    pr = W.make_problem(f"tiny-b{bins}", (12, 12, 6), 2.0, 3, 8, bins, 1.5, 214.0, seed=4, scanner=scanner,
                        radius_cm=8.0)
    ref = _oracle_compact(pr, att_table)
    assert np.abs(ref).max() > 0
    runs = {k: _gpu_compact(pr, att_table, kahan=k) for k in (False, True)}
    b = BatchSSS([(_engine(pr, att_table), pr.activity, pr.attenuation, pr.image_size)])
    runs["batch"] = leg_pair_to_compact(b.run()[0].cpu().numpy(), pr.nr_rings_used, pr.nr_detectors_used)
    b.close()
    for name, got in runs.items():
        assert_same_support(got, ref)
        assert rel_l2(got, ref) < TOL, name


def test_tof_offsets_past_the_table_are_an_error(cuda_ok, att_table):
    """A 2 m wide body in a 1.5 m ring: the reference raises IndexError on its
    TOF table (recorded in the fixture); the engine reports SSS_ERR_TOF_RANGE."""
    from opensss_gb300._lib import SSSError

    g = golden("sss_tofrange")
    assert str(g["reference_error"]).startswith("IndexError")
    pr = problem_from_golden(g)
    with pytest.raises(SSSError) as e:
        _gpu_compact(pr, att_table)
    assert e.value.code == 4


def test_caller_index_tables_out_of_range_are_an_error(cuda_ok, att_table):
    """The device index tables a C caller passes are checked where they are
    read: a cell-table entry past the sampled pairs (sss_tof_densify_full),
    LOR coordinates past the sinogram (sss_tof_densify), and a sampled crystal
    or ring past the scanner (sss_tof_run) each set SSS_ERR_TABLE; the
    kernels read nothing at such an entry."""
    import ctypes as C

    import torch

    from opensss_gb300 import _lib, geometry as G
    from opensss_gb300._lib import SSSError

    def ptr(t):
        return C.c_void_p(t.data_ptr())

    g = golden("sss_tiny_b5")
    pr = problem_from_golden(g)
    nd, nru, ndu = pr.scanner.nr_detectors, pr.nr_rings_used, pr.nr_detectors_used
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, pr.scanner.nr_rings, ID_Shidt=False)
    eng = _engine(pr, att_table)
    lp = eng.run(pr.activity, pr.attenuation, pr.image_size).clone()
    L = _lib.lib()
    shape = (pr.nr_bins, nd + 1, nd // 2, nru * nru)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")

    cells = torch.from_numpy(G.dense_cell_pairs(lor, eng.dets_np, nd)).cuda()
    bad_cells = cells.clone()
    bad_cells[int(torch.nonzero(cells >= 0)[0])] = ndu * ndu + 3
    out = torch.zeros(shape, device="cuda")
    assert L.sss_tof_densify_full(ptr(lp), pr.nr_bins, nru, ndu, nd, ptr(bad_cells), ptr(out), ptr(st), None) == 0
    torch.cuda.synchronize()
    assert L.sss_status_code(int(st.item())) == 11

    d = eng.dets_np
    bad_lor = torch.from_numpy(np.ascontiguousarray(lor, dtype=np.int16)).cuda()
    bad_lor[int(d[0]), int(d[1]), 0] = nd // 2  # one past the last angle
    st.zero_()
    out.zero_()
    assert L.sss_tof_densify(ptr(lp), pr.nr_bins, nru, ndu, nd, ptr(bad_lor), ptr(eng.dets), ptr(out), ptr(st),
                             None) == 0
    torch.cuda.synchronize()
    assert L.sss_status_code(int(st.item())) == 11

    for table, bad in ((eng.dets, nd + 2), (eng.rings, pr.scanner.nr_rings)):
        keep = int(table[1])
        table[1] = bad
        with pytest.raises(SSSError) as e:
            eng.run(pr.activity, pr.attenuation, pr.image_size)
        assert e.value.code == 11
        table[1] = keep
    again = eng.run(pr.activity, pr.attenuation, pr.image_size)
    # the two tasks of a pair add to its cells with atomics, in either order
    assert rel_l2(again.cpu().numpy(), lp.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("name", ["sss_tiny_far", "sss_wide_body_tof13"])
def test_far_tof_offsets_match_reference(cuda_ok, att_table, name):
    """TOF offsets far past the last bin centre, where the pair kernel takes
    per-bin weights instead of the factored chain: 5 bins of 1 cm with a
    60 ps kernel (offsets to ~575 ps, factored range ~346 ps), and a 50 cm
    wide body at 13 bins of 3.9 cm and 214 ps (offsets to ~1770 ps, split at
    1675 ps).  The reference's weights there sit on the last bin.  The
    engine's result is finite, its status clean, and it matches."""
    g = golden(name)
    pr = problem_from_golden(g)
    got = _gpu_compact(pr, att_table)
    ref = g["compact"]
    assert np.isfinite(got).all()
    assert_same_support(got, ref)
    assert rel_l2(got, ref) < TOL


def test_tof13_slice_matches_reference(cuda_ok, att_table):
    """One sampled z-slice of the 13-bin benchmark workload on the 760 x 80
    scanner (the reference's own driver restricted to that slice): a seeded
    subset of 50,000 cells and every bin's total."""
    from opensss_gb300 import workloads as W
    from opensss_gb300.engine import leg_pair_to_compact

    g = golden("sss_tof13_slice")
    pr = W.tof13_64x64x48(seed=0)
    k = int(g["lattice_slice"])
    lp = _engine(pr, att_table).run(pr.activity, pr.attenuation, pr.image_size, slice_range=(k, k + 1))
    cmp = leg_pair_to_compact(lp.cpu().numpy(), pr.nr_rings_used, pr.nr_detectors_used)
    assert tuple(cmp.shape) == tuple(g["shape"])
    flat = cmp.reshape(cmp.shape[0], -1)
    got, ref = flat[:, g["cells"]], g["values"]
    assert_same_support(got, ref)
    assert rel_l2(got, ref) < TOL
    np.testing.assert_allclose(flat.astype(np.float64).sum(axis=1), g["bin_totals"], rtol=TOL)


def test_full_densify_to_device_and_pinned_host(cuda_ok, att_table):
    """sss_tof_densify_full writes every element of the reference layout,
    zeros included: into device memory and into page-locked host memory (the
    GPU writes it over the host link) it equals the oracle's densify of the
    same result; a pageable host pointer is refused before any launch."""
    import ctypes as C

    import torch

    from opensss_gb300 import _lib, geometry as G
    from opensss_gb300.engine import leg_pair_to_compact

    g = golden("sss_tiny_b5")  # 4 sampled rings: 16 slices a cell
    pr = problem_from_golden(g)
    nd = pr.scanner.nr_detectors
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, pr.scanner.nr_rings, ID_Shidt=False)
    eng = _engine(pr, att_table)
    lp = eng.run(pr.activity, pr.attenuation, pr.image_size)
    ref = O.densify(leg_pair_to_compact(lp.cpu().numpy(), pr.nr_rings_used, pr.nr_detectors_used), lor, nd,
                    pr.nr_rings_used, pr.nr_detectors_used)
    cells = torch.from_numpy(G.dense_cell_pairs(lor, eng.dets_np, nd)).cuda()
    shape = (pr.nr_bins, nd + 1, nd // 2, pr.nr_rings_used ** 2)
    for out in (torch.full(shape, 7.0, device="cuda"), torch.full(shape, 7.0).pin_memory()):
        eng.densify_full(lp, cells, out)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref.astype(np.float32))
    # sss_tof_densify_cells: the sampled pairs' cells alone, every element of them; the rest is left as it is
    sampled = cells.cpu().numpy() >= 0
    for out in (torch.full(shape, 7.0, device="cuda"), torch.full(shape, 7.0).pin_memory()):
        eng.densify_full(lp, cells, out, sampled_only=True)
        eng.check_status()
        got = out.cpu().numpy().reshape(shape[0], -1, shape[3])
        want = ref.astype(np.float32).reshape(shape[0], -1, shape[3])
        assert np.array_equal(got[:, sampled], want[:, sampled])
        assert (got[:, ~sampled] == 7.0).all()
    pageable = np.zeros(shape, np.float32)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = _lib.lib().sss_tof_densify_full(C.c_void_p(lp.data_ptr()), pr.nr_bins, pr.nr_rings_used,
                                         pr.nr_detectors_used, nd, C.c_void_p(cells.data_ptr()),
                                         C.c_void_p(pageable.ctypes.data), C.c_void_p(st.data_ptr()), None)
    assert rc == 1 and "page-locked" in _lib.last_error()
    assert not pageable.any()


def test_dropin_full_dense_path(cuda_ok, att_table):
    """The drop-in with NRU^2 a multiple of 4 writes its result straight into
    page-locked host memory: same array as the oracle's densify."""
    from opensss_gb300 import SingleScatterSimulationTOF
    from opensss_gb300.geometry import SinogramCoordinates

    g = golden("sss_tiny_b5")
    pr = problem_from_golden(g)
    lor, _, _ = SinogramCoordinates(1, 1, 1, 1, pr.scanner.nr_detectors, pr.scanner.nr_rings, ID_Shidt=False)
    args = (pr.image_size, pr.scanner.geometry, lor, pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
            pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step,
            pr.tof_resolution, pr.tof_range, pr.nr_bins, None)
    out = SingleScatterSimulationTOF(pr.activity, pr.attenuation, *args)
    ref = O.densify(g["compact"].astype(np.float64), lor, pr.scanner.nr_detectors, pr.nr_rings_used,
                    pr.nr_detectors_used)
    assert_same_support(out, ref)
    assert rel_l2(out, ref) < TOL
    out2 = SingleScatterSimulationTOF(pr.activity, pr.attenuation, *args)
    assert not np.shares_memory(out, out2) and rel_l2(out2, out) < 1e-6
    # with few host threads the GPU writes every element instead of the host clearing the result
    import torch

    threads = torch.get_num_threads()
    torch.set_num_threads(2)
    try:
        out3 = SingleScatterSimulationTOF(pr.activity, pr.attenuation, *args)
    finally:
        torch.set_num_threads(threads)
    assert_same_support(out3, ref)
    assert rel_l2(out3, out) < 1e-6
