"""The FP64 GPU oracle (oracle/sss_oracle_gpu.cu): pinned to the C restatement
whose arithmetic it shares (oracle/orc_core.h) and to the reference's own
outputs, then used to state the engine's error on the 33-bin precision
workload over far more scatter points than the host cores finish in a test.

Tolerances: the two oracles run the same FP64 operations in the same order
and differ only where the device's exp/pow/acos/cos/sin round differently
from the host's libm, so they agree to 1e-13 relative L2 with the same
contributing cells; against the reference (float32 sums) the C restatement's
1e-6 bar holds; the engine stays within its 1e-4 bar."""

import numpy as np
import pytest

from conftest import golden, problem_from_golden, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ORACLE_TOL = 1e-13

GOLDENS = ["sss_tiny_b1", "sss_tiny_b3", "sss_tiny_b5", "sss_tiny_nx14_ny10", "sss_tiny_wide", "sss_tiny_far",
           "sss_wide_body_tof13", "sss_tiny_even_aniso", "sss_edge_empty_mu", "sss_edge_empty_act", "sss_edge_one_ring",
           "sss_edge_one_crystal", "sss_edge_step_past_volume"]


def _oracle(pr, att, **kw):
    return O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry, pr.scanner.normals,
                         pr.scanner.detector_size_mm, att, pr.energy_resolution, pr.energy_threshold,
                         pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                         pr.nr_bins, **kw)


def _same_cells_and_close(a, b, tol):
    assert np.array_equal(a != 0, b != 0)
    assert rel_l2(a, b) < tol


@pytest.mark.parametrize("name", GOLDENS)
def test_gpu_oracle_matches_host_oracle_and_reference(cuda_ok, att_table, name):
    g = golden(name)
    pr = problem_from_golden(g)
    dev = _oracle(pr, att_table, gpu=True)
    _same_cells_and_close(dev, _oracle(pr, att_table), ORACLE_TOL)
    _same_cells_and_close(dev, g["compact"], 1e-6)


def test_gpu_oracle_point_launches_do_not_change_the_sums(cuda_ok, att_table):
    """Each cell's thread adds the slice's points in lattice order whatever
    the launch holds, so one point per launch gives the identical result."""
    pr = problem_from_golden(golden("sss_tiny_b5"))
    whole = _oracle(pr, att_table, gpu=True)
    one_at_a_time = _oracle(pr, att_table, gpu=True, leg_bytes=1)
    assert np.array_equal(whole, one_at_a_time)


def test_gpu_oracle_point_list_matches_host_oracle(cuda_ok, att_table):
    pr = problem_from_golden(golden("sss_tiny_b5"))
    idx = np.array([0, 3, 4, 9, 17, 30])
    _same_cells_and_close(_oracle(pr, att_table, gpu=True, points=idx), _oracle(pr, att_table, points=idx),
                          ORACLE_TOL)


def test_gpu_oracle_reports_tof_offsets_past_the_table(cuda_ok, att_table):
    pr = problem_from_golden(golden("sss_tofrange"))
    with pytest.raises(RuntimeError, match="status -2"):
        _oracle(pr, att_table, gpu=True)


def test_gpu_oracle_tof13_slice_matches_reference(cuda_ok, att_table):
    """One sampled z-slice of the 13-bin, 64x64x48 @ 6 mm workload: the
    reference's own driver on that slice against the GPU oracle."""
    from opensss_gb300 import workloads as W

    g = golden("sss_tof13_slice")
    pr = W.tof13_64x64x48(seed=0)
    _, sl = O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)
    idx = np.flatnonzero(sl == int(g["z_index"]))
    cmp = _oracle(pr, att_table, gpu=True, sp_begin=int(idx[0]), sp_end=int(idx[-1]) + 1)
    flat = cmp.reshape(cmp.shape[0], -1)
    got, ref = flat[:, g["cells"]], g["values"]
    tiny = 1e-25 * float(np.abs(ref).max())
    differ = (got != 0) != (ref != 0)
    assert not np.any(differ & ((np.abs(got) > tiny) | (np.abs(ref) > tiny)))
    assert int(np.count_nonzero(flat.any(axis=0))) == int(g["contributing"])
    assert rel_l2(got, ref) < 1e-6


def test_tof33_engine_against_gpu_oracle(cuda_ok, att_table):
    """The 33-bin precision workload (128x128x96 @ 4 mm, 32 x 96 sampled,
    11,362 scatter points): one point in sixteen, spread evenly over every
    sampled z-slice, through the plain and the precision launch against the
    FP64 GPU oracle on the same points (each slice normalised over its kept
    points).  Relative L2 and the largest bin error over the largest bin."""
    from opensss_gb300 import TofSSS, workloads as W
    from opensss_gb300.engine import leg_pair_to_compact

    pr = W.tof33_128x128x96()
    xyz, _ = O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)
    idx = W.stratified_points(len(xyz), len(xyz) // 16)
    ref = _oracle(pr, att_table, gpu=True, points=idx)
    eng = TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                 pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                 pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins)
    peak = float(np.abs(ref).max())
    for kahan, l2_bar, bin_bar in ((False, 1e-4, 1e-3), (True, 2e-6, 1e-5)):
        lp = eng.run(pr.activity, pr.attenuation, pr.image_size, points=idx, kahan=kahan).cpu().numpy()
        got = leg_pair_to_compact(lp, pr.nr_rings_used, pr.nr_detectors_used)
        tiny = 1e-25 * peak
        differ = (got != 0) != (ref != 0)
        assert not np.any(differ & ((np.abs(got) > tiny) | (np.abs(ref) > tiny)))
        assert rel_l2(got, ref) < l2_bar
        assert float(np.abs(got.astype(np.float64) - ref).max()) / peak < bin_bar
