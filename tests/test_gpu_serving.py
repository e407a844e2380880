"""Served scatter updates: every request served in a mixed, batched stream
gives the same sinogram as the same request run alone (1e-5 relative L2:
only the order of FP32 atomic additions over z-slices differs), also when the
HBM budget forces requests to wait."""

import types

import numpy as np
import pytest

from conftest import rel_l2

TOL = 1e-5


def test_poisson_stream_is_seeded_and_mixed():
    from opensss_gb300.serving import poisson_stream

    beds = [types.SimpleNamespace(large=i >= 4) for i in range(8)]
    a = poisson_stream(200.0, 5.0, beds, 0.7, seed=3)
    b = poisson_stream(200.0, 5.0, beds, 0.7, seed=3)
    assert [(r.arrival, r.bed, r.seed) for r in a] == [(r.arrival, r.bed, r.seed) for r in b]
    assert 800 < len(a) < 1200
    frac = np.mean([not beds[r.bed].large for r in a])
    assert 0.65 < frac < 0.75
    assert all(x.arrival < y.arrival for x, y in zip(a, a[1:]))


def _beds(att):
    from opensss_gb300 import TofSSS, workloads as W
    from opensss_gb300.serving import make_bed

    small = W.ring_scanner(96, 12, radius_cm=25.0, ring_pitch_cm=1.2, phase=0.5)
    probs = [
        (W.make_problem("s0", (20, 20, 12), 1.5, 4, 12, 1, None, 1.0e6, seed=1, scanner=small,
                        radius_cm=9.0), False),
        (W.make_problem("s1", (16, 16, 10), 1.7, 3, 16, 5, 3.0, 214.0, seed=2, scanner=small,
                        radius_cm=8.0), False),
        (W.make_problem("L0", (24, 24, 16), 1.2, 6, 16, 13, 3.9, 214.0, seed=3, scanner=small,
                        radius_cm=10.0), True),
    ]
    beds = []
    for pr, large in probs:
        e = TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att,
                   pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                   pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins)
        beds.append(make_bed(e, pr.activity, pr.attenuation, pr.image_size, large=large))
    return beds


@pytest.mark.gpu
@pytest.mark.parametrize("budget_mb,large_ws_mb", [(80 << 10, 16 << 10), (400, 8)])
def test_served_results_match_solo_runs(cuda_ok, att_table, budget_mb, large_ws_mb):
    from opensss_gb300.serving import PlainServer, ScatterServer, poisson_stream, request_activity

    beds = _beds(att_table)
    reqs = poisson_stream(2000.0, 0.015, beds, 0.7, seed=1)
    assert len(reqs) >= 10
    srv = ScatterServer(beds, hbm_budget=budget_mb << 20, large_workspace=large_ws_mb << 20)
    served = srv.serve(reqs)
    assert all(np.isfinite(r.done) and r.done >= r.arrival for r in served)
    if large_ws_mb == 8:
        assert srv.stats["waves"] > srv.stats["batches_small"] + srv.stats["batches_large"]
    for r in served:
        bed = beds[r.bed]
        ref = bed.engine.run_flat(request_activity(bed, r.seed), bed.mu, bed.shape, bed.image_size)
        got = r.out.cpu().numpy()
        assert np.abs(ref.cpu().numpy()).max() > 0
        assert rel_l2(got, ref.cpu().numpy()) < TOL, (r.rid, r.bed)
    # the plain server gives the same results too
    plain = PlainServer(beds).serve(poisson_stream(2000.0, 0.015, beds, 0.7, seed=1))
    for a, b in zip(served, plain):
        assert rel_l2(a.out.cpu().numpy(), b.out.cpu().numpy()) < TOL


@pytest.mark.gpu
def test_request_over_the_hbm_budget_is_refused(cuda_ok, att_table):
    """Admission: with nothing in flight, a batch that cannot fit the HBM
    budget raises MemoryError before any of its work is enqueued."""
    from opensss_gb300.serving import Request, ScatterServer

    beds = _beds(att_table)[:1]
    srv = ScatterServer(beds, hbm_budget=1 << 20)
    with pytest.raises(MemoryError, match="HBM budget"):
        srv.serve([Request(0, 0.0, 0, seed=1)])


@pytest.mark.gpu
def test_device_error_of_a_served_request_is_raised(cuda_ok, att_table):
    """A served problem whose TOF offsets pass the 8001-entry table (the
    reference raises IndexError there): the batch's status word reports it
    and serve() raises SSS_ERR_TOF_RANGE once the stream has drained."""
    from conftest import golden, problem_from_golden
    from opensss_gb300 import TofSSS
    from opensss_gb300._lib import SSSError
    from opensss_gb300.serving import Request, ScatterServer, make_bed

    pr = problem_from_golden(golden("sss_tofrange"))
    e = TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
               pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
               pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins)
    bed = make_bed(e, pr.activity, pr.attenuation, pr.image_size)
    srv = ScatterServer([bed], hbm_budget=8 << 30)
    with pytest.raises(SSSError) as err:
        srv.serve([Request(0, 0.0, 0, seed=1)])
    assert err.value.code == 4
