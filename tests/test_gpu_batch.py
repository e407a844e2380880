"""Batched TOF-SSS (sss_batch_*): every problem of an uneven batch gives the
same sampled sinogram as its own sss_tof_run, in one wave or many, and again
after its activity map is replaced in place.

Tolerance: 1e-5 relative L2 per problem (the two paths add the same FP32
terms, only the order of the atomic additions over z-slices differs)."""

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _engine(pr, att):
    from opensss_gb300 import TofSSS

    return TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att,
                  pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                  pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                  pr.nr_bins)


def _uneven_problems():
    from opensss_gb300 import workloads as W

    small = W.ring_scanner(96, 12, radius_cm=25.0, ring_pitch_cm=1.2)
    big = W.ring_scanner(160, 16, radius_cm=30.0, ring_pitch_cm=1.0)
    return [
        W.make_problem("u0", (20, 20, 12), 1.5, 4, 12, 13, 3.9, 214.0, seed=1, scanner=small,
                       radius_cm=9.0),
        W.make_problem("u1", (20, 20, 10), 1.6, 3, 16, 1, None, 1.0e6, seed=2, scanner=big,
                       radius_cm=8.0),
        W.make_problem("u2", (24, 24, 16), 1.2, 6, 10, 5, 3.0, 214.0, seed=3, scanner=small,
                       radius_cm=10.0, sample_step=(3, 3, 2)),
        W.make_problem("u3", (17, 17, 9), 1.7, 4, 12, 13, 3.9, 214.0, seed=4, scanner=small,
                       radius_cm=12.0),
        W.make_problem("u4", (24, 24, 14), 1.4, 5, 20, 8, 2.5, 300.0, seed=5, scanner=big,
                       radius_cm=11.0),
    ]


def _solo(eng, pr):
    return eng.run(pr.activity, pr.attenuation, pr.image_size).cpu().numpy()


@pytest.mark.parametrize("workspace_mb", [None, 24])
def test_batch_matches_solo_runs(cuda_ok, att_table, workspace_mb):
    from opensss_gb300.batch import BatchSSS

    probs = _uneven_problems()
    engines = [_engine(pr, att_table) for pr in probs]
    ws = None if workspace_mb is None else workspace_mb << 20
    b = BatchSSS([(e, pr.activity, pr.attenuation, pr.image_size) for e, pr in zip(engines, probs)],
                 workspace_bytes=ws)
    if workspace_mb is not None:
        assert b.waves > 1  # the small workspace forces several waves
    outs = [o.cpu().numpy() for o in b.run()]
    for e, pr, got in zip(engines, probs, outs):
        ref = _solo(e, pr)
        assert got.shape == ref.shape
        assert np.abs(ref).max() > 0
        assert rel_l2(got, ref) < TOL, pr.name
    # a second run of the same plan gives the same result
    again = [o.cpu().numpy() for o in b.run()]
    for a, g in zip(again, outs):
        assert rel_l2(a, g) < TOL
    b.close()


def test_uneven_batch_classes_against_fp64_oracle(cuda_ok, att_table):
    """One problem of each TOF class (1, 13 and 33 bins) of the 64-instance
    uneven batch, planned together: each problem's result over a stratified
    sample of its scatter points (every sampled z-slice) against the FP64
    oracle on the same points (1e-4, the engine's bar)."""
    from opensss_gb300 import workloads as W
    from opensss_gb300.batch import BatchSSS
    from opensss_gb300.engine import fortran_flat, leg_pair_to_compact, select_points
    from oracle import oracle as O

    inst = W.uneven_instances(64, seed=0)
    chosen = {}
    for pr in inst:
        work = int(np.prod(pr.grid)) * pr.nr_rings_used * pr.nr_detectors_used
        if pr.nr_bins not in chosen or work < chosen[pr.nr_bins][0]:
            chosen[pr.nr_bins] = (work, pr)
    assert sorted(chosen) == [1, 13, 33]
    probs = [chosen[b][1] for b in (1, 13, 33)]
    engines = [_engine(pr, att_table) for pr in probs]
    jobs, pts, idxs = [], [], []
    for e, pr in zip(engines, probs):
        act, mu = fortran_flat(pr.activity, e.device), fortran_flat(pr.attenuation, e.device)
        p, c = e.scatter_points(e.problem(act, mu, pr.grid, pr.image_size))
        idx = W.stratified_points(len(p), 24)
        pts.append(select_points(p, c, idx))
        idxs.append(idx)
        jobs.append((e, act, mu, pr.image_size, pr.grid))
    b = BatchSSS(jobs, points=pts)
    outs = [o.cpu().numpy() for o in b.run()]
    b.close()
    for pr, got, idx in zip(probs, outs, idxs):
        ref = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                            pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                            pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                            pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                            pr.nr_bins, points=idx)
        cmp = leg_pair_to_compact(got, pr.nr_rings_used, pr.nr_detectors_used)
        assert np.abs(ref).max() > 0
        assert rel_l2(cmp, ref) < 1e-4, pr.name


def test_batch_rerun_with_new_activity(cuda_ok, att_table):
    import torch

    from opensss_gb300.batch import BatchSSS
    from opensss_gb300.engine import fortran_flat

    probs = _uneven_problems()[:3]
    engines = [_engine(pr, att_table) for pr in probs]
    b = BatchSSS([(e, pr.activity, pr.attenuation, pr.image_size) for e, pr in zip(engines, probs)])
    b.run()
    rng = np.random.default_rng(7)
    new = [pr.activity * rng.uniform(0.95, 1.05, size=pr.activity.shape).astype(np.float32)
           for pr in probs]
    for i, a in enumerate(new):
        b.activity(i).copy_(fortran_flat(a, engines[i].device))
    torch.cuda.synchronize()
    outs = [o.cpu().numpy() for o in b.run()]
    for e, pr, a, got in zip(engines, probs, new, outs):
        ref = e.run(a, pr.attenuation, pr.image_size).cpu().numpy()
        assert rel_l2(got, ref) < TOL, pr.name


def test_batch_workspace_too_small_is_an_error(cuda_ok, att_table):
    from opensss_gb300._lib import SSSError
    from opensss_gb300.batch import BatchSSS

    pr = _uneven_problems()[0]
    e = _engine(pr, att_table)
    with pytest.raises(SSSError):
        BatchSSS([(e, pr.activity, pr.attenuation, pr.image_size)], workspace_bytes=1 << 16)


def test_index_past_the_volume_is_an_error(cuda_ok, att_table):
    """Nx != Ny: the reference's sub2ind (Ny as the x stride) yields linear
    indices past the volume, where its numpy indexing raises IndexError; the
    engine reports SSS_ERR_VOXEL and the oracle status -6."""
    from opensss_gb300 import workloads as W
    from opensss_gb300._lib import SSSError
    from oracle import oracle as O

    pr = W.make_problem("nx-ne-ny", (16, 24, 10), 1.6, 3, 16, 1, None, 1.0e6, seed=2,
                        scanner=W.ring_scanner(160, 16, radius_cm=30.0, ring_pitch_cm=1.0),
                        radius_cm=8.0)
    with pytest.raises(RuntimeError, match="status -6"):
        O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                      pr.scanner.normals, pr.scanner.detector_size_mm, att_table,
                      pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used,
                      pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                      pr.nr_bins)
    with pytest.raises(SSSError) as e:
        _solo(_engine(pr, att_table), pr)
    assert e.value.code == 6


def test_batch_graph_replay_matches_run(cuda_ok, att_table):
    """A captured plan replays to the same outputs, also after the activity
    changes in place."""
    import torch

    from opensss_gb300.batch import BatchSSS

    probs = _uneven_problems()
    engines = [_engine(pr, att_table) for pr in probs]
    b = BatchSSS([(e, pr.activity, pr.attenuation, pr.image_size) for e, pr in zip(engines, probs)],
                 workspace_bytes=24 << 20)
    ref = [o.cpu().numpy() for o in b.run()]
    b.capture()
    got = [o.cpu().numpy() for o in b.replay()]
    for r, g in zip(ref, got):
        assert rel_l2(g, r) < TOL
    b.activity(1).mul_(2.0)
    torch.cuda.synchronize()
    got2 = [o.cpu().numpy() for o in b.replay()]
    assert rel_l2(got2[1], 2.0 * ref[1]) < TOL  # SSS is linear in the activity
    assert rel_l2(got2[0], ref[0]) < TOL
    b.close()


def test_batch_run_on_a_side_stream(cuda_ok, att_table):
    """run(stream=s) with s not the current stream resets the status word on s
    and gives the default-stream outputs."""
    import torch

    from opensss_gb300.batch import BatchSSS

    probs = _uneven_problems()[:2]
    engines = [_engine(pr, att_table) for pr in probs]
    b = BatchSSS([(e, pr.activity, pr.attenuation, pr.image_size) for e, pr in zip(engines, probs)])
    ref = [o.cpu().numpy() for o in b.run()]
    side = torch.cuda.Stream(b.device)
    side.wait_stream(torch.cuda.current_stream(b.device))
    got = [o.cpu().numpy() for o in b.run(stream=side)]  # synchronises side
    for a, r in zip(got, ref):
        assert rel_l2(a, r) < TOL
    b.close()


def test_batch_with_degenerate_problems(cuda_ok, att_table):
    """A batch mixing ordinary problems with one that has no scatter point
    (empty attenuation map) and one with no activity: the degenerate ones
    plan no item and come out all zero; the others match their solo runs."""
    from opensss_gb300.batch import BatchSSS

    probs = _uneven_problems()[:2]
    empty_mu, empty_act = _uneven_problems()[2], _uneven_problems()[3]
    empty_mu.attenuation = np.zeros_like(empty_mu.attenuation)
    empty_act.activity = np.zeros_like(empty_act.activity)
    probs += [empty_mu, empty_act]
    engines = [_engine(pr, att_table) for pr in probs]
    b = BatchSSS([(e, pr.activity, pr.attenuation, pr.image_size) for e, pr in zip(engines, probs)])
    outs = [o.cpu().numpy() for o in b.run()]
    for e, pr, got in zip(engines[:2], probs[:2], outs[:2]):
        assert rel_l2(got, _solo(e, pr)) < TOL, pr.name
    assert not outs[2].any() and not outs[3].any()
    b.close()
