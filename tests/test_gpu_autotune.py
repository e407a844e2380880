"""Launch shapes on the GPU: every candidate gives the default shape's result
(the pair terms are the same; only the order of the two tasks' atomic adds to
a cell can differ), the tuner picks a candidate, and shapes outside the
compiled bounds are rejected."""

import pytest

from conftest import rel_l2
from opensss_gb300 import TofSSS, autotune, workloads as W
from opensss_gb300._lib import SSSError

pytestmark = pytest.mark.gpu


def _engine(pr, att):
    return TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att,
                  pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                  pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins)


@pytest.mark.parametrize("bins", [5, 33])
def test_every_launch_shape_gives_the_same_result(cuda_ok, att_table, bins):
    pr = W.tiny_problem(bins, seed=4, shape=(16, 16, 8), nd=64, nr=8, nru=4, ndu=12)
    eng = _engine(pr, att_table)
    ref = eng.run(pr.activity, pr.attenuation, pr.image_size).cpu().numpy()
    for w in autotune.pair_warp_candidates(bins):
        for t in autotune.LEG_THREADS:
            eng.pair_warps, eng.leg_threads = w, t
            got = eng.run(pr.activity, pr.attenuation, pr.image_size).cpu().numpy()
            assert rel_l2(got, ref) <= 1e-6, (w, t)


def test_tune_picks_a_candidate_and_caches_it(cuda_ok, att_table, tmp_path, monkeypatch):
    monkeypatch.setenv("OPENSSS_GB300_TUNE_CACHE", str(tmp_path / "shapes.json"))
    monkeypatch.setattr(autotune, "_memory", {})
    pr = W.tiny_problem(3, seed=5, shape=(16, 16, 8), nd=64, nr=8, nru=4, ndu=12)
    eng = _engine(pr, att_table)
    r = autotune.tune(eng, pr.activity, pr.attenuation, pr.image_size, sample_points=64, reps=1)
    assert not r["cached"] and r["pair_warps"] in autotune.pair_warp_candidates(3)
    assert r["leg_threads"] in autotune.LEG_THREADS
    assert (eng.pair_warps, eng.leg_threads) == (r["pair_warps"], r["leg_threads"])
    eng2 = _engine(pr, att_table)
    r2 = autotune.tune(eng2, pr.activity, pr.attenuation, pr.image_size, sample_points=64, reps=1)
    assert r2["cached"] and (eng2.pair_warps, eng2.leg_threads) == (eng.pair_warps, eng.leg_threads)


def test_batch_autotune_keeps_results(cuda_ok, att_table, tmp_path, monkeypatch):
    from opensss_gb300.batch import BatchSSS

    monkeypatch.setenv("OPENSSS_GB300_TUNE_CACHE", str(tmp_path / "shapes.json"))
    monkeypatch.setattr(autotune, "_memory", {})
    probs = [W.tiny_problem(b, seed=6 + b, shape=(16, 16, 8), nd=64, nr=8, nru=4, ndu=12) for b in (1, 3, 5)]
    solo = []
    for pr in probs:
        solo.append(_engine(pr, att_table).run(pr.activity, pr.attenuation, pr.image_size).cpu().numpy())
    b = BatchSSS([(_engine(pr, att_table), pr.activity, pr.attenuation, pr.image_size) for pr in probs],
                 workspace_bytes=1 << 28, autotune=True)
    assert set(b.tuned) == {"bins=1", "bins=3", "bins=5"}
    b.run()
    for o, s in zip(b.outs, solo):
        assert rel_l2(o.cpu().numpy(), s) <= 1e-5
    b.close()


def test_launch_shape_outside_the_bounds_is_an_error(cuda_ok, att_table):
    pr = W.tiny_problem(3, seed=1)
    eng = _engine(pr, att_table)
    eng.pair_warps = 99
    with pytest.raises(SSSError):
        eng.run(pr.activity, pr.attenuation, pr.image_size)
    eng.pair_warps, eng.leg_threads = 0, 48
    with pytest.raises(SSSError):
        eng.run(pr.activity, pr.attenuation, pr.image_size)
