"""Host-side helpers that the GPU tests lean on, checked on the CPU: the
leg-pair <-> compact sinogram layouts, the scatter-point subset selection, the
spread sample of scatter points and the seeded request stream of the server."""

import types

import numpy as np
import pytest
import torch

from opensss_gb300 import workloads as W
from opensss_gb300.engine import compact_to_leg_pair, leg_pair_to_compact, select_points
from opensss_gb300.serving import poisson_stream


@pytest.mark.parametrize("nru,ndu,nb", [(1, 1, 1), (3, 8, 5), (4, 6, 2)])
def test_leg_pair_layout_maps_each_cell_and_round_trips(nru, ndu, nb):
    rng = np.random.default_rng(nru * 100 + ndu)
    lp = rng.standard_normal((nb, nru * ndu, nru * ndu)).astype(np.float32)
    cmp = leg_pair_to_compact(lp, nru, ndu)
    assert cmp.shape == (nb, nru * nru, ndu, ndu)
    # leg = crystal index * NRU + ring index; sino = ri1 * NRU + ri2
    for b, ri1, ri2, d1, d2 in [(0, 0, nru - 1, 0, ndu - 1), (nb - 1, nru - 1, 0, ndu - 1, 0),
                                (nb // 2, nru // 2, nru - 1, ndu // 2, ndu // 3)]:
        assert cmp[b, ri1 * nru + ri2, d1, d2] == lp[b, d1 * nru + ri1, d2 * nru + ri2]
    back = compact_to_leg_pair(cmp, nru, ndu)
    assert back.flags["C_CONTIGUOUS"]
    assert np.array_equal(back, lp)


def test_select_points_keeps_rows_and_counts_per_slice():
    counts = np.array([3, 0, 2, 4])
    pts = torch.arange(9 * 4, dtype=torch.float64).reshape(9, 4)
    rows, kept = select_points(pts, counts, [0, 2, 3, 5, 8])
    assert torch.equal(rows, pts[[0, 2, 3, 5, 8]])
    assert kept.tolist() == [2, 0, 1, 2]
    rows, kept = select_points(pts, counts, [])
    assert rows.shape == (0, 4) and kept.tolist() == [0, 0, 0, 0]
    for bad in ([3, 2], [0, 0], [-1, 2], [8, 9]):
        with pytest.raises(IndexError):
            select_points(pts, counts, bad)


def test_stratified_points_spread_over_the_whole_range():
    idx = W.stratified_points(11362, 710)
    assert len(idx) == 710 and idx[0] == 0 and idx[-1] == 11361
    assert np.all(np.diff(idx) > 0)
    gaps = np.diff(idx)
    assert gaps.max() - gaps.min() <= 1  # evenly spread, so every slice contributes
    assert np.array_equal(W.stratified_points(5, 9), np.arange(5))


def test_poisson_stream_is_seeded_and_keeps_size_classes():
    beds = [types.SimpleNamespace(large=flag) for flag in (False, True, False, True, False)]
    a = poisson_stream(200.0, 1.0, beds, 0.7, seed=2026)
    b = poisson_stream(200.0, 1.0, beds, 0.7, seed=2026)
    assert [(r.arrival, r.bed, r.seed) for r in a] == [(r.arrival, r.bed, r.seed) for r in b]
    arrivals = np.array([r.arrival for r in a])
    assert np.all(np.diff(arrivals) > 0) and arrivals[-1] < 1.0
    assert 140 < len(a) < 260  # Poisson(200)
    small = np.mean([not beds[r.bed].large for r in a])
    assert 0.55 < small < 0.85
    assert [r.rid for r in a] == list(range(len(a)))
    only_small = poisson_stream(50.0, 1.0, [types.SimpleNamespace(large=False)], 0.0, seed=1)
    assert all(r.bed == 0 for r in only_small)  # no large bed: every request takes a small one
