"""Several ranks on the CPU (gloo, world size 2): the z-slice partition covers
every sampled slice once, the ranks' partial sinograms add up to the full
one (with the FP64 oracle as each rank's compute), and the bench's timing
takes the slowest rank."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def test_partition_covers_every_slice_once():
    from opensss_gb300.replicas import partition_slices

    rng = np.random.default_rng(0)
    for world in (1, 2, 3, 8):
        counts = rng.integers(0, 50, size=24)
        parts = [partition_slices(counts, r, world) for r in range(world)]
        assert parts[0][0] == 0 and parts[-1][1] == len(counts)
        assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
        loads = [counts[a:b].sum() for a, b in parts]
        assert max(loads) - min(loads) <= 2 * counts.max()  # every cut within one slice of its target
    assert partition_slices([5, 0, 0], 1, 2) == (1, 3)
    with pytest.raises(ValueError):
        partition_slices([1, 2], 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, result_path):
    import torch
    import torch.distributed as dist

    from opensss_gb300 import workloads as W
    from opensss_gb300.replicas import max_over_ranks, partition_slices, sum_over_ranks
    from oracle import oracle as O

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        att = np.load(os.path.join(os.path.dirname(__file__), "golden", "tables.npz"))["att_table"]
        pr = W.tiny_problem(3, seed=2)
        _, sl = O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)
        lz = -(-pr.grid[2] // int(pr.sample_step[2]))
        counts = np.bincount(sl // int(pr.sample_step[2]), minlength=lz)
        a, b = partition_slices(counts, rank, world)
        first, last = int(counts[:a].sum()), int(counts[:b].sum())
        part = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry, pr.scanner.normals,
                             pr.scanner.detector_size_mm, att, pr.energy_resolution, pr.energy_threshold,
                             pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step, pr.tof_resolution,
                             pr.tof_range, pr.nr_bins, sp_begin=first, sp_end=last, nthreads=1)
        total = sum_over_ranks(torch.from_numpy(np.ascontiguousarray(part)))
        slowest = max_over_ranks(1.0 + rank)
        if rank == 0:
            np.savez(result_path, total=total.numpy(), slowest=slowest)
    finally:
        dist.destroy_process_group()


def test_two_ranks_add_up_to_the_full_simulation(tmp_path, att_table):
    from opensss_gb300 import workloads as W
    from oracle import oracle as O

    out = str(tmp_path / "r.npz")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    res = np.load(out)
    pr = W.tiny_problem(3, seed=2)
    full = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry, pr.scanner.normals,
                         pr.scanner.detector_size_mm, att_table, pr.energy_resolution, pr.energy_threshold,
                         pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                         pr.nr_bins, nthreads=1)
    assert np.abs(full).max() > 0
    assert np.allclose(res["total"], full, rtol=1e-12, atol=1e-12 * np.abs(full).max())
    assert float(res["slowest"]) == 2.0
