"""Benchmark: TOF-SSS scatter-point x detector-pair x TOF-bin throughput.

Workload (one "step"): a full TOF single scatter simulation of the plain
single-instance configuration — 64x64x48 voxels of 6 mm, 760-crystal x
80-ring scanner (820 mm diameter) sampled as 16 rings x 48 crystals, 13 TOF
bins of 39 mm, 214 ps FWHM, scatter points every 2nd voxel with mu > 0.
Inputs are a seeded synthetic water cylinder with lung insert and six hot
spheres (no public dataset is used).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --profile CASE [--reps N]     (a small case for ncu)

Prints one JSON line (rank 0).  For N > 1 (launched by torch.distributed.run)
every rank runs an independent replica on its own GPU ("replicas only": the
path does not shard), the time is the max over ranks.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TOF-SSS scatter-pt x det-pair x TOF-bin / s"
UNIT = "units/s"


def _att_table():
    return np.load(os.path.join(ROOT, "tests", "golden", "tables.npz"))["att_table"]


def _pairs(nru, ndu):
    return nru * nru * ndu * (ndu - 1) // 2 + ndu * nru * (nru - 1)


def _workload():
    from opensss_gb300 import workloads as W

    return W.tof13_64x64x48(seed=0)


def _config(pr, extra=None):
    c = {"workload": pr.name, "volume": list(pr.grid), "voxel_mm": 6.0,
         "scanner": "760 crystals x 80 rings, 820 mm", "sampled_rings": pr.nr_rings_used,
         "sampled_crystals": pr.nr_detectors_used, "tof_bins": pr.nr_bins,
         "tof_fwhm_ps": pr.tof_resolution, "sample_step": [int(s) for s in pr.sample_step],
         "l2": "flushed between timed steps (256 MiB write); leg lists also exceed L2",
         "parallelism": "replicas"}
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------- clocks


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------- CPU side


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_sample(pr, att, idx, threads):
    """FP64 C restatement of the reference over the scatter points numbered
    ``idx`` (ascending, lattice order; each z-slice normalised over its kept
    points)."""
    from oracle import build_oracle
    from oracle import oracle as O

    build_oracle.build_oracle()
    t0 = time.perf_counter()
    out = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry,
                        pr.scanner.normals, pr.scanner.detector_size_mm, att, pr.energy_resolution,
                        pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step,
                        pr.tof_resolution, pr.tof_range, pr.nr_bins, points=idx, nthreads=threads)
    return out, time.perf_counter() - t0


def stratified_sample(pr, count):
    """``count`` scatter points spread evenly over the workload's points in
    lattice order (every sampled z-slice contributes)."""
    from opensss_gb300 import workloads as W
    from oracle import oracle as O

    n = len(O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)[0])
    return W.stratified_points(n, count), n


def run_reference(args, rank):
    if rank != 0:
        return
    pr = _workload()
    att = _att_table()
    threads = cpu_threads()
    P = _pairs(pr.nr_rings_used, pr.nr_detectors_used)
    idx, n_all = stratified_sample(pr, args.ref_points)
    units = len(idx) * P * pr.nr_bins
    times = []
    for i in range(args.warmup + args.steps):
        _, dt = oracle_sample(pr, att, idx, threads)
        if i >= args.warmup:
            times.append(dt)
    t = statistics.mean(times) if times else float("nan")
    v = units / t
    sample = (f"{len(idx)} of the workload's {n_all} scatter points, evenly spread in lattice order "
              f"({units:.3e} units per step)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": _config(pr, {"sample_points": len(idx)}),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "statistic": "mean over steps"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU side


def run_ours(args, rank, world, local_rank):
    import torch

    from opensss_gb300 import TofSSS, _lib
    from opensss_gb300.engine import fortran_flat, leg_pair_to_compact
    from opensss_gb300.replicas import max_over_ranks

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    pr = _workload()
    att = _att_table()
    L = _lib.lib()
    eng = TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att,
                 pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                 pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins, device=dev)
    act = torch.from_numpy(np.ascontiguousarray(pr.activity)).to(dev)
    mu = torch.from_numpy(np.ascontiguousarray(pr.attenuation)).to(dev)
    P = _pairs(pr.nr_rings_used, pr.nr_detectors_used)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # scatter points of this workload
    act_f, mu_f = fortran_flat(act, dev), fortran_flat(mu, dev)
    p = eng.problem(act_f, mu_f, pr.grid, pr.image_size)
    pts, counts = eng.scatter_points(p)
    nsp = int(counts.sum()) if args.max_points is None else min(int(counts.sum()), args.max_points)
    units = nsp * P * pr.nr_bins

    # launch shapes picked by the tuner on the first 400 scatter points (untimed)
    from opensss_gb300 import autotune

    tuned = None if args.no_autotune else autotune.tune(eng, act, mu, pr.image_size, sample_points=400,
                                                        use_cache=False)
    L.sss_set_timing(1)
    out = torch.empty((pr.nr_bins, eng.nl, eng.nl), dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        eng.run(act, mu, pr.image_size, out=out, max_points=args.max_points)
    stage = np.zeros(6)
    step_ms = []
    pair_ms = []
    leg_ms = []
    launches = 0
    with ClockSampler(local_rank) as clk:
        barrier()
        torch.cuda.synchronize(dev)
        for _ in range(args.steps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.run(act, mu, pr.image_size, out=out, check=False, max_points=args.max_points)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            L.sss_get_timing(stage.ctypes.data_as(C.c_void_p))
            leg_ms.append(stage[0])
            pair_ms.append(stage[1])
            launches += 1 + int(stage[2])  # scatter-point kernel + per-wave leg and pair kernels
        torch.cuda.synchronize(dev)
        barrier()
    _lib.check_status(int(eng._status.item()))
    clocks = clk.summary()
    total_s = max_over_ranks(sum(step_ms) / 1e3, dev)
    value = world * units * args.steps / total_s

    # ---- end to end through the drop-in SingleScatterSimulationTOF: NumPy maps
    # in, the reference's dense (B, ND+1, ND//2, NRU^2) float32 array out; the
    # map uploads, the run, the densify and the device-to-host copy are timed
    dropin = run_dropin(pr, att, dev, args)

    # ---- end to end through the engine (TofSSS.run): pinned host volumes in,
    # the compact leg-pair result copied back
    act_h = torch.from_numpy(np.ascontiguousarray(pr.activity)).pin_memory()
    mu_h = torch.from_numpy(np.ascontiguousarray(pr.attenuation)).pin_memory()
    res_h = torch.empty((pr.nr_bins, eng.nl, eng.nl), dtype=torch.float32).pin_memory()
    e2e_s = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        a = act_h.to(dev, non_blocking=True)
        m = mu_h.to(dev, non_blocking=True)
        r = eng.run(a, m, pr.image_size, out=out, check=False, max_points=args.max_points)
        res_h.copy_(r, non_blocking=True)
        torch.cuda.synchronize(dev)
        if i >= args.warmup:
            e2e_s.append(time.perf_counter() - t0)
    e2e_total = max_over_ranks(sum(e2e_s), dev)
    engine_e2e = {"value": world * units * args.steps / e2e_total, "unit": UNIT,
                  "h2d_bytes_per_step": act_h.numel() * 4 + mu_h.numel() * 4,
                  "d2h_bytes_per_step": res_h.numel() * 4,
                  "path": "TofSSS.run on pinned host volumes, compact leg-pair result copied back"}
    dropin_total = max_over_ranks(dropin["seconds"] * args.steps, dev)
    e2e = {"value": world * units * args.steps / dropin_total, "unit": UNIT,
           "h2d_bytes_per_step": dropin["h2d_bytes"], "d2h_bytes_per_step": dropin["d2h_bytes"],
           "ms_per_step": dropin["seconds"] * 1e3,
           "path": "opensss_gb300.SingleScatterSimulationTOF (the drop-in): NumPy maps in, the reference's "
                   f"dense {dropin['shape']} float32 array out (pageable host memory in, page-locked out; the "
                   "host's cores clear the result during the simulation and the GPU writes its sampled cells "
                   "over the host link)"}
    L.sss_set_timing(0)

    if rank != 0:
        return
    # ---- roofline of the dominant kernel.  The pair kernel reads, per
    # (voxel of a walked leg, detector pair), the bins' TOF factors (4 B a
    # bin) and the voxel's activity x length and distance (8 B): the per-unit
    # bytes of the reference's TOF-table gather, taken from shared memory.
    pair_s = statistics.mean(pair_ms) / 1e3
    walked = stage[4] / pr.nr_bins if stage[4] > 0 else None  # (voxel, pair) terms of one step
    alg_bytes = walked * (4 * pr.nr_bins + 8) if walked else None
    peaks = _probe_peaks()
    achieved = alg_bytes / pair_s / 1e9 if alg_bytes else None
    # FP32 work of the weights: per term and bin one FMA into the bin's sum and
    # one multiply of the running power (3 flops); SFU: 2^x of the two legs'
    # attenuation terms per evaluated pair and scatter point
    fp32_gflops = 3 * stage[4] / pair_s / 1e9 if stage[4] > 0 else None
    sfu_g = 2 * stage[5] / pair_s / 1e9 if stage[5] > 0 else None
    roof = {"bound": "smem", "unit": "GB/s", "kernel": "pair_kernel", "achieved": achieved,
            "peak": peaks["smem"], "peak_source": "measured (sss_probe_smem_rate, this run)",
            "frac": achieved / peaks["smem"] if achieved and peaks["smem"] else None,
            "traffic": None,
            "traffic_note": "DRAM bytes come from an ncu capture only, not from this run; "
                            "the TOF factors are read from shared memory, not DRAM",
            "algorithmic_bytes_per_launch": alg_bytes,
            "bytes_rule": "(4 B x bins + 8 B) per (voxel, detector pair) term walked",
            "terms_per_launch": walked, "launch_ms": pair_s * 1e3,
            "fp32_pipe": {"achieved_gflops": fp32_gflops, "peak_gflops": peaks["ffma"],
                          "frac": fp32_gflops / peaks["ffma"] if fp32_gflops and peaks["ffma"] else None,
                          "rule": "3 flops (FMA + power multiply) per (voxel, pair) term and bin",
                          "peak_source": "measured (sss_probe_ffma_rate, FFMA2 chains, this run)"},
            "sfu": {"achieved_g_per_s": sfu_g, "peak_g_per_s": peaks["ex2"],
                    "frac": sfu_g / peaks["ex2"] if sfu_g and peaks["ex2"] else None,
                    "rule": "two 2^x per evaluated (pair, scatter point)",
                    "peak_source": "measured (sss_probe_ex2_rate, this run)"},
            "l2_reference_gather": {
                "achieved": achieved, "peak": peaks["l2"], "unit": "GB/s",
                "frac": achieved / peaks["l2"] if achieved and peaks["l2"] else None,
                "peak_source": "measured (sss_probe_l2_rate, 32 MB L2-resident, this run)",
                "note": "same bytes against the L2 load bandwidth a TOF-table gather would be bound by"},
            "weights_per_s": stage[4] / pair_s if stage[4] > 0 else None}

    # ---- CPU baseline (oracle port on the host cores) and the error against
    # FP64 on the same stratified sample of scatter points
    cpu = None
    err = None
    if world == 1 and not args.no_cpu:
        threads = cpu_threads()
        idx, n_all = stratified_sample(pr, args.ref_points)
        ref, dt = oracle_sample(pr, att, idx, threads)
        u = len(idx) * P * pr.nr_bins
        cpu = {"value": u / dt, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{len(idx)} of the workload's {n_all} scatter points, evenly spread in lattice "
                         f"order ({u:.3e} units)"}
        sub = eng.run(act, mu, pr.image_size, points=idx).cpu().numpy()
        got = leg_pair_to_compact(sub, pr.nr_rings_used, pr.nr_detectors_used)
        err = {"rel_l2": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
               "max_bin": float(np.abs(got - ref).max() / np.abs(ref).max()),
               "sample": cpu["sample"]}

    pipeline = None if args.no_pipeline else run_pipeline(eng, pr, out, dev, args)
    batch = None if args.no_batch or world > 1 else run_batch(dev, args, att)
    precision = None if args.no_precision or world > 1 else run_precision(dev, args, att)
    serving = None if args.no_serving or world > 1 else run_serving(dev, args, att)
    listmode = None if args.no_listmode or world > 1 else run_listmode(dev, args)
    prep = None if args.no_prep or world > 1 else run_prep(dev, args)

    ms = 1e3 * total_s / args.steps
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 ray walk)",
            "data": "synthetic", "config": _config(pr, {"scatter_points": nsp,
                                                        "detector_pairs": P,
                                                        "units_per_step": units}),
            "e2e": e2e, "e2e_engine": engine_e2e, "dropin": dropin,
            "gpu_launches": launches, "clocks": clocks, "roofline": roof,
            "launch_shape": {"pair_warps": eng.pair_warps, "leg_threads": eng.leg_threads,
                             "tuned": tuned},
            "stages_ms": {"legs": statistics.mean(leg_ms), "pairs": statistics.mean(pair_ms)},
            "device_rates": {"fp64_add_g_per_s": peaks["dadd"], "fp64_div_g_per_s": peaks["ddiv"],
                             "ffma2_gflops": peaks["ffma"],
                             "ex2_g_per_s": peaks["ex2"], "smem_gbs": peaks["smem"], "l2_gbs": peaks["l2"],
                             "source": "probe kernels of libsss300_probe.so, this run"},
            "error_vs_fp64_oracle": err, "cpu_baseline": cpu, "pipeline": pipeline,
            "batch": batch, "precision": precision, "serving": serving, "listmode": listmode,
            "image_prep": prep}
    print(json.dumps(line), flush=True)


def run_dropin(pr, att, dev, args):
    """The drop-in call a reference script makes, timed on the host clock:
    ``SingleScatterSimulationTOF`` with NumPy maps and the LOR table, the
    dense float32 result returned.  Warm-up calls build and cache the engine
    and page-locked output memory; each timed call drops its result before
    the next."""
    import contextlib
    import io

    import torch

    from opensss_gb300 import SingleScatterSimulationTOF, geometry as G

    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, pr.scanner.nr_detectors, pr.scanner.nr_rings, ID_Shidt=False)
    args_ = (pr.image_size, pr.scanner.geometry, lor, pr.scanner.normals, pr.scanner.detector_size_mm, att,
             pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step,
             pr.tof_resolution, pr.tof_range, pr.nr_bins, None)
    act = np.ascontiguousarray(pr.activity)
    mu = np.ascontiguousarray(pr.attenuation)
    times, shape = [], None
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize(dev)
        with contextlib.redirect_stdout(io.StringIO()):  # the reference's timing print
            t0 = time.perf_counter()
            dense = SingleScatterSimulationTOF(act, mu, *args_, device=dev)
            t1 = time.perf_counter()
        shape = list(dense.shape)
        nbytes = dense.nbytes
        del dense
        if i >= args.warmup:
            times.append(t1 - t0)
    return {"seconds": statistics.mean(times), "shape": shape, "h2d_bytes": act.nbytes + mu.nbytes,
            "d2h_bytes": nbytes, "ms_min": min(times) * 1e3, "ms_max": max(times) * 1e3}


def run_pipeline(eng, pr, sampled, dev, args):
    """Downstream rows on the same scanner: upsampling of all bins, tail mask,
    and the per-bin scale fit, each timed with CUDA events.  Prompts are
    seeded Poisson draws of 1.4 x the upsampled scatter plus flat randoms
    (trues are zero on the tail LORs the fit uses), so every fitted scale
    should come out near 1.4."""
    import torch

    from opensss_gb300 import geometry as G
    from opensss_gb300.BackProjection import fit_bins_device, fit_device
    from opensss_gb300.Interpolation import upsample_device
    from opensss_gb300.TailsMask import tail_mask_device

    nd, nr = pr.scanner.nr_detectors, pr.scanner.nr_rings
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    tables = G.upsample_tables(lor, si, pr.nr_rings_used, pr.nr_detectors_used, "legpair")
    ncell, nsl = (nd + 1) * (nd // 2), nr * nr
    cs = torch.from_numpy(tables[0]).to(dev)
    rs = torch.from_numpy(tables[1]).to(dev)
    t_tables = tables
    st = torch.cuda.current_stream(dev)

    def timed(fn, reps=3):
        """One untimed call (allocations, table uploads), then the mean of
        ``reps`` calls timed with CUDA events."""
        fn()
        ms = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            r = fn()
            e1.record(st)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return r, statistics.mean(ms)

    up = torch.empty((ncell, nsl), dtype=torch.float32, device=dev)
    _, up_ms = timed(lambda: upsample_device(sampled, t_tables, pr.nr_bins, ncell, nsl, out=up))
    af = args.af
    mask, mask_ms = timed(lambda: tail_mask_device(pr.attenuation, pr.image_size, pr.scanner.geometry,
                                                   lor, si, af, device=dev))
    fit_grid = np.array([40, 40, 26])
    zr = float(pr.scanner.geometry[-1, 0, 2]) + 0.16
    fit_bounds = np.array([pr.image_size[0], pr.image_size[1], -zr, pr.image_size[3], pr.image_size[4], zr])
    order = si[:nr, :nr].T
    gen = torch.Generator(device=dev)
    gen.manual_seed(7)
    randoms = torch.full((ncell, nsl), 0.1 * 1.4 * 20.0, dtype=torch.float32, device=dev)
    # prompts of every bin: Poisson(1.4 x scatter + randoms), each bin scaled to
    # ~20 counts per sinogram bin on average (SSS values are probabilities)
    nb = pr.nr_bins
    prompts = torch.empty((nb, ncell, nsl), dtype=torch.float32, device=dev)
    counts_per_unit = []
    for b in range(nb):
        upsample_device(sampled, t_tables, nb, ncell, nsl, bin_index=b, out=up)
        k = 20.0 / max(float(up.mean()), 1e-30)
        counts_per_unit.append(k)
        prompts[b] = torch.poisson(1.4 * k * up + randoms, generator=gen)
    del up
    # one bin alone (the reference's per-bin call), then all bins in one pass
    bc = nb // 2
    s1, one_ms = timed(lambda: fit_device(prompts[bc], randoms, mask, sampled[bc], cs, rs, fit_grid, fit_bounds,
                                          pr.scanner.geometry, lor, order, af, scat_clamp=True, device=dev))
    nl2 = int(sampled[0].numel())
    sc, all_ms = timed(lambda: fit_bins_device(prompts, randoms, mask, sampled, nl2, cs, rs, fit_grid, fit_bounds,
                                               pr.scanner.geometry, lor, order, af, scat_clamp=True, device=dev))
    scales = [float(sc[b]) / counts_per_unit[b] for b in range(nb)]
    n_mask_lors = int(mask.sum())
    del prompts
    return {"upsample_all_bins_ms": up_ms, "upsample_gbs": ncell * nsl * 4 / (up_ms * 1e-3) / 1e9,
            "tail_mask_ms": mask_ms, "mask_af": af, "masked_bins": n_mask_lors,
            "fit_one_bin_ms": one_ms, "fit_all_bins_ms": all_ms, "fit_bins": nb,
            "fit_one_bin_scale": s1 / counts_per_unit[bc], "fitted_scales": scales,
            "expected_scale": 1.4, "full_sinogram": [nd + 1, nd // 2, nsl]}


def run_batch(dev, args, att):
    """The uneven batch: 64 seeded instances (33..95 voxels across a 40 cm
    FOV, 24..64 crystals x 8..24 rings, 1/13/33 TOF bins) planned once and
    replayed as one CUDA graph per step, inputs resident on the device.
    Compared with the same instances run one after another through
    TofSSS.run (the plain per-problem path)."""
    import torch

    from opensss_gb300 import TofSSS, workloads as W
    from opensss_gb300.batch import BatchSSS
    from opensss_gb300.engine import fortran_flat

    inst = W.uneven_instances(args.batch_size, seed=0)
    engines, jobs = [], []
    for pr in inst:
        e = TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att,
                   pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                   pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins, device=dev)
        engines.append(e)
        jobs.append((e, fortran_flat(pr.activity, dev), fortran_flat(pr.attenuation, dev), pr.image_size,
                     pr.grid))
    t0 = time.perf_counter()
    b = BatchSSS(jobs, autotune=not args.no_autotune)
    torch.cuda.synchronize(dev)
    plan_s = time.perf_counter() - t0
    b.run()  # checked run (status word) before capturing
    b.capture()
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        b.replay(check=False)
    steps = max(1, min(args.steps, args.batch_steps))
    ms = []
    with ClockSampler(dev.index or 0) as clk:
        torch.cuda.synchronize(dev)
        for _ in range(steps):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            b.replay(check=False)
            e1.record(st)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
    b.replay(check=True)
    # plain path: the same problems one after another (one warm-up pass of the smallest)
    engines[0].run(inst[0].activity, inst[0].attenuation, inst[0].image_size)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for (e, a, m, size, shape) in jobs:
        e.run_flat(a, m, shape, size, check=False)
        e._ws = None  # stream-ordered reuse: the next instance takes the same memory
    e1.record(st)
    e1.synchronize()
    solo_ms = e0.elapsed_time(e1)
    mean_ms = statistics.mean(ms)
    res = {"workload": f"{len(inst)} uneven instances (seed 0)", "units_per_step": b.units,
           "scatter_points": b.points, "waves": b.waves, "launches_per_step": b.launches,
           "graph": True, "launch_shapes": b.tuned, "steps": steps, "ms_per_step": mean_ms,
           "value": b.units / (mean_ms / 1e3),
           "unit": UNIT, "plan_s": plan_s, "plan_includes_autotune": not args.no_autotune,
           "plain_sequential_ms": solo_ms,
           "plain_sequential_value": b.units / (solo_ms / 1e3),
           "speedup_vs_plain": solo_ms / mean_ms, "clocks": clk.summary(),
           "plain_note": "scatter points, host sync and leg/pair waves per instance, kernels only"}
    b.close()
    del b
    torch.cuda.empty_cache()
    res["small_instances"] = _small_batch(dev, args, att)
    return res


def _small_batch(dev, args, att):
    """64 bed positions of the plain non-TOF size (40x40x20 @ 1 cm, 8 x 32
    virtual, phantoms seeded per bed): one graph replay of the batch against
    the same problems one after another through TofSSS.run_flat."""
    import torch

    from opensss_gb300 import TofSSS, workloads as W
    from opensss_gb300.batch import BatchSSS
    from opensss_gb300.engine import fortran_flat

    inst = [W.nontof_40x40x20(seed=100 + i) for i in range(64)]
    pr0 = inst[0]
    e = TofSSS(pr0.scanner.geometry, pr0.scanner.normals, pr0.scanner.detector_size_mm, att,
               pr0.energy_resolution, pr0.energy_threshold, pr0.nr_rings_used, pr0.nr_detectors_used,
               pr0.sample_step, pr0.tof_resolution, pr0.tof_range, pr0.nr_bins, device=dev)
    jobs = [(e, fortran_flat(pr.activity, dev), fortran_flat(pr.attenuation, dev), pr.image_size, pr.grid)
            for pr in inst]
    b = BatchSSS(jobs)
    b.run()
    b.capture()
    st = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        b.replay(check=False)
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        b.replay(check=False)
        e1.record(st)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    b.replay(check=True)
    for (_, a, m, size, shape) in jobs[:4]:
        e.run_flat(a, m, shape, size, check=False)  # warm-up of the plain path
    plain = []
    for _ in range(args.steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for (_, a, m, size, shape) in jobs:
            e.run_flat(a, m, shape, size, check=False)
        torch.cuda.synchronize(dev)
        plain.append((time.perf_counter() - t0) * 1e3)
    mean_ms, plain_ms = statistics.mean(ms), statistics.mean(plain)
    out = {"workload": "64 plain non-TOF beds, 40x40x20 @ 1 cm, 8 x 32 virtual", "units_per_step": b.units,
           "waves": b.waves, "launches_per_step": b.launches, "ms_per_step": mean_ms,
           "value": b.units / (mean_ms / 1e3), "plain_sequential_ms": plain_ms,
           "plain_note": "wall time of 64 TofSSS.run_flat calls (each synchronises once for its scatter points)",
           "speedup_vs_plain": plain_ms / mean_ms}
    b.close()
    return out


def run_precision(dev, args, att):
    """The precision-stress instance: 128x128x96 @ 4 mm, 32 rings x 96
    crystals, 33 TOF bins of 15 mm.  Full-size throughput of the plain launch
    and of the precision launch ("kahan": SSS_FLAG_KAHAN, Kahan-compensated
    scatter-point reduction and float-pair TOF offsets), then both against the
    FP64 GPU oracle (the C restatement's SSS run on the GPU, oracle/
    sss_oracle_gpu.cu) on a sample of scatter points: relative L2, largest bin
    error (over the largest reference bin) and the fitted scale of the centre
    TOF bin (prompts drawn from the FP64 scatter).  The sample is one scatter
    point in ``--precision-every``, spread evenly over the workload in
    lattice order (1: the whole workload)."""
    import torch

    from opensss_gb300 import TofSSS, geometry as G, workloads as W
    from opensss_gb300.BackProjection import fit_device
    from opensss_gb300.engine import compact_to_leg_pair, fortran_flat, leg_pair_to_compact
    from opensss_gb300.Interpolation import upsample_device
    from opensss_gb300.TailsMask import tail_mask_device

    pr = W.tof33_128x128x96(seed=0)
    eng = TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att,
                 pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                 pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins, device=dev)
    act, mu = fortran_flat(pr.activity, dev), fortran_flat(pr.attenuation, dev)
    p = eng.problem(act, mu, pr.grid, pr.image_size)
    _, counts = eng.scatter_points(p)
    nsp = int(counts.sum())
    units = nsp * _pairs(pr.nr_rings_used, pr.nr_detectors_used) * pr.nr_bins
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    full = {}
    with ClockSampler(dev.index or 0) as clk:
        for kahan in (False, True):
            for _ in range(args.precision_warmup):
                eng.run_flat(act, mu, pr.grid, pr.image_size, kahan=kahan)
            ms = []
            for _ in range(args.precision_steps):
                flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                eng.run_flat(act, mu, pr.grid, pr.image_size, kahan=kahan, check=False)
                e1.record(st)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
            key = "kahan" if kahan else "plain"
            full[key] = {"ms_per_step": statistics.mean(ms), "value": units / (statistics.mean(ms) / 1e3),
                         "steps": args.precision_steps, "warmup": args.precision_warmup}
    eng._ws = None
    # errors on a stratified sample (every sampled z-slice) against the FP64 oracle
    from oracle import oracle as O

    n_all = len(O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)[0])
    idx = W.stratified_points(n_all, max(1, n_all // max(1, args.precision_every)))
    n = len(idx)
    t0 = time.perf_counter()
    ref = O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry, pr.scanner.normals,
                        pr.scanner.detector_size_mm, att, pr.energy_resolution, pr.energy_threshold,
                        pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step, pr.tof_resolution, pr.tof_range,
                        pr.nr_bins, points=idx, gpu=True)
    oracle_s = time.perf_counter() - t0
    nru, ndu = pr.nr_rings_used, pr.nr_detectors_used
    outs = {k: eng.run_flat(act, mu, pr.grid, pr.image_size, points=idx, kahan=(k == "kahan"))
            for k in ("plain", "kahan")}
    err = {}
    for k, o in outs.items():
        got = leg_pair_to_compact(o.cpu().numpy(), nru, ndu).astype(np.float64)
        err[k] = {"rel_l2": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
                  "max_bin": float(np.abs(got - ref).max() / np.abs(ref).max())}
    # fitted scale of the centre bin
    nd, nr = pr.scanner.nr_detectors, pr.scanner.nr_rings
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    tables = G.upsample_tables(lor, si, nru, ndu, "legpair")
    cs, rs = torch.from_numpy(tables[0]).to(dev), torch.from_numpy(tables[1]).to(dev)
    ncell, nsl = (nd + 1) * (nd // 2), nr * nr
    b = pr.nr_bins // 2
    ref_lp = torch.from_numpy(compact_to_leg_pair(ref.astype(np.float32), nru, ndu)[b]).to(dev)
    up = upsample_device(ref_lp.reshape(1, -1), tables, 1, ncell, nsl)
    k = 20.0 / max(float(up.mean()), 1e-30)
    randoms = torch.full_like(up, 0.1 * 1.4 * 20.0)
    gen = torch.Generator(device=dev)
    gen.manual_seed(11)
    prompts = torch.poisson(1.4 * k * up + randoms, generator=gen)
    del up
    mask = tail_mask_device(pr.attenuation, pr.image_size, pr.scanner.geometry, lor, si, args.af, device=dev)
    zr = float(pr.scanner.geometry[-1, 0, 2]) + 0.16
    fit_bounds = np.array([pr.image_size[0], pr.image_size[1], -zr, pr.image_size[3], pr.image_size[4], zr])
    order = si[:nr, :nr].T

    def fit(scatter_lp):
        return fit_device(prompts, randoms, mask, scatter_lp, cs, rs, np.array([40, 40, 26]), fit_bounds,
                          pr.scanner.geometry, lor, order, args.af, scat_clamp=True, device=dev) / k

    s_ref = fit(ref_lp)
    for key, o in outs.items():
        s = fit(o[b].contiguous())
        err[key]["fitted_scale"] = s
        err[key]["fitted_scale_rel_err"] = abs(s - s_ref) / abs(s_ref)
    del prompts, randoms, mask
    torch.cuda.empty_cache()
    return {"workload": pr.name, "volume": list(pr.grid), "sampled_rings": nru, "sampled_crystals": ndu,
            "tof_bins": pr.nr_bins, "scatter_points": nsp, "units_per_step": units, "full": full,
            "clocks": clk.summary(),
            "error_vs_fp64_oracle": err, "fp64_fitted_scale": s_ref, "fit_bin": b,
            "sample": f"{n} of {n_all} scatter points, evenly spread in lattice order "
                      f"({n * _pairs(nru, ndu) * pr.nr_bins:.3e} units)",
            "fp64_oracle": "oracle/sss_oracle_gpu.cu: the FP64 C restatement's SSS on this GPU (shared "
                           "arithmetic in oracle/orc_core.h, no fused multiply-adds)",
            "fp64_oracle_seconds": oracle_s,
            "kahan": "SSS_FLAG_KAHAN: Kahan-compensated scatter-point sums and TOF offsets from float-pair "
                     "distances and samples"}


def run_serving(dev, args, att):
    """The served workload: seeded Poisson arrivals (``--serve-rate`` req/s for
    ``--serve-seconds``), 70% small requests (four plain non-TOF bed positions,
    40x40x20 @ 1 cm, 8 x 32 virtual) and 30% large ones (four beds drawn by the
    uneven-batch generator), each a scatter update with the bed's activity
    times 1 +- 5% seeded noise.  The batching server (admission by an 80 GB
    HBM budget, continuous batching at wave granularity) against the plain
    path, one request at a time in arrival order, on the same stream."""
    from opensss_gb300 import TofSSS, workloads as W
    from opensss_gb300.engine import leg_pair_to_compact
    from opensss_gb300.serving import (PlainServer, ScatterServer, latency_summary, make_bed,
                                       poisson_stream, request_activity)
    from oracle import oracle as O

    small, large = W.served_beds()
    beds = []
    for pr, is_large in [(p, False) for p in small] + [(p, True) for p in large]:
        e = TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att,
                   pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                   pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins, device=dev)
        beds.append(make_bed(e, pr.activity, pr.attenuation, pr.image_size, large=is_large))
    problems = small + large
    # warm-up stream (first launches of every kernel shape)
    ScatterServer(beds).serve(poisson_stream(args.serve_rate, 0.05, beds, 0.7, seed=1))
    PlainServer(beds).serve(poisson_stream(args.serve_rate, 0.02, beds, 0.7, seed=1))
    with ClockSampler(dev.index or 0) as clk:
        srv = ScatterServer(beds, hbm_budget=80 << 30)
        served = srv.serve(poisson_stream(args.serve_rate, args.serve_seconds, beds, 0.7, seed=2026))
        plain = PlainServer(beds).serve(poisson_stream(args.serve_rate, args.serve_seconds, beds, 0.7,
                                                       seed=2026))
    s, p = latency_summary(served, beds), latency_summary(plain, beds)
    offered = sum(beds[r.bed].units for r in served) / args.serve_seconds
    # served results against the FP64 oracle: small requests whole, large
    # ones on a stratified sample of their scatter points (the served result
    # is first compared with the same request run alone, 1e-5, then that
    # run's point sample with the oracle's)
    errs_small, errs_large, solo_large = [], [], []
    for r in [r for r in served if not beds[r.bed].large][:args.serve_check]:
        bed, pr = beds[r.bed], problems[r.bed]
        act = request_activity(bed, r.seed).cpu().numpy().reshape(bed.shape, order="F")
        ref = O.sss_compact(act, pr.attenuation, pr.image_size, pr.scanner.geometry, pr.scanner.normals,
                            pr.scanner.detector_size_mm, att, pr.energy_resolution, pr.energy_threshold,
                            pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step, pr.tof_resolution,
                            pr.tof_range, pr.nr_bins, nthreads=cpu_threads())
        got = leg_pair_to_compact(r.out.cpu().numpy(), pr.nr_rings_used, pr.nr_detectors_used)
        errs_small.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    seen_beds = set()
    for r in [r for r in served if beds[r.bed].large]:
        if r.bed in seen_beds or len(seen_beds) >= 2:
            continue
        seen_beds.add(r.bed)
        bed, pr = beds[r.bed], problems[r.bed]
        act_t = request_activity(bed, r.seed)
        alone = bed.engine.run_flat(act_t, bed.mu, bed.shape, bed.image_size).cpu().numpy()
        solo_large.append(float(np.linalg.norm(r.out.cpu().numpy() - alone) / np.linalg.norm(alone)))
        idx = W.stratified_points(int(bed.counts.sum()), 16)
        sub = bed.engine.run_flat(act_t, bed.mu, bed.shape, bed.image_size, points=idx).cpu().numpy()
        act = act_t.cpu().numpy().reshape(bed.shape, order="F")
        ref = O.sss_compact(act, pr.attenuation, pr.image_size, pr.scanner.geometry, pr.scanner.normals,
                            pr.scanner.detector_size_mm, att, pr.energy_resolution, pr.energy_threshold,
                            pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step, pr.tof_resolution,
                            pr.tof_range, pr.nr_bins, points=idx, nthreads=cpu_threads())
        got = leg_pair_to_compact(sub, pr.nr_rings_used, pr.nr_detectors_used)
        errs_large.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    sweep = run_serving_sweep(beds, args)
    return {"workload": f"Poisson {args.serve_rate:g} req/s for {args.serve_seconds:g} s (seed 2026), "
                        "70% small / 30% large over 8 resident beds",
            "beds": [{"name": pr.name, "volume": list(pr.grid), "rings": pr.nr_rings_used,
                      "crystals": pr.nr_detectors_used, "bins": pr.nr_bins, "units": b.units}
                     for pr, b in zip(problems, beds)],
            "offered_units_per_s": offered, "hbm_budget_gb": 80, "served": s, "plain": p,
            "p99_speedup": p["p99_ms"] / s["p99_ms"], "throughput_ratio": s["units_per_s"] / p["units_per_s"],
            "server_stats": dict(srv.stats), "clocks": clk.summary(),
            "rel_l2_vs_fp64_small": errs_small, "rel_l2_served_vs_alone_large": solo_large,
            "rel_l2_vs_fp64_large_sample": errs_large,
            "large_sample": "16 scatter points spread evenly over the bed's points, same points in the oracle",
            "sweep": sweep}


def run_serving_sweep(beds, args):
    """Latency against offered rate: the same 70/30 mix at several Poisson
    rates for ``--sweep-seconds`` of arrivals each, the batching server and the
    plain one, and the highest rate each sustains: p99 under
    ``--p99-bound-ms`` and requests completed at no less than 90% of the rate
    they arrived (no growing backlog)."""
    from opensss_gb300.serving import PlainServer, ScatterServer, latency_summary, poisson_stream

    rates = [float(x) for x in args.sweep_rates.split(",") if x]
    rows = []
    for rate in rates:
        row = {"rate": rate}
        for name, mk in (("served", lambda: ScatterServer(beds, hbm_budget=80 << 30)),
                         ("plain", lambda: PlainServer(beds))):
            reqs = mk().serve(poisson_stream(rate, args.sweep_seconds, beds, 0.7, seed=int(rate * 10) + 7))
            summ = latency_summary(reqs, beds)
            row[name] = {k: summ[k] for k in ("requests", "p50_ms", "p99_ms", "small_p99_ms", "large_p99_ms",
                                              "requests_per_s", "makespan_s")}
        rows.append(row)

    def best(name):
        ok = [r["rate"] for r in rows
              if r[name]["p99_ms"] is not None and r[name]["p99_ms"] <= args.p99_bound_ms
              and r[name]["requests_per_s"] >= 0.9 * r[name]["requests"] / args.sweep_seconds]
        return max(ok) if ok else None

    return {"rates": rates, "seconds": args.sweep_seconds, "p99_bound_ms": args.p99_bound_ms, "rows": rows,
            "sustained_rate_served": best("served"), "sustained_rate_plain": best("plain")}


def run_prep(dev, args):
    """Image preparation (CropAndDownscale): a seeded 400x400x280 map of
    1.6 mm x 1.6 mm x 2 mm voxels (179 MB, above the L2) cropped to
    600 x 600 x 480 mm (376 x 376 x 240 voxels) and resized to 75 x 75 x 48
    voxels of 8 x 8 x 10 mm (anti-aliasing sigma 2 voxels).  GPU time with the map resident, end to end from a host
    array, and the scipy.ndimage restatement of the reference's resize on the
    host (the oracle, one run)."""
    import torch

    from opensss_gb300 import Utils

    rng = np.random.default_rng(3)
    img = rng.gamma(2.0, 1.0, size=(400, 400, 280)).astype(np.float32)
    vox, crop, dims = (1.6, 1.6, 2.0), (600.0, 600.0, 480.0), (75, 75, 48)
    t = torch.from_numpy(img).to(dev)
    win = Utils.crop_window(img.shape, vox, crop)
    st = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        Utils.crop_downscale_device(t, win, dims)
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        out = Utils.crop_downscale_device(t, win, dims)
        e1.record(st)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    e2e = []
    for _ in range(args.steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        host = Utils.CropAndDownscale(img, vox, crop, dims)
        e2e.append((time.perf_counter() - t0) * 1e3)
    res = {"workload": "400x400x280 float32 map, crop 600x600x480 mm, resize to 75x75x48 (order 3, anti-aliased)",
           "ms": statistics.mean(ms), "e2e_ms": statistics.mean(e2e), "input_gb": img.nbytes / 1e9,
           "h2d_bytes": img.nbytes, "d2h_bytes": int(np.prod(dims)) * 4}
    if not args.no_cpu:
        from oracle import prep as P

        t0 = time.perf_counter()
        ref = P.crop_and_downscale(img, vox, crop, dims)
        cpu_ms = (time.perf_counter() - t0) * 1e3
        res["cpu_baseline"] = {"ms": cpu_ms, "cores": 1, "kind": "port",
                               "sample": "the whole map, scipy.ndimage gaussian_filter + zoom (float32)"}
        res["max_err_vs_oracle"] = float(np.abs(host.astype(np.float64) - ref).max() / np.abs(ref).max())
        del out
    return res


def run_listmode(dev, args):
    """Prompt histogramming of ``--listmode-events`` seeded list-mode events
    (TOF, randoms and normalisation fields, 24-byte records) of the
    760-crystal x 80-ring scanner with the demo's data reduction (mash 2,
    span 19, MRD 79: 381 x 190 x 815 cells) into 6 TOF bins.  Device-resident
    events (``value``) and through the drop-in path with the events in pinned
    host memory and the uint16 sinogram copied back (``e2e``); the CPU
    baseline is the host restatement of the reference's per-event loop on
    the first ``--listmode-cpu-events`` events."""
    import struct

    import torch

    from opensss_gb300 import Coincidence, Datafile, DataReduction as D, geometry as G, workloads as W

    n = args.listmode_events
    header = W.listmode_header("bench_df", n)
    ev = W.synthetic_events(header, 760, 80, seed=2026)
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, 380, 80, ID_Shidt=False)
    _, _, lut, _ = D.SinogramLUT(80, 19, 79)
    raw = torch.from_numpy(ev.view(np.uint8).reshape(-1))
    ev_h = raw.pin_memory()
    ev_d = ev_h.to(dev)
    st = torch.cuda.current_stream(dev)

    def once(events):
        return Datafile.histogram_device(events, header, lor, lut, 6, 1000.0, mash=2, Shift=0, device=dev)

    for _ in range(args.warmup):
        once(ev_d)
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        once(ev_d)
        e1.record(st)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    e2e = []
    for _ in range(args.steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        p, r, nrm = once(ev_h.to(dev, non_blocking=True))
        host = (p.cpu(), r.cpu(), nrm.cpu())
        e2e.append(time.perf_counter() - t0)
    out_bytes = sum(t.numel() * t.element_size() for t in host)
    # CPU: the reference's loop restated (struct.iter_unpack + ParseCASToRIDs per event)
    m = min(n, args.listmode_cpu_events)
    fmt, pos = Coincidence.GenerateEventClass(header)
    table = lut
    t0 = time.perf_counter()
    acc = 0
    for e in struct.iter_unpack(fmt, ev[:m].tobytes()):
        d1, r1, d2, r2, tof = Coincidence.ParseCASToRIDs(e, pos, 760, 0)
        a, rr = lor[d1 // 2, d2 // 2]
        s = table[r1, r2]
        if s == -1 or rr == -1 or a == -1 or abs(tof) > 1000.0:
            continue
        t = (tof + 1000.0) / (2 * 1000.0 / 6)
        acc += 0 <= t < 6
    cpu_s = time.perf_counter() - t0
    mean_ms = statistics.mean(ms)
    return {"workload": f"{n} seeded list-mode events, 760 x 80 scanner, mash 2, span 19 (381x190x815 cells), "
                        "6 TOF bins", "unit": "events/s", "value": n / (mean_ms / 1e3), "ms_per_step": mean_ms,
            "steps": args.steps, "warmup": args.warmup,
            "e2e": {"value": n / statistics.mean(e2e), "unit": "events/s", "h2d_bytes_per_step": int(raw.numel()),
                    "d2h_bytes_per_step": int(out_bytes)},
            "gbs_event_read": raw.numel() / (mean_ms / 1e3) / 1e9,
            "cpu_baseline": {"value": m / cpu_s, "unit": "events/s", "cores": 1, "kind": "port",
                             "sample": f"first {m} events, per-event Python loop as the reference's"}}


def _probe_peaks():
    """Roofline denominators measured on this device by the probe kernels of
    libsss300_probe.so (built beside the engine, loaded only here): shared
    memory and L2 load bandwidth (GB/s), FFMA2 rate (GFLOP/s), 2^x and FP64
    add rates (1e9/s); None where a probe fails."""
    import torch

    from opensss_gb300 import _build

    probe = C.CDLL(_build.PROBE_LIB)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = {}
    for key, fn in (("smem", "sss_probe_smem_rate"), ("l2", "sss_probe_l2_rate"),
                    ("ffma", "sss_probe_ffma_rate"), ("ex2", "sss_probe_ex2_rate"),
                    ("dadd", "sss_probe_dadd_rate"), ("ddiv", "sss_probe_ddiv_rate")):
        f = getattr(probe, fn)
        f.restype, f.argtypes = C.c_int, [C.POINTER(C.c_double), C.c_void_p]
        v = C.c_double(0.0)
        out[key] = v.value if f(C.byref(v), st) == 0 and v.value > 0 else None
    return out


# ---------------------------------------------------------------- profiler cases
#
#     python bench.py --profile CASE [--reps N]
#
# Small, self-contained cases of each GPU kernel for profiler captures.  Each
# builds seeded inputs larger than the 129 MB L2 but a few GB at most on the
# device and runs the kernel --reps times (checking the status word), so that
# a capture of one to three launches ends within a minute or two.


def _profile_engine(pr):
    from opensss_gb300.engine import TofSSS

    return TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, _att_table(),
                  pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                  pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins)


def case_upsample(reps):
    """13 bins of a 16 x 48 sampled sinogram onto a 380-crystal x 40-ring
    scanner: 381 x 190 x 1600 outputs (463 MB)."""
    import torch  # noqa: F401

    from opensss_gb300 import geometry as G, workloads as W  # noqa: F401
    from opensss_gb300.Interpolation import upsample_device

    nd, nr, nru, ndu, nb = 380, 40, 16, 48, 13
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    t = G.upsample_tables(lor, si, nru, ndu, "legpair")
    nl = nru * ndu
    sampled = torch.rand((nb, nl, nl), device="cuda")
    out = torch.empty(((nd + 1) * (nd // 2), nr * nr), device="cuda")
    for _ in range(reps):
        upsample_device(sampled, t, nb, (nd + 1) * (nd // 2), nr * nr, out=out)
    torch.cuda.synchronize()


def case_mask(reps):
    """Tail mask of the 64x64x48 phantom on a 380 x 40 scanner, AF 4."""
    import torch  # noqa: F401

    from opensss_gb300 import geometry as G, workloads as W  # noqa: F401
    from opensss_gb300.TailsMask import tail_mask_device

    pr = W.tof13_64x64x48()
    sc = W.ring_scanner(380, 40, radius_cm=41.0, ring_pitch_cm=0.64)
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, 380, 40, ID_Shidt=False)
    for _ in range(reps):
        tail_mask_device(pr.attenuation, pr.image_size, sc.geometry, lor, si, 4)


def case_fit(reps, nbins=4, rings=40):
    """Back-projection fit of ``nbins`` TOF bins of seeded sinograms in one
    pass on a 380 x ``rings`` scanner, AF 4."""
    import torch  # noqa: F401

    from opensss_gb300 import geometry as G, workloads as W  # noqa: F401
    from opensss_gb300.BackProjection import fit_bins_device

    pr = W.tof13_64x64x48()
    sc = W.ring_scanner(380, rings, radius_cm=41.0, ring_pitch_cm=0.64)
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, 380, rings, ID_Shidt=False)
    shp = (381 * 190, rings * rings)
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    prm = torch.poisson(torch.full((nbins,) + shp, 3.0, device="cuda"), generator=g)
    rnd = torch.full(shp, 0.3, device="cuda")
    scat = torch.rand((nbins,) + shp, device="cuda", generator=g)
    mask = (torch.rand(shp, device="cuda", generator=g) < 0.3).to(torch.uint8)
    cell = np.arange(shp[0], dtype=np.int64) * shp[1]
    ring = np.arange(shp[1], dtype=np.int64)
    zr = float(sc.geometry[-1, 0, 2]) + 0.3
    bounds = np.array([pr.image_size[0], pr.image_size[1], -zr, pr.image_size[3], pr.image_size[4], zr])
    for _ in range(reps):
        fit_bins_device(prm, rnd, mask, scat, shp[0] * shp[1], cell, ring, np.array([40, 40, 26]), bounds,
                        sc.geometry, lor, si[:rings, :rings].T, 4)


def case_fit13(reps):
    """The same fit over 13 TOF bins (the 13-bin workload's bin count) on a
    380 x 16 scanner: 1.9 GB of seeded sinograms."""
    case_fit(reps, nbins=13, rings=16)


def case_listmode(reps):
    """10M list-mode events into the demo's reduced sinogram (mash 2, span 19)."""
    import torch  # noqa: F401

    from opensss_gb300 import DataReduction as D, geometry as G, workloads as W  # noqa: F401
    from opensss_gb300.Datafile import histogram_device

    header = W.listmode_header("p_df", 10_000_000)
    ev = torch.from_numpy(W.synthetic_events(header, 760, 80, seed=1).view(np.uint8).reshape(-1)).cuda()
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, 380, 80, ID_Shidt=False)
    _, _, lut, _ = D.SinogramLUT(80, 19, 79)
    for _ in range(reps):
        histogram_device(ev, header, lor, lut, 6, 1000.0, mash=2)


def case_pair(reps):
    """The 64x64x48, 16 x 48, 13-bin instance on its first 400 scatter points."""
    import torch  # noqa: F401

    from opensss_gb300 import geometry as G, workloads as W  # noqa: F401
    pr = W.tof13_64x64x48()
    e = _profile_engine(pr)
    for _ in range(reps):
        e.run(pr.activity, pr.attenuation, pr.image_size, max_points=400)


def case_batch(reps):
    """Eight instances of the uneven-batch generator as one plan."""
    import torch  # noqa: F401

    from opensss_gb300 import geometry as G, workloads as W  # noqa: F401
    from opensss_gb300.batch import BatchSSS

    inst = W.uneven_instances(8, seed=3)
    b = BatchSSS([(_profile_engine(pr), pr.activity, pr.attenuation, pr.image_size) for pr in inst],
                 workspace_bytes=4 << 30)
    for _ in range(reps):
        b.run()


def case_prep(reps):
    """CropAndDownscale of a seeded 400x400x280 float32 map (1.6 x 1.6 x 2 mm)
    cropped to 600 x 600 x 480 mm and resized to 75 x 75 x 48."""
    import torch  # noqa: F401

    from opensss_gb300 import geometry as G, workloads as W  # noqa: F401
    from opensss_gb300.Utils import crop_downscale_device, crop_window

    rng = np.random.default_rng(3)
    img = torch.from_numpy(rng.gamma(2.0, 1.0, size=(400, 400, 280)).astype(np.float32)).cuda()
    win = crop_window(tuple(img.shape), (1.6, 1.6, 2.0), (600.0, 600.0, 480.0))
    for _ in range(reps):
        crop_downscale_device(img, win, (75, 75, 48))
    torch.cuda.synchronize()


PROFILE_CASES = {"upsample": case_upsample, "mask": case_mask, "fit": case_fit, "fit13": case_fit13,
                 "listmode": case_listmode, "pair": case_pair, "batch": case_batch, "prep": case_prep}




def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-points", type=int, default=1024,
                    help="scatter points in the bounded CPU sample")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-pipeline", action="store_true", help="skip upsampling / mask / fit timings")
    ap.add_argument("--af", type=int, default=6, help="AccelerationFactor of the mask and fit")
    ap.add_argument("--no-batch", action="store_true", help="skip the uneven-batch measurement")
    ap.add_argument("--batch-size", type=int, default=64, help="instances in the uneven batch")
    ap.add_argument("--batch-steps", type=int, default=3, help="timed replays of the batch (at most --steps)")
    ap.add_argument("--no-precision", action="store_true", help="skip the 33-bin precision study")
    ap.add_argument("--precision-every", type=int, default=16,
                    help="one scatter point in this many (evenly spread) enters the FP64 GPU oracle's check "
                         "of the 33-bin instance (1: all points)")
    ap.add_argument("--precision-steps", type=int, default=1)
    ap.add_argument("--precision-warmup", type=int, default=1)
    ap.add_argument("--no-serving", action="store_true", help="skip the served request stream")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="mean arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=1.0, help="length of the arrival window")
    ap.add_argument("--serve-check", type=int, default=16,
                    help="served small requests checked against the FP64 oracle")
    ap.add_argument("--sweep-rates", default="8,16,24,32,40,48,64",
                    help="offered rates (req/s) of the serving latency sweep")
    ap.add_argument("--sweep-seconds", type=float, default=3.0, help="arrival window of each sweep point")
    ap.add_argument("--p99-bound-ms", type=float, default=1000.0,
                    help="p99 latency bound of the sustained-rate figure")
    ap.add_argument("--no-listmode", action="store_true", help="skip the list-mode histogramming")
    ap.add_argument("--no-prep", action="store_true", help="skip the image preparation (CropAndDownscale)")
    ap.add_argument("--no-autotune", action="store_true", help="run with the library's default launch shapes")
    ap.add_argument("--listmode-events", type=int, default=50_000_000)
    ap.add_argument("--listmode-cpu-events", type=int, default=200_000)
    ap.add_argument("--max-points", type=int, default=None,
                    help="limit each step to the first scatter points (profiling runs only)")
    ap.add_argument("--profile", choices=sorted(PROFILE_CASES), default=None,
                    help="run one small kernel case for a profiler capture instead of the benchmark")
    ap.add_argument("--reps", type=int, default=2, help="launches of the --profile case")
    args = ap.parse_args()
    if args.profile:
        PROFILE_CASES[args.profile](args.reps)
        print(f"{args.profile}: ok")
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
