"""Generate the golden fixtures in this folder from the reference itself.

Runs the unmodified openSSS v1.0 Python modules (interpreted, through the
pass-through numba stub in ``oracle/numba_stub``) and the reference's MEX ray
tracers compiled from source (``oracle/_ref``), on seeded synthetic inputs,
and stores inputs + outputs as compressed ``.npz`` fixtures.  It needs the
reference checkout, named by ``OPENSSS_REFERENCE`` (its ``Python`` folder),
and is run by hand where that checkout exists:

    OPENSSS_REFERENCE=<checkout>/Python python tests/golden/make_golden.py [--only name,...]

The fixtures are then used by the CPU tests (oracle pinning) and the GPU
parity tests, which never need the reference checkout.
"""

from __future__ import annotations

import argparse
import hashlib
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle import refpy  # noqa: E402
from opensss_gb300 import workloads as W  # noqa: E402

ATT_TABLE = os.path.join(refpy.REFERENCE_PY, "openSSS", "AttenuationTable_AttenuationTable.npy")


def _save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


def _sino(R, nd, nr):
    return R["Sinogram"].SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)


# ---------------------------------------------------------------- rays


def ray_cases(seed=7):
    """Seeded rays on several grids, with the edge cases the tracer has:
    axis-parallel rays, rays along voxel planes and through voxel corners,
    rays starting or ending inside the grid, misses and rays that only touch
    a face."""
    rng = np.random.default_rng(seed)
    cases = []
    grids = [
        (np.array([12, 12, 6]), np.array([-12.0, -12.0, -6.0, 12.0, 12.0, 6.0])),
        (np.array([40, 40, 20]), np.array([-20.0, -20.0, -10.0, 20.0, 20.0, 10.0])),
        (np.array([16, 16, 16]), np.array([-3.2, -3.2, -3.2, 3.2, 3.2, 3.2])),
        (np.array([10, 14, 7]), np.array([-5.0, -7.0, -3.5, 5.0, 7.0, 3.5])),  # Nx != Ny
    ]
    for grid, gb in grids:
        ext = gb[3:] - gb[:3]
        n = 600
        a = rng.uniform(gb[:3] - 0.8 * ext, gb[3:] + 0.8 * ext, size=(n, 3))
        b = rng.uniform(gb[:3] - 0.8 * ext, gb[3:] + 0.8 * ext, size=(n, 3))
        lines = np.concatenate([a, b], axis=1)
        # axis-parallel in one or two coordinates
        lines[0:40, 3] = lines[0:40, 0]
        lines[40:80, 4] = lines[40:80, 1]
        lines[80:120, 5] = lines[80:120, 2]
        lines[120:150, 3:5] = lines[120:150, 0:2]
        # endpoints inside the grid
        lines[150:200, 0:3] = rng.uniform(gb[:3], gb[3:], size=(50, 3))
        lines[200:230, 3:6] = rng.uniform(gb[:3], gb[3:], size=(30, 3))
        # points on the voxel lattice (corner and plane crossings, ties)
        vox = ext / grid
        k = rng.integers(-2, grid.max() + 3, size=(120, 6))
        lat = np.concatenate([gb[:3] + k[:, :3] * vox, gb[:3] + k[:, 3:] * vox], axis=1)
        lines[230:350] = lat
        # exact diagonals through corners
        lines[350:360, 0:3] = gb[:3] - vox
        lines[350:360, 3:6] = gb[3:] + vox * rng.integers(0, 3, size=(10, 1))
        # lines along a face plane (touching only)
        lines[360:380, 0] = gb[0]
        lines[360:380, 3] = gb[0]
        # zero-length segments (appended; no draw from rng): inside a voxel, on
        # a voxel corner, on each corner of the grid, on a face, outside
        pts = np.array([(gb[:3] + gb[3:]) / 2 + 0.3 * vox, gb[:3] + 2 * vox, gb[:3], gb[3:],
                        np.array([gb[0], (gb[1] + gb[4]) / 2, (gb[2] + gb[5]) / 2]), gb[3:] + vox])
        lines = np.concatenate([lines, np.concatenate([pts, pts], axis=1)])
        cases.append((grid, gb, lines))
    return cases


def gen_rays(R):
    RT = R["RayTracing3DTOF"].RayTracing3DTOF
    tof = O.RefTracer(True)
    non = O.RefTracer(False)
    out = {}
    for ci, (grid, gb, lines) in enumerate(ray_cases()):
        cap = int(grid.sum())
        n = lines.shape[0]
        cnt = np.zeros(n, np.int32)
        ln = np.zeros((n, cap))
        ix = np.zeros((n, cap), np.int32)
        sm = np.zeros((n, cap))
        cnt3 = np.zeros(n, np.int32)
        ln3 = np.zeros((n, cap), np.float32)
        ix3 = np.zeros((n, cap), np.int32)
        mex_mismatch = 0
        raised = 0
        for i in range(n):
            try:
                a, b, c = RT(grid, gb, lines[i])
            except IndexError:
                # the traversal overran its Nx+Ny+Nz storage: the reference
                # raises here (and the MEX build would keep stepping)
                cnt[i] = -1
                cnt3[i] = -1
                raised += 1
                continue
            k = len(a)
            cnt[i] = k
            ln[i, :k], ix[i, :k], sm[i, :k] = a, b, c
            ma, mb, mc = tof(grid, gb, lines[i])
            if len(ma) != k or not np.array_equal(mb, b):
                mex_mismatch += 1
            na, nb_, _ = non(grid, gb, lines[i])
            cnt3[i] = len(na)
            ln3[i, :len(na)] = na
            ix3[i, :len(na)] = nb_
        print(f"rays case {ci}: {n} rays, {int((cnt > 0).sum())} hits, {raised} overruns, "
              f"MEX/Python index mismatches {mex_mismatch}")
        out[f"grid{ci}"] = grid
        out[f"bounds{ci}"] = gb
        out[f"lines{ci}"] = lines
        out[f"count{ci}"] = cnt
        out[f"len{ci}"] = ln
        out[f"idx{ci}"] = ix
        out[f"samples{ci}"] = sm
        out[f"count_nontof{ci}"] = cnt3
        out[f"len_nontof{ci}"] = ln3
        out[f"idx_nontof{ci}"] = ix3
    out["ncases"] = np.array(len(ray_cases()))
    _save("rays", **out)


# ---------------------------------------------------------------- SSS


def _run_sss(R, pr, LC):
    AT = np.load(ATT_TABLE)
    with tempfile.TemporaryDirectory() as d:
        t0 = time.time()
        dense = R["SingleScatterSimulationTOF"].SingleScatterSimulationTOF(
            pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry, LC,
            pr.scanner.normals, pr.scanner.detector_size_mm, AT, pr.energy_resolution,
            pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step,
            pr.tof_resolution, pr.tof_range, pr.nr_bins, d)
        dt = time.time() - t0
    return dense, dt


def _compact_from_dense(dense, LC, nd, nru, ndu):
    det = W.sampled_detectors(nd, ndu)
    a, b = np.triu_indices(ndu)
    ang = LC[det[a], det[b], 0].astype(np.int64)
    rad = LC[det[a], det[b], 1].astype(np.int64)
    cmp = np.zeros((dense.shape[0], nru * nru, ndu, ndu), np.float32)
    for s in range(nru * nru):
        cmp[:, s, a, b] = dense[:, rad, ang, s]
    # everything else in the dense output must be zero
    check = dense.copy()
    for s in range(nru * nru):
        check[:, rad, ang, s] = 0
    assert not check.any(), "reference wrote outside the sampled detector pairs"
    return cmp


def _problem_arrays(pr):
    return dict(activity=pr.activity, attenuation=pr.attenuation, image_size=pr.image_size,
                geometry=pr.scanner.geometry, normals=pr.scanner.normals,
                detector_size=pr.scanner.detector_size_mm,
                params=np.array([pr.nr_rings_used, pr.nr_detectors_used, pr.nr_bins,
                                 *pr.sample_step]),
                fparams=np.array([pr.energy_resolution, pr.energy_threshold, pr.tof_resolution,
                                  pr.tof_range]))


def gen_sss(R, which):
    problems = []
    if "tiny" in which:
        problems += [("sss_tiny_b1", W.tiny_problem(1, seed=3)),
                     ("sss_tiny_b3", W.tiny_problem(3, seed=4)),
                     ("sss_tiny_b5", W.tiny_problem(5, seed=5, shape=(14, 14, 8), nd=64, nr=8,
                                                    nru=4, ndu=10, voxel_cm=1.7))]
    if "nontof_40x40x20" in which:
        problems.append(("sss_nontof_40x40x20", W.nontof_40x40x20(seed=0)))
    if "nxgt" in which:
        # Nx > Ny: the reference's sub2ind strides x by Ny, so it reads shifted
        # voxels without leaving the volume, and its scatter-point grid spaces y
        # with the x extent (:377-394)
        # (the ring is turned by half a crystal so that no leg runs exactly
        # through voxel corners, where the reference's traversal overruns)
        problems.append(("sss_tiny_nx14_ny10",
                         W.make_problem("tiny-nx14-ny10", (14, 10, 6), 2.0, 3, 8, 3, 3.0, 214.0, seed=6,
                                        scanner=W.ring_scanner(48, 6, radius_cm=20.0, ring_pitch_cm=1.0,
                                                               phase=0.5), radius_cm=8.0)))
    if "bins" in which:
        # bins wider than 1.33 x the timing FWHM: the pair kernel evaluates
        # every bin's weight with its own 2^x instead of the factored product
        problems.append(("sss_tiny_wide",
                         W.make_problem("tiny-wide", (12, 12, 6), 2.0, 3, 8, 3, 5.0, 214.0, seed=10,
                                        scanner=W.ring_scanner(48, 6, radius_cm=20.0, ring_pitch_cm=1.0),
                                        radius_cm=8.0)))
        # a 60 ps timing kernel with 5 bins of 1 cm: TOF offsets run up to
        # ~575 ps, far past the last bin centre (133 ps), where the normalised
        # column's weight sits almost entirely on the last bin
        problems.append(("sss_tiny_far",
                         W.make_problem("tiny-far", (12, 12, 6), 2.0, 3, 8, 5, 1.0, 60.0, seed=8,
                                        scanner=W.ring_scanner(48, 6, radius_cm=20.0, ring_pitch_cm=1.0,
                                                               phase=0.5), radius_cm=8.0)))
    if "widebody" in which:
        # a 50 cm wide body (radius 25 cm, 17 x 17 x 4 voxels of 3.1 cm) in the
        # 41 cm ring at the benchmark's 13 bins of 3.9 cm and 214 ps: offsets
        # reach ~1770 ps, past the last bin centre (1561 ps) by more than the
        # factored weights take, but stay inside the +-4000 ps table (an odd
        # grid keeps scatter points off the centre, where opposite crystals
        # would make the reference's acos argument leave [-1, 1])
        problems.append(("sss_wide_body_tof13",
                         W.make_problem("wide-body-tof13", (17, 17, 4), 3.1, 2, 12, 13, 3.9, 214.0, seed=21,
                                        scanner=W.ring_scanner(48, 4, radius_cm=41.0, ring_pitch_cm=1.0,
                                                               phase=0.5), radius_cm=25.0)))
    if "evenaniso" in which:
        # an even bin count (no bin centred on offset 0), an odd sampled
        # crystal count, a sampling step that differs per axis and more
        # slices than columns (Nz > Nx = Ny)
        problems.append(("sss_tiny_even_aniso",
                         W.make_problem("tiny-even-aniso", (10, 10, 14), 1.6, 3, 7, 4, 2.5, 214.0, seed=23,
                                        scanner=W.ring_scanner(48, 8, radius_cm=20.0, ring_pitch_cm=1.0,
                                                               phase=0.5),
                                        radius_cm=7.0, sample_step=(1, 2, 3))))
    if "edge" in which:
        # degenerate inputs: no scatter point (empty attenuation map, or a
        # sampling step past the volume), no activity, one sampled ring, and
        # one sampled crystal per ring (only same-crystal pairs, all backscatter,
        # whose FP64 energy efficiency is exactly 0)
        pr = W.tiny_problem(3, seed=11)
        pr.attenuation = np.zeros_like(pr.attenuation)
        problems.append(("sss_edge_empty_mu", pr))
        pr = W.tiny_problem(3, seed=12)
        pr.activity = np.zeros_like(pr.activity)
        problems.append(("sss_edge_empty_act", pr))
        problems.append(("sss_edge_one_ring", W.tiny_problem(3, seed=13, nru=1, ndu=8)))
        problems.append(("sss_edge_one_crystal", W.tiny_problem(3, seed=14, nru=3, ndu=1)))
        pr = W.tiny_problem(3, seed=15)
        pr.sample_step = np.array([13, 13, 7])
        problems.append(("sss_edge_step_past_volume", pr))
    if "tofrange" in which:
        # a 2 m wide body in a scanner of 1.5 m radius: TOF offsets of pairs
        # pass the 8001-entry table (+-4000 ps, 120 cm), where the reference
        # indexes past the table and raises IndexError (:521, :527)
        pr = W.make_problem("tiny-tofrange", (80, 80, 6), 2.5, 3, 8, 3, 3.0, 214.0, seed=7,
                            scanner=W.ring_scanner(48, 6, radius_cm=150.0, ring_pitch_cm=1.0, phase=0.5),
                            radius_cm=99.0)
        nd, nr = pr.scanner.nr_detectors, pr.scanner.nr_rings
        LC, _, _ = _sino(R, nd, nr)
        try:
            _run_sss(R, pr, LC)
            err = ""
        except IndexError as e:
            err = f"IndexError: {e}"
        print(f"sss_tofrange: reference {err or 'ran'}")
        _save("sss_tofrange", **_problem_arrays(pr), reference_error=np.array(err))
    for name, pr in problems:
        nd, nr = pr.scanner.nr_detectors, pr.scanner.nr_rings
        LC, SI, _ = _sino(R, nd, nr)
        dense, dt = _run_sss(R, pr, LC)
        cmp = _compact_from_dense(dense, LC, nd, pr.nr_rings_used, pr.nr_detectors_used)
        print(f"{name}: reference SSS {dt:.1f} s, {int((cmp != 0).sum())} non-zero cells")
        _save(name, **_problem_arrays(pr), compact=cmp, ref_seconds=np.array(dt),
              ref_cores=np.array(os.cpu_count()))


class _OneSlice:
    """Stand-in for joblib.Parallel inside the reference's driver: runs the
    delayed bodySSS call of one z-slice only (argument 0 is zIndex) and
    returns its dense slice term, so that one slice of a full-size problem
    fits in host memory (each term is a dense [B, ND+1, ND/2, NRU^2] array)."""

    def __init__(self, z):
        self.z = z

    def __call__(self, *args, **kwargs):
        def run(calls):
            out = [f(*a, **kw) for f, a, kw in calls if a[0] == self.z]
            assert len(out) == 1, "the chosen z-slice is not on the sampling lattice"
            return out
        return run


def gen_sss_slice(R, z=24, ncells=50000, seed=17):
    """One sampled z-slice (zIndex 24 of the 48) of the 13-bin, 64x64x48 @ 6 mm
    workload on the 760 x 80 scanner, 16 x 48 sampled: the reference's own
    driver with its parallel loop restricted to that slice.  The fixture keeps
    a seeded subset of the compact cells and every bin's total."""
    S = R["SingleScatterSimulationTOF"]
    pr = W.tof13_64x64x48(seed=0)
    nd, nr = pr.scanner.nr_detectors, pr.scanner.nr_rings
    LC, _, _ = _sino(R, nd, nr)
    saved = S.Parallel
    S.Parallel = _OneSlice(z)
    try:
        dense, dt = _run_sss(R, pr, LC)
    finally:
        S.Parallel = saved
    cmp = _compact_from_dense(dense, LC, nd, pr.nr_rings_used, pr.nr_detectors_used)
    del dense
    flat = cmp.reshape(cmp.shape[0], -1)
    rng = np.random.default_rng(seed)
    nz = np.flatnonzero(flat.any(axis=0))
    cells = np.sort(rng.choice(nz, size=min(ncells, len(nz)), replace=False))
    print(f"sss_tof13_slice: zIndex {z}, reference {dt:.0f} s, {len(nz)} contributing cells, kept {len(cells)}")
    _save("sss_tof13_slice", z_index=np.array(z), lattice_slice=np.array(z // int(pr.sample_step[2])),
          cells=cells.astype(np.int64), values=flat[:, cells], bin_totals=flat.astype(np.float64).sum(axis=1),
          contributing=np.array(len(nz)), shape=np.array(cmp.shape), ref_seconds=np.array(dt))


# ---------------------------------------------------------------- tables / LUTs


def gen_tables(R):
    S = R["SingleScatterSimulationTOF"]
    AT = np.load(ATT_TABLE)
    out = {}
    for tag, nb, rng_ps, res in (("b1", 1, 1000.0, 1.0e6), ("b13", 13, None, 214.0),
                                 ("b33", 33, None, 214.0), ("b6", 6, 1000.0, 214.0)):
        if rng_ps is None:
            rng_ps, _ = W.tof_bins(nb, 3.9 if nb == 13 else 1.5)
        bw = 2 * rng_ps / nb
        import warnings

        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            T = S.TOFEfficiencyTable(np.arange(-4000, 4001), bw, nb, res)
        out[f"tof_{tag}"] = T[:, ::3]  # every 3rd offset keeps the fixture small
        out[f"tof_{tag}_params"] = np.array([nb, rng_ps, res])
    from scipy.special import erf

    eff = 0.5 * (1 - erf((435.0 - AT[:, 0]) / (511 * 0.12 / 2 / np.sqrt(np.log(2)))))
    out["eff_435_012"] = eff
    out["att_table"] = AT
    _save("tables", **out)

    lc48, si6, _ = _sino(R, 48, 6)
    lc64, si10, _ = _sino(R, 64, 10)
    lc760, si80, _ = _sino(R, 760, 80)
    digest = hashlib.sha256(np.ascontiguousarray(lc760).tobytes()).hexdigest()
    _save("sinogram", lor48=lc48, sino6=si6, lor64=lc64, sino10=si10, sino80=si80,
          lor760_sha256=np.array(digest), lor760_row0=lc760[0], lor760_row379=lc760[379],
          lor760_diag=np.stack([lc760[i, i] for i in range(760)]))


def gen_upsample_luts(R):
    """For the 760-crystal scanner, the nearest-neighbour source cell that the
    reference's radial/angular fill picks for every full-sinogram bin, found
    by running Interpolation.interpolate_radial_angular on a sinogram whose
    cells hold their own (rad, ang) code."""
    I = R["Interpolation"]
    lc760, _, _ = _sino(R, 760, 80)
    out = {}
    code = (np.arange(761)[:, None] * 1000 + np.arange(380)[None, :]).astype(np.float32)
    gx, gy = np.mgrid[0:761, 0:380]
    for ndu in (32, 48, 96):
        det = np.tile(W.sampled_detectors(760, ndu), (80, 1))
        F = I.interpolate_radial_angular(code, 0, 0, lc760, det, gx, gy)
        out[f"src_ndu{ndu}"] = F.astype(np.int32)
        print(f"upsample LUT ndu={ndu}: {len(np.unique(F))} distinct sources")
    _save("upsample_lut760", **out)


def gen_upsample(R):
    """Full InterpolateAllBins on a small geometry (NR must be a multiple of 5)."""
    I = R["Interpolation"]
    rng = np.random.default_rng(11)
    cases = {}
    for ci, (nd, nr, nru, ndu, nb) in enumerate(((48, 10, 3, 8, 2), (64, 10, 4, 12, 1))):
        lc, si, _ = _sino(R, nd, nr)
        det = W.sampled_detectors(nd, ndu)
        rings = W.sampled_rings(nr, nru)
        # a sampled sinogram as the SSS writes it: values on the sampled pairs only
        cmp = np.zeros((nb, nru * nru, ndu, ndu), np.float32)
        a, b = np.triu_indices(ndu)
        for s in range(nru * nru):
            r1, r2 = divmod(s, nru)
            v = rng.uniform(0.5, 2.0, size=(nb, len(a))).astype(np.float32)
            same = (a == b) & (r1 == r2)
            v[:, same] = 0
            cmp[:, s, a, b] = v
        dense = O.densify(cmp.astype(np.float64), lc, nd, nru, ndu)
        with tempfile.TemporaryDirectory() as d:
            Ib = I.InterpolateScatters(dense, nr, nru, nd, ndu, lc, si, d, False)
            per_bin = [np.load(os.path.join(d, f"SSS_mashed_bin{k}.npz"))["arr_0"] for k in range(nb)]
        cases[f"case{ci}_dims"] = np.array([nd, nr, nru, ndu, nb])
        cases[f"case{ci}_compact"] = cmp
        cases[f"case{ci}_sum"] = Ib
        cases[f"case{ci}_bins"] = np.stack(per_bin)
        cases[f"case{ci}_rings"] = rings
        print(f"upsample case {ci}: out {Ib.shape}")
    _save("upsample", **cases)


# ---------------------------------------------------------------- mask / fit


def _small_scan(nd, nr, radius=20.3, pitch=1.1):
    # 20 cm / 1 cm would put 45-degree LORs exactly through voxel corners,
    # where the reference tracer overruns its storage and raises
    return W.ring_scanner(nd, nr, radius_cm=radius, ring_pitch_cm=pitch)


def gen_mask(R):
    T = R["TailsMask"]
    out = {}
    for ci, (nd, nr, shape, vox, af) in enumerate(((48, 6, (12, 12, 6), 2.0, 1),
                                                    (64, 8, (16, 16, 8), 1.5, 3),
                                                    (48, 6, (12, 12, 6), 2.0, 5),
                                                    (48, 6, (12, 12, 6), 2.0, 2))):
        sc = _small_scan(nd, nr)
        act, mu, bounds = W.cylinder_phantom(shape, vox, seed=ci, radius_cm=6.0)
        if ci == 3:  # empty attenuation map: every LOR of the lattice is a tail
            mu = np.zeros_like(mu)
        lc, si, _ = _sino(R, nd, nr)
        m = T.MaskGenerator(act, mu, bounds, sc.geometry, lc, si, True, af)
        out[f"case{ci}_dims"] = np.array([nd, nr, af])
        out[f"case{ci}_mu"] = mu
        out[f"case{ci}_bounds"] = bounds
        out[f"case{ci}_geometry"] = sc.geometry
        out[f"case{ci}_mask"] = m
        print(f"mask case {ci}: {int(m.sum())} masked bins of {m.size}")
    _save("mask", **out)


def gen_fit(R):
    B = R["BackProjection"]
    T = R["TailsMask"]
    rng = np.random.default_rng(5)
    out = {}
    for ci, (nd, nr, shape, vox, fgrid, af) in enumerate(((48, 6, (12, 12, 6), 2.0, (10, 10, 6), 1),
                                                           (64, 10, (16, 16, 8), 1.5, (12, 12, 10), 2))):
        sc = _small_scan(nd, nr)
        act, mu, bounds = W.cylinder_phantom(shape, vox, seed=ci, radius_cm=6.0)
        lc, si, _ = _sino(R, nd, nr)
        m = T.MaskGenerator(act, mu, bounds, sc.geometry, lc, si, True, af)
        maskf = np.float32(m >= 1)
        shp = (nd + 1, nd // 2, nr * nr)
        scat = rng.uniform(0.2, 1.0, size=shp).astype(np.float32)
        scat[rng.uniform(size=shp) < 0.1] = 0
        rnd = np.full(shp, 0.1, np.float32)
        prm = (rng.poisson(3.0, size=shp) / 1.0).astype(np.float32)
        fit_bounds = np.array([bounds[0], bounds[1], sc.geometry[0, 0, 2] - 0.5,
                               bounds[3], bounds[4], sc.geometry[-1, 0, 2] + 0.5])
        order = si[:nr, :nr].T
        scale = B.BackProjectionScatterRandFit(prm, scat, rnd, maskf, np.array(fgrid), fit_bounds,
                                               sc.geometry, lc, order, af)
        out[f"case{ci}_dims"] = np.array([nd, nr, af])
        out[f"case{ci}_grid"] = np.array(fgrid)
        out[f"case{ci}_bounds"] = fit_bounds
        out[f"case{ci}_geometry"] = sc.geometry
        out[f"case{ci}_mask"] = maskf
        out[f"case{ci}_scatter"] = scat
        out[f"case{ci}_randoms"] = rnd
        out[f"case{ci}_prompts"] = prm
        out[f"case{ci}_scale"] = np.asarray(scale, np.float32)
        print(f"fit case {ci}: scale {scale}")
        if ci == 0:
            # degenerate inputs on case 0: no masked LOR, no scatter, and prompts
            # below the randoms everywhere (T = 0): the reference's lstsq gives 0
            zero = {"mask": (prm, scat, np.zeros_like(maskf)), "scatter": (prm, np.zeros_like(scat), maskf),
                    "trues": (np.zeros_like(prm), scat, maskf)}
            for name, (p_, s_, m_) in zero.items():
                sc0 = B.BackProjectionScatterRandFit(p_, s_, rnd, m_, np.array(fgrid), fit_bounds, sc.geometry, lc,
                                                     order, af)
                out[f"edge_no_{name}_scale"] = np.asarray(sc0, np.float32)
                print(f"fit case 0 without {name}: scale {sc0}")
    _save("fit", **out)


# ---------------------------------------------------------------- span / mash


def _mashed(R, nr, span, mrd):
    si, ring_lut, lut, counts = R["DataReduction"].SinogramLUT(nr, span, mrd)
    return si, ring_lut, lut, counts


def gen_span(R):
    """The span (axial mashing) / mash (angular) path on small geometries:
    SinogramLUT, expandRings, mashDetectors, SumLORsCounts,
    InterpolateAllBinsSpan (through InterpolateScatters), MaskGeneratorMashing
    and BackProjectionScatterRandFitMashing."""
    D, G, I, T, B = (R[k] for k in ("DataReduction", "Geometry", "Interpolation", "TailsMask",
                                    "BackProjection"))
    out = {}
    # look-up tables, including the demo's 80 rings / span 19 / MRD 79
    for ci, (nr, span, mrd) in enumerate(((10, 3, 9), (12, 5, None), (9, 3, 4), (80, 19, 79))):
        si, ring_lut, lut, counts = _mashed(R, nr, span, mrd)
        out[f"lut{ci}_args"] = np.array([nr, span, -1 if mrd is None else mrd])
        out[f"lut{ci}_index"] = si
        out[f"lut{ci}_ringlut"] = ring_lut
        out[f"lut{ci}_table"] = lut
        out[f"lut{ci}_counts"] = counts
        print(f"span lut {ci}: {si.shape[0]} mashed sinograms")
    # geometry helpers
    sc = _small_scan(48, 6)
    eg, en = G.expandRings(sc.geometry, sc.normals)
    mg, mn = G.mashDetectors(sc.geometry, sc.normals, 2)
    out["geom_in"] = sc.geometry
    out["normals_in"] = sc.normals
    out["geom_expanded"] = eg
    out["normals_expanded"] = en
    out["geom_mashed2"] = mg
    out["normals_mashed2"] = mn
    si, _, lut, counts = _mashed(R, 6, 3, 5)
    out["lorcounts"] = D.SumLORsCounts(sc.geometry, lut, si, 2, 3, counts.shape[0])
    # upsampling with span
    rng = np.random.default_rng(21)
    nd, nr, nru, ndu, nb = 48, 10, 3, 8, 2
    lc, _, _ = _sino(R, nd, nr)
    msi, _, _, _ = _mashed(R, nr, 3, 9)
    cmp = np.zeros((nb, nru * nru, ndu, ndu), np.float32)
    a, b = np.triu_indices(ndu)
    for s in range(nru * nru):
        r1, r2 = divmod(s, nru)
        v = rng.uniform(0.5, 2.0, size=(nb, len(a))).astype(np.float32)
        v[:, (a == b) & (r1 == r2)] = 0
        cmp[:, s, a, b] = v
    dense = O.densify(cmp.astype(np.float64), lc, nd, nru, ndu)
    with tempfile.TemporaryDirectory() as d:
        up = I.InterpolateScatters(dense, nr, nru, nd, ndu, lc, msi, d, True)
        per_bin = [np.load(os.path.join(d, f"SSS_mashed_bin{k}.npz"))["arr_0"] for k in range(nb)]
    out["up_dims"] = np.array([nd, nr, nru, ndu, nb, 3, 9])
    out["up_compact"] = cmp
    out["up_sum"] = up
    out["up_bins"] = np.stack(per_bin)
    print(f"span upsample: out {up.shape}")
    # tail mask and fit with span on the expanded geometry
    for ci, (nd, nr, span, shape, vox, af, fgrid) in enumerate(((48, 6, 3, (12, 12, 6), 2.0, 1, (10, 10, 6)),
                                                                 (64, 9, 3, (16, 16, 8), 1.5, 2, (12, 12, 8)))):
        sc = _small_scan(nd, nr)
        eg, _ = G.expandRings(sc.geometry, sc.normals)
        act, mu, bounds = W.cylinder_phantom(shape, vox, seed=10 + ci, radius_cm=6.0)
        lc, _, _ = _sino(R, nd, nr)
        msi, _, _, _ = _mashed(R, nr, span, nr - 1)
        m = T.MaskGeneratorMashing(act, mu, bounds, eg, lc, msi, True, af)
        ma = T.MaskGeneratorMashing(act, mu, bounds, eg, lc, msi, False, af)
        maskf = np.float32(m >= 1)
        shp = (nd + 1, nd // 2, msi.shape[0])
        scat = rng.uniform(0.2, 1.0, size=shp).astype(np.float32)
        scat[rng.uniform(size=shp) < 0.1] = 0
        rnd = np.full(shp, 0.1, np.float32)
        prm = rng.poisson(3.0, size=shp).astype(np.float32)
        fit_bounds = np.array([bounds[0], bounds[1], sc.geometry[0, 0, 2] - 0.5,
                               bounds[3], bounds[4], sc.geometry[-1, 0, 2] + 0.5])
        scale = B.BackProjectionScatterRandFitMashing(prm, scat, rnd, maskf, np.array(fgrid), fit_bounds, eg, lc,
                                                      af, msi)
        out[f"case{ci}_dims"] = np.array([nd, nr, span, af])
        out[f"case{ci}_act"] = act
        out[f"case{ci}_mu"] = mu
        out[f"case{ci}_bounds"] = bounds
        out[f"case{ci}_geometry"] = sc.geometry
        out[f"case{ci}_mask"] = m
        out[f"case{ci}_mask_activity"] = ma
        out[f"case{ci}_grid"] = np.array(fgrid)
        out[f"case{ci}_fit_bounds"] = fit_bounds
        out[f"case{ci}_scatter"] = scat
        out[f"case{ci}_randoms"] = rnd
        out[f"case{ci}_prompts"] = prm
        out[f"case{ci}_scale"] = np.asarray(scale, np.float32)
        print(f"span case {ci}: {int(m.sum())} masked bins, scale {scale}")
    _save("span", **out)


# ---------------------------------------------------------------- list-mode


def gen_listmode(R):
    """ExportPrompts and InjectScatters (the reference's Timber package) on
    seeded synthetic list-mode files: plain, with mash 2 and a crystal
    shift, with span (LookUpTable slices), and an empty file."""
    sys.path.insert(0, refpy.REFERENCE_PY)
    from Timber import Datafile as TD

    out = {}
    cases = (("plain", 48, 6, 1, 0, None, 20000), ("mash_shift", 48, 6, 2, 3, None, 20000),
             ("span", 48, 10, 1, 0, (3, 9), 20000), ("empty", 48, 6, 1, 0, None, 0))
    for ci, (tag, ncr, nr, mash, shift, span, nev) in enumerate(cases):
        with tempfile.TemporaryDirectory() as d:
            hdr = W.synthetic_listmode(d, f"case{ci}_df", nev, ncr, nr, seed=30 + ci, tof_range=1000.0)
            lor, si, _ = R["Sinogram"].SinogramCoordinates(1, 1, 1, 1, ncr // mash, nr, ID_Shidt=False)
            if span:
                msi, _, lut, _ = R["DataReduction"].SinogramLUT(nr, span[0], span[1])
                table = lut
            else:
                msi, lut, table = si, np.array([]), si
            p, r, n = TD.ExportPrompts(d, hdr, lor, table, 5, 1000.0, mash=mash, Shift=shift)
            out[f"case{ci}_args"] = np.array([ncr, nr, mash, shift, -1 if not span else span[0],
                                              -1 if not span else span[1]])
            out[f"case{ci}_events"] = np.fromfile(os.path.join(d, f"case{ci}_df.Cdf"), dtype=np.uint8)
            out[f"case{ci}_prompts"] = p
            out[f"case{ci}_randoms"] = r
            out[f"case{ci}_norm"] = n
            # injection of a seeded scatter estimate
            rng = np.random.default_rng(40 + ci)
            nsl = msi.shape[0] if span else int(np.max(si)) + 1
            shp = (int(lor[:, :, 1].max()) + 1, int(lor[:, :, 0].max()) + 1, nsl)
            scale = rng.uniform(0.5, 2.0, size=5).astype(np.float32)
            np.save(os.path.join(d, "ScaleFactors.npy"), scale)
            sc = []
            for b in range(5):
                arr = rng.uniform(0.0, 1.0, size=shp).astype(np.float32)
                np.savez_compressed(os.path.join(d, f"SSS_mashed_bin{b}"), arr)
                sc.append(arr)
            TD.InjectScatters(d, hdr, lor, msi, d, lut, bool(span), 1000.0, None, mash=mash, Shift=shift)
            out[f"case{ci}_scale"] = scale
            out[f"case{ci}_scatters"] = np.stack(sc)
            new_name = hdr[:-6] + "scatter_" + hdr[-6:]
            with open(os.path.join(d, new_name)) as f:
                out[f"case{ci}_injected_header"] = np.frombuffer(f.read().encode(), dtype=np.uint8)
            dname = f"case{ci}_df.Cdf"
            out[f"case{ci}_injected"] = np.fromfile(os.path.join(d, dname[:-6] + "scatter_" + dname[-6:]),
                                                    dtype=np.uint8)
            print(f"listmode case {ci} ({tag}): {int(p.sum())} prompts, {out[f'case{ci}_injected'].size} "
                  "injected bytes")
    _save("listmode", **out)


# parameter-file lines covering every typing rule of ReadParameters (one file
# per entry of SUPPORT_BAD: lines the reference rejects)
SUPPORT_LINES = [
    "# comment line", "", "   ", "Path2Data = 'Data'", 'Name = "scan_df.Cdh"', "Plain = some text",
    "Flag = True", "Off = False", "QuotedFlag = 'True'", "Int = 42", "Neg = -7", "Float = 0.108", "Sci = 1e-3",
    "Inf = inf", "Tuple = (1, 2, 3)", "TupleF = (1.5, 2, 3)", "Tuple4 = (1, 2, 3, 4)", "TupleS = (a, b, c)",
    "TupleNoSpace = (1,2,3)", "List = [1, 2, 3]", "ListF = [0.5, 2]", "ListS = [x, y]", "ListEmpty = []",
    "Nested = ([1, 2])", "Empty =", "Quote = '", "Spaces   =   8   ", "Mixed = '(4, 5, 6)'", "Under = 1_000",
]
SUPPORT_BAD = ["Two = a = b", "NoEquals", "Short = (1, 2)"]
NORMALIZE_CASES = [
    (np.linspace(-3.0, 5.0, 24).reshape(2, 3, 4), 0, 255),
    (np.full((2, 2, 2), 7.0), 0, 255),
    (np.arange(8, dtype=np.float32).reshape(2, 2, 2), -1.0, 1.0),
    (np.arange(12).reshape(3, 2, 2), 0, 100),
]


def gen_support(R):
    S = R["Support"]
    out = {}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "params.txt")
        with open(path, "w") as f:
            f.write("\n".join(SUPPORT_LINES) + "\n")
        out["params_repr"] = np.array(repr(S.ReadParameters(path)))
        errors = []
        for line in SUPPORT_BAD:
            with open(path, "w") as f:
                f.write(line + "\n")
            try:
                S.ReadParameters(path)
                errors.append("")
            except Exception as e:  # the reference's exception type is the fixture
                errors.append(type(e).__name__)
        out["bad_errors"] = np.array(errors)
    out["lines"] = np.array(SUPPORT_LINES)
    out["bad_lines"] = np.array(SUPPORT_BAD)
    for i, (a, lo, hi) in enumerate(NORMALIZE_CASES):
        out[f"normalize{i}_in"] = a
        out[f"normalize{i}_range"] = np.array([lo, hi], dtype=np.float64)
        out[f"normalize{i}"] = S.NormalizeArray(a, lo, hi)
    print(f"support: {out['params_repr']}; errors {errors}")
    _save("support", **out)


ALL = ["rays", "tables", "sss_tiny", "sss_nontof_40x40x20", "sss_nxgt", "sss_tofrange", "sss_bins", "sss_widebody",
       "sss_evenaniso", "sss_edge",
       "sss_tof13_slice", "upsample", "upsample_lut",
       "mask", "fit", "span", "listmode", "prep", "support"]


# ---------------------------------------------------------------- image preparation

PREP_CASES = [
    # (image shape, voxel mm, crop mm, output dims): a plain crop, a window
    # overhanging both ends of one axis (zero pad), Python's negative-start
    # slice on an odd axis (a one-sample window), and an upscaled axis
    ((40, 36, 30), (2.0, 2.0, 3.0), (60.0, 50.0, 81.0), (10, 8, 9)),
    ((20, 24, 16), (4.0, 4.0, 4.0), (100.0, 80.0, 64.0), (9, 7, 16)),
    ((21, 20, 19), (1.0, 1.0, 1.0), (22.0, 10.0, 7.0), (4, 5, 3)),
    ((17, 18, 12), (3.0, 2.5, 4.0), (45.0, 40.0, 44.0), (5, 16, 11)),
]


def _interfile(folder, name, image, scale):
    """Writes an interfile header + float32 data as the reference's LoadImage
    reads them (image [x][y][z], data stored z-major)."""
    nx, ny, nz = image.shape
    with open(os.path.join(folder, name + ".hdr"), "w") as f:
        f.write("!INTERFILE :=\n")
        f.write(f"name of data file := {name}.img\n")
        for i, (n, sc) in enumerate(zip(image.shape, scale)):
            f.write(f"matrix size [{i + 1}] := {n}\n")
            f.write(f"scaling factor (mm/pixel) [{i + 1}] := {sc}\n")
    image.transpose(2, 1, 0).astype(np.float32).tofile(os.path.join(folder, name + ".img"))
    return os.path.join(folder, name + ".hdr")


def gen_prep(_R):
    """CropAndDownscale and PrepareImages of the reference run with a recording
    identity resize: the crop windows, the resize options the reference passes,
    the sizes PrepareImages derives and its attenuation threshold."""
    Utils, T = refpy.load_utils()
    rng = np.random.default_rng(11)
    out = {}
    for i, (shape, vox, crop, dims) in enumerate(PREP_CASES):
        img = (rng.random(shape) * 4.0 - 0.5).astype(np.float32)
        T.CALLS.clear()
        cropped = Utils.CropAndDownscale(img, np.array(vox), np.array(crop), np.array(dims))
        (seen, oshape, kw), = T.CALLS
        assert np.array_equal(seen, cropped)
        out[f"case{i}_image"] = img
        out[f"case{i}_args"] = np.array(list(vox) + list(crop) + list(dims), dtype=np.float64)
        out[f"case{i}_cropped"] = cropped
        out[f"case{i}_out_shape"] = np.array(oshape)
        out[f"case{i}_resize_kwargs"] = np.array(sorted(f"{k}={v}" for k, v in kw.items()))
    # PrepareImages on interfile maps (mm): activity 30x28x20 @ (4, 4, 5),
    # attenuation with values around its 0.001 threshold
    act = (rng.random((30, 28, 20)) * 3.0).astype(np.float32)
    atn = (rng.random((30, 28, 20)) * 0.004).astype(np.float32)
    with tempfile.TemporaryDirectory() as tmp:
        fa = _interfile(tmp, "act", act, (4.0, 4.0, 5.0))
        fm = _interfile(tmp, "atn", atn, (4.0, 4.0, 5.0))
        loaded, size, scale = Utils.LoadImage(fa)
        assert np.array_equal(loaded, act)
        T.CALLS.clear()
        size_desired = [96.0, 88.0, None]
        scale_desired = np.array([8.0, 8.0, 10.0])
        a, m, sd, dd = Utils.PrepareImages(fa, fm, size_desired, scale_desired)
        out["prep_act"] = act
        out["prep_atn"] = atn
        out["prep_scale"] = np.array([4.0, 4.0, 5.0])
        out["prep_size_desired_in"] = np.array([96.0, 88.0, np.nan])
        out["prep_scale_desired"] = scale_desired
        out["prep_act_cropped"] = a
        out["prep_atn_cropped_thresholded"] = m
        out["prep_size_desired"] = np.asarray(sd, dtype=np.float64)
        out["prep_dims_desired"] = np.asarray(dd)
        out["prep_resize_shapes"] = np.array([c[1] for c in T.CALLS])
    _save("prep", **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=",".join(ALL))
    args = ap.parse_args()
    which = set(args.only.split(","))
    import warnings

    warnings.simplefilter("ignore")
    R = refpy.load()
    from oracle import build_oracle

    build_oracle.build_ref()
    if "rays" in which:
        gen_rays(R)
    if "tables" in which:
        gen_tables(R)
    if "sss_tof13_slice" in which:
        gen_sss_slice(R)
    sss = [w.split("_", 1)[1] for w in which if w.startswith("sss_") and w != "sss_tof13_slice"]
    if sss:
        gen_sss(R, sss)
    if "upsample" in which:
        gen_upsample(R)
    if "upsample_lut" in which:
        gen_upsample_luts(R)
    if "mask" in which:
        gen_mask(R)
    if "fit" in which:
        gen_fit(R)
    if "span" in which:
        gen_span(R)
    if "listmode" in which:
        gen_listmode(R)
    if "prep" in which:
        gen_prep(R)
    if "support" in which:
        gen_support(R)


if __name__ == "__main__":
    main()
