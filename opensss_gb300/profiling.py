"""Small, self-contained cases of each GPU kernel for profiler captures.

    python -m opensss_gb300.profiling CASE [--reps N]

CASE is one of ``upsample``, ``mask``, ``fit``, ``listmode``, ``pair``,
``batch``, ``prep``.  Each case builds seeded inputs larger than the 129 MB L2 but a
few GB at most on the device, runs the kernel ``--reps`` times and checks
the status word, so that a capture of one to three launches ends within a
minute or two.
"""

from __future__ import annotations

import argparse
import os

import numpy as np
import torch

from . import geometry as G, workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _att():
    return np.load(os.path.join(ROOT, "tests", "golden", "tables.npz"))["att_table"]


def _engine(pr):
    from .engine import TofSSS

    return TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, _att(),
                  pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                  pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins)


def case_upsample(reps):
    """13 bins of a 16 x 48 sampled sinogram onto a 380-crystal x 40-ring
    scanner: 381 x 190 x 1600 outputs (463 MB)."""
    from .Interpolation import upsample_device

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
    from .TailsMask import tail_mask_device

    pr = W.tof13_64x64x48()
    sc = W.ring_scanner(380, 40, radius_cm=41.0, ring_pitch_cm=0.64)
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, 380, 40, ID_Shidt=False)
    for _ in range(reps):
        tail_mask_device(pr.attenuation, pr.image_size, sc.geometry, lor, si, 4)


def case_fit(reps):
    """Back-projection fit of four TOF bins of seeded sinograms in one pass on
    a 380 x 40 scanner, AF 4."""
    from .BackProjection import fit_bins_device

    pr = W.tof13_64x64x48()
    sc = W.ring_scanner(380, 40, radius_cm=41.0, ring_pitch_cm=0.64)
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, 380, 40, ID_Shidt=False)
    shp = (381 * 190, 1600)
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    prm = torch.poisson(torch.full((4,) + shp, 3.0, device="cuda"), generator=g)
    rnd = torch.full(shp, 0.3, device="cuda")
    scat = torch.rand((4,) + shp, device="cuda", generator=g)
    mask = (torch.rand(shp, device="cuda", generator=g) < 0.3).to(torch.uint8)
    cell = np.arange(shp[0], dtype=np.int64) * shp[1]
    ring = np.arange(shp[1], dtype=np.int64)
    zr = float(sc.geometry[-1, 0, 2]) + 0.3
    bounds = np.array([pr.image_size[0], pr.image_size[1], -zr, pr.image_size[3], pr.image_size[4], zr])
    for _ in range(reps):
        fit_bins_device(prm, rnd, mask, scat, shp[0] * shp[1], cell, ring, np.array([40, 40, 26]), bounds,
                        sc.geometry, lor, si[:40, :40].T, 4)


def case_listmode(reps):
    """10M list-mode events into the demo's reduced sinogram (mash 2, span 19)."""
    from .Datafile import histogram_device

    header = W.listmode_header("p_df", 10_000_000)
    ev = torch.from_numpy(W.synthetic_events(header, 760, 80, seed=1).view(np.uint8).reshape(-1)).cuda()
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, 380, 80, ID_Shidt=False)
    _, _, lut, _ = G.SinogramLUT(80, 19, 79)
    for _ in range(reps):
        histogram_device(ev, header, lor, lut, 6, 1000.0, mash=2)


def case_pair(reps):
    """The 64x64x48, 16 x 48, 13-bin instance on its first 400 scatter points."""
    pr = W.tof13_64x64x48()
    e = _engine(pr)
    for _ in range(reps):
        e.run(pr.activity, pr.attenuation, pr.image_size, max_points=400)


def case_batch(reps):
    """Eight instances of the uneven-batch generator as one plan."""
    from .batch import BatchSSS

    inst = W.uneven_instances(8, seed=3)
    b = BatchSSS([(_engine(pr), pr.activity, pr.attenuation, pr.image_size) for pr in inst],
                 workspace_bytes=4 << 30)
    for _ in range(reps):
        b.run()


def case_prep(reps):
    """CropAndDownscale of a seeded 400x400x280 float32 map (1.6 x 1.6 x 2 mm)
    cropped to 600 x 600 x 480 mm and resized to 75 x 75 x 48."""
    from .Utils import crop_downscale_device, crop_window

    rng = np.random.default_rng(3)
    img = torch.from_numpy(rng.gamma(2.0, 1.0, size=(400, 400, 280)).astype(np.float32)).cuda()
    win = crop_window(tuple(img.shape), (1.6, 1.6, 2.0), (600.0, 600.0, 480.0))
    for _ in range(reps):
        crop_downscale_device(img, win, (75, 75, 48))
    torch.cuda.synchronize()


CASES = {"upsample": case_upsample, "mask": case_mask, "fit": case_fit, "listmode": case_listmode,
         "pair": case_pair, "batch": case_batch, "prep": case_prep}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()
    CASES[a.case](a.reps)
    print(f"{a.case}: ok")


if __name__ == "__main__":
    main()
