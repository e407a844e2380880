"""Synthetic scanners, phantoms and problem presets for the TOF-SSS engine.

The reference runs on CASToR geometries and reconstructed images that are not
available here; these seeded generators stand in for them with the shapes,
sizes and value ranges of the benchmark workloads.  Units follow the
reference's internal convention (``Python/openSSS/Geometry.py:94-97`` and
``Python/openSSS/Utils.py:100-109``): positions and image bounds in cm,
attenuation in cm^-1, detector face size in mm.

Array layouts match the reference:

* ``Geometry``      float64 ``[rings, detectors, 3]`` crystal centres (cm)
* ``NormalVectors`` float64 ``[rings, detectors, 3]`` crystal face normals
* ``ActivityMap`` / ``AttenuationMap`` float32 ``[Nx, Ny, Nz]`` (x fastest
  when flattened in Fortran order, as ``SingleScatterSimulationTOF.py:187-188``
  does)
* ``ImageSize``     float64 ``[xMin, yMin, zMin, xMax, yMax, zMax]`` (cm)
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

LIGHT_SPEED_CM_PER_PS = 299792458.0 * 1e-10


@dataclasses.dataclass
class Scanner:
    geometry: np.ndarray  # [NR, ND, 3] cm
    normals: np.ndarray  # [NR, ND, 3]
    detector_size_mm: np.ndarray  # [2]

    @property
    def nr_rings(self) -> int:
        return self.geometry.shape[0]

    @property
    def nr_detectors(self) -> int:
        return self.geometry.shape[1]


def ring_scanner(nr_detectors: int = 760, nr_rings: int = 80, radius_cm: float = 41.0,
                 ring_pitch_cm: float = 0.32, crystal_mm: float = 3.2,
                 phase: float = 0.0) -> Scanner:
    """Ideal cylindrical scanner: crystal k of ring r sits at angle
    2*pi*(k + phase)/ND, axial position (r - (NR-1)/2) * pitch, with an inward
    unit face normal."""
    phi = 2.0 * np.pi * (np.arange(nr_detectors) + phase) / nr_detectors
    z = (np.arange(nr_rings) - (nr_rings - 1) / 2.0) * ring_pitch_cm
    geom = np.zeros((nr_rings, nr_detectors, 3))
    geom[:, :, 0] = radius_cm * np.cos(phi)[None, :]
    geom[:, :, 1] = radius_cm * np.sin(phi)[None, :]
    geom[:, :, 2] = z[:, None]
    normals = np.zeros_like(geom)
    normals[:, :, 0] = -np.cos(phi)[None, :]
    normals[:, :, 1] = -np.sin(phi)[None, :]
    return Scanner(geom, normals, np.array([crystal_mm, crystal_mm]))


def image_bounds(shape, voxel_cm) -> np.ndarray:
    """Centred image bounds in the reference's ImageSize order (cm)."""
    vx = np.broadcast_to(np.asarray(voxel_cm, dtype=np.float64), (3,))
    half = np.asarray(shape, dtype=np.float64) * vx / 2.0
    return np.array([-half[0], -half[1], -half[2], half[0], half[1], half[2]])


def cylinder_phantom(shape, voxel_cm, seed: int, radius_cm: float = 10.0,
                     length_cm: float = 18.0, mu_water: float = 0.096,
                     lung_radius_cm: float = 2.5, mu_lung: float = 0.025,
                     sphere_diam_mm=(10, 13, 17, 22, 28, 37), sphere_ring_cm: float = 5.7,
                     jitter_cm: float = 0.2, background: float = 1.0, contrast: float = 4.0):
    """Water cylinder with a centred lung insert and six hot spheres.

    Returns ``(activity, attenuation, image_size)``; the volumes are float32
    ``[Nx, Ny, Nz]``.  Membership is decided at voxel centres.  Sphere centres
    sit on a ring of ``sphere_ring_cm`` in the central plane, 60 degrees apart,
    each jittered by up to ``jitter_cm`` per axis from ``seed``.
    """
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    bounds = image_bounds(shape, voxel_cm)
    vx = np.broadcast_to(np.asarray(voxel_cm, dtype=np.float64), (3,))
    xc = bounds[0] + (np.arange(nx) + 0.5) * vx[0]
    yc = bounds[1] + (np.arange(ny) + 0.5) * vx[1]
    zc = bounds[2] + (np.arange(nz) + 0.5) * vx[2]
    X, Y, Z = np.meshgrid(xc, yc, zc, indexing="ij")
    r2 = X * X + Y * Y
    body = (r2 <= radius_cm ** 2) & (np.abs(Z) <= length_cm / 2.0)
    lung = body & (r2 <= lung_radius_cm ** 2)
    mu = np.zeros(shape, dtype=np.float32)
    mu[body] = mu_water
    mu[lung] = mu_lung
    act = np.zeros(shape, dtype=np.float32)
    act[body] = background
    for i, d_mm in enumerate(sphere_diam_mm):
        ang = 2.0 * np.pi * i / len(sphere_diam_mm)
        c = np.array([sphere_ring_cm * math.cos(ang), sphere_ring_cm * math.sin(ang), 0.0])
        c = c + rng.uniform(-jitter_cm, jitter_cm, size=3)
        rad = d_mm / 20.0
        inside = ((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) <= rad * rad
        act[inside & body] = background * contrast
    return act, mu, bounds


def sampled_rings(nr_rings: int, nr_rings_used: int) -> np.ndarray:
    """Rings simulated by the SSS (``SingleScatterSimulationTOF.py:153``)."""
    return np.floor(np.linspace(0, nr_rings - 1, nr_rings_used) + 0.5).astype(np.int64)


def sampled_detectors(nr_detectors: int, nr_detectors_used: int) -> np.ndarray:
    """Detectors simulated per ring (``SingleScatterSimulationTOF.py:159-167``):
    an accumulated floor with step ND/NDU starting from crystal 0."""
    step = nr_detectors / nr_detectors_used
    det = np.zeros(nr_detectors_used, dtype=np.int64)
    for d in range(1, nr_detectors_used):
        det[d] = int(np.floor(det[d - 1] + step))
    return det


def tof_bins(nr_bins: int, bin_width_cm: float):
    """(TOFRange, bin width in ps) for ``nr_bins`` bins of ``bin_width_cm``:
    a path difference of w cm is a time difference of 2w/c."""
    width_ps = 2.0 * bin_width_cm / LIGHT_SPEED_CM_PER_PS
    return nr_bins * width_ps / 2.0, width_ps


@dataclasses.dataclass
class SSSProblem:
    """All inputs of one ``SingleScatterSimulationTOF`` call."""
    name: str
    activity: np.ndarray
    attenuation: np.ndarray
    image_size: np.ndarray
    scanner: Scanner
    nr_rings_used: int
    nr_detectors_used: int
    sample_step: np.ndarray
    energy_resolution: float
    energy_threshold: float
    tof_resolution: float
    tof_range: float
    nr_bins: int

    @property
    def grid(self):
        return tuple(int(s) for s in self.activity.shape)


def make_problem(name: str, shape, voxel_cm, nru: int, ndu: int, nr_bins: int,
                 bin_width_cm: float | None, tof_resolution_ps: float, seed: int = 0,
                 scanner: Scanner | None = None, radius_cm: float = 10.0,
                 sample_step=(2, 2, 2), energy_threshold: float = 435.0,
                 energy_resolution: float = 0.12) -> SSSProblem:
    scanner = scanner if scanner is not None else ring_scanner()
    act, mu, bounds = cylinder_phantom(shape, voxel_cm, seed, radius_cm=radius_cm)
    if bin_width_cm is None:
        tof_range = 1000.0
    else:
        tof_range, _ = tof_bins(nr_bins, bin_width_cm)
    return SSSProblem(name, act, mu, bounds, scanner, nru, ndu,
                      np.asarray(sample_step, dtype=np.int64), energy_resolution,
                      energy_threshold, tof_resolution_ps, tof_range, nr_bins)


def nontof_40x40x20(seed: int = 0) -> SSSProblem:
    """Plain non-TOF SSS, small: 40x40x20 @ 10 mm, 8 rings x 32 detectors,
    one TOF bin with a 1e6 ps kernel (unit TOF weights)."""
    return make_problem("nontof-40x40x20", (40, 40, 20), 1.0, 8, 32, 1, None, 1.0e6, seed)


def tof13_64x64x48(seed: int = 0) -> SSSProblem:
    """Plain TOF-SSS single instance: 64x64x48 @ 6 mm, 16 rings x 48
    detectors, 13 TOF bins of 39 mm, 214 ps FWHM timing kernel."""
    return make_problem("tof13-64x64x48", (64, 64, 48), 0.6, 16, 48, 13, 3.9, 214.0, seed)


def tof33_128x128x96(seed: int = 0) -> SSSProblem:
    """Precision stress: 128x128x96 @ 4 mm, 32 rings x 96 detectors,
    33 TOF bins of 15 mm, 214 ps FWHM.

    The scanner is rotated by half a crystal: with crystal 0 at (41, 0) cm,
    736 of the 35 million legs of this volume (scatter points on voxel faces
    to that crystal, through exact voxel corners) make the reference's
    traversal run past Nx+Ny+Nz voxels and raise IndexError."""
    return make_problem("tof33-128x128x96", (128, 128, 96), 0.4, 32, 96, 33, 1.5, 214.0, seed,
                        scanner=ring_scanner(phase=0.5))


def uneven_instances(count: int = 64, seed: int = 0):
    """Uneven batch: volumes from 32x32x24 to 96x96x64 on a 40 cm FOV,
    24-64 detectors x 8-24 rings, TOF bins in {1, 13, 33}, body radius
    8-18 cm, all drawn from ``seed``.

    The scanner is rotated by half a crystal.  Scatter points sit on voxel
    faces ((x+1)*FOV/n - FOV/2, SingleScatterSimulationTOF.py:388, :394); a
    leg from such a point to a crystal on an axis (x or y exactly 0 or
    +-41 cm) can pass exactly through voxel corners, where the reference's
    traversal runs past Nx+Ny+Nz voxels and raises IndexError (on 15 of these 64
    volumes with the unrotated ring).  No crystal sits on an axis
    after the half-crystal rotation."""
    rng = np.random.default_rng(seed)
    scanner = ring_scanner(phase=0.5)
    out = []
    for i in range(count):
        n = int(rng.integers(32, 97))
        nz = int(rng.integers(24, 65))
        vox_xy = 40.0 / n
        vox = (vox_xy, vox_xy, vox_xy)
        ndu = int(rng.integers(24, 65))
        nru = int(rng.integers(8, 25))
        bins = int(rng.choice([1, 13, 33]))
        radius = float(rng.uniform(8.0, 18.0))
        if bins == 1:
            width, res = None, 1.0e6
        elif bins == 13:
            width, res = 3.9, 214.0
        else:
            width, res = 1.5, 214.0
        out.append(make_problem(f"uneven-{i}", (n, n, nz), vox, nru, ndu, bins, width, res,
                                seed=seed * 1000 + i, radius_cm=min(radius, 19.0), scanner=scanner))
    return out


def stratified_points(n_points: int, count: int) -> np.ndarray:
    """``count`` scatter-point numbers spread evenly over ``0..n_points-1``
    (lattice order, so every sampled z-slice contributes): a sample for
    checks that a first-N cut would take from the lowest slices only."""
    if count >= n_points:
        return np.arange(n_points, dtype=np.int64)
    return np.unique(np.floor(np.linspace(0, n_points - 1, count) + 0.5).astype(np.int64))


def tiny_problem(nr_bins: int = 3, seed: int = 0, shape=(12, 12, 6), nd: int = 48, nr: int = 6,
                 nru: int = 3, ndu: int = 8, voxel_cm: float = 2.0) -> SSSProblem:
    """Small case the interpreted reference finishes in seconds."""
    scanner = ring_scanner(nd, nr, radius_cm=20.0, ring_pitch_cm=1.0)
    if nr_bins == 1:
        width, res = None, 1.0e6
    else:
        width, res = 3.0, 214.0
    return make_problem(f"tiny-b{nr_bins}", shape, voxel_cm, nru, ndu, nr_bins, width, res,
                        seed=seed, scanner=scanner, radius_cm=8.0)


def served_beds(seed: int = 0):
    """Resident problems of the served workload: four small bed positions of
    the plain non-TOF size (40x40x20 @ 1 cm, 8 rings x 32 crystals, phantoms
    seeded per bed) and four large ones drawn by the uneven-batch generator
    (seed 5).  Returns (small, large)."""
    small = [dataclasses.replace(nontof_40x40x20(seed=seed * 10 + b), name=f"bed{b}-small") for b in range(4)]
    large = [dataclasses.replace(pr, name=f"bed{b}-large")
             for b, pr in enumerate(uneven_instances(4, seed=5))]
    return small, large


def listmode_header(name: str, n_events: int, tof_range: float = 1000.0, random_flag: bool = True,
                    normalization_flag: bool = True, attenuation_flag: bool = False,
                    duration: float = 600.0) -> dict:
    """CASToR header fields of the synthetic list-mode files (single line per
    event, TOF)."""
    return {"data_filename": f"{name}.Cdf", "nb_events": int(n_events), "data_mode": "list-mode",
            "data_type": "PET", "start_time": 0.0, "duration": float(duration), "scanner_name": "SYNTH",
            "isotope": "F18", "calibration_factor": 1.0, "nb_max_lines": 1,
            "attenuation_flag": attenuation_flag, "normalization_flag": normalization_flag,
            "scatter_flag": False, "random_flag": random_flag, "tof_flag": True, "tof_resolution": 214.0,
            "tof_bin_size": None, "tof_nb_bins": None, "tof_range": float(tof_range)}


def synthetic_listmode(directory: str, name: str, n_events: int, crystals_per_ring: int, rings: int,
                       seed: int = 0, tof_range: float = 1000.0, tof_sigma: float = 400.0,
                       random_flag: bool = True, normalization_flag: bool = True,
                       attenuation_flag: bool = False, duration: float = 600.0) -> str:
    """Writes a seeded CASToR list-mode file pair ``<name>.Cdh`` / ``<name>.Cdf``
    (single line per event, TOF) and returns the header's file name.  Crystal
    IDs are uniform over the scanner (ring * crystals_per_ring + crystal); TOF
    differences are Gaussian with ``tof_sigma`` ps, so some fall outside
    ``tof_range``; correction factors are seeded uniform values."""
    import os

    from . import Headerfile

    header = listmode_header(name, n_events, tof_range, random_flag, normalization_flag, attenuation_flag,
                             duration)
    ev = synthetic_events(header, crystals_per_ring, rings, seed, tof_sigma)
    ev.tofile(os.path.join(directory, header["data_filename"]))
    Headerfile.WriteHeaderFile(header, os.path.join(directory, f"{name}.Cdh"))
    return f"{name}.Cdh"


def synthetic_events(header: dict, crystals_per_ring: int, rings: int, seed: int = 0,
                     tof_sigma: float = 400.0) -> np.ndarray:
    """Seeded event records for ``header`` (see ``synthetic_listmode``) as a
    structured array whose bytes are the data file."""
    from . import Coincidence

    rng = np.random.default_rng(seed)
    n_events = header["nb_events"]
    fmt, _ = Coincidence.GenerateEventClass(header)
    ncorr = (int(header["attenuation_flag"]) + int(header["random_flag"]) + int(header["normalization_flag"])
             + 1)
    duration = header["duration"]
    fields = [("time", "<u4")] + [(f"c{i}", "<f4") for i in range(ncorr)] + [("id1", "<u4"), ("id2", "<u4")]
    ev = np.zeros(int(n_events), dtype=np.dtype(fields))
    ev["time"] = np.sort(rng.integers(0, int(duration * 1000), size=n_events)).astype(np.uint32)
    for i in range(ncorr - 1):
        ev[f"c{i}"] = rng.uniform(0.5, 2.0, size=n_events).astype(np.float32)
    ev[f"c{ncorr - 1}"] = (rng.normal(0.0, tof_sigma, size=n_events)).astype(np.float32)
    ncrystals = crystals_per_ring * rings
    ev["id1"] = rng.integers(0, ncrystals, size=n_events).astype(np.uint32)
    ev["id2"] = rng.integers(0, ncrystals, size=n_events).astype(np.uint32)
    assert ev.dtype.itemsize == Coincidence.record_bytes(fmt)
    return ev
