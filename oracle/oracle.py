"""Python face of the oracle (test infrastructure only).

ORACLE — only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its
CPU baseline and its error checks against FP64) import this module, and only
as the test oracle or the timed CPU reference arm.  It loads ``oracle/_build/libsssoracle.so`` (the FP64 C
restatement) and, where it was built, the reference's own MEX ray tracers from
``oracle/_ref``; ``sss_compact(..., gpu=True)`` runs the same restatement's
SSS on the current CUDA device (``oracle/_build/libsssoracle_gpu.so``, the
FP64 GPU oracle).  The per-problem tables are rebuilt here independently of the
engine, with the same NumPy/SciPy calls the reference makes
(``Python/openSSS/SingleScatterSimulationTOF.py:99-150``).
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TOF_ENTRIES = 8001

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_build", "libsssoracle.so")
        if not os.path.exists(path):
            from oracle import build_oracle  # noqa: WPS433

            build_oracle.build_oracle()
        _lib = C.CDLL(path)
        _lib.orc_trace_batch.restype = C.c_int
        _lib.orc_sss.restype = C.c_int
        _lib.orc_mask.restype = C.c_int
        _lib.orc_fit.restype = C.c_int
        _lib.orc_scatter_points.restype = C.c_int64
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- tables


def efficiency_table(energies, threshold, resolution, eref=511):
    """0.5*(1 - erf((Eth - E)/(511*ER/2/sqrt(ln 2)))) (SingleScatterSimulationTOF.py:139-140)."""
    from scipy.special import erf

    return 0.5 * (1 - erf((threshold - energies) / (eref * resolution / 2 / np.sqrt(np.log(2)))))


def tof_table(nbins, tof_range, resolution):
    """TOFEfficiencyTable over -4000..4000 ps (SingleScatterSimulationTOF.py:261-295)."""
    offset = np.arange(-4000, 4001)
    bw = 2 * tof_range / nbins
    shifts = ((np.arange(1, nbins + 1) - (nbins + 1) / 2) * bw).reshape(-1, 1)
    prob = offset.reshape(1, -1) - shifts
    prob = np.exp(-(prob ** 2) / (resolution ** 2 / 4 / np.log(2)))
    s = np.sum(prob, axis=0)
    zero = s == 0
    with np.errstate(invalid="ignore", divide="ignore"):
        prob = prob / s
    prob[:, zero] = 0
    return np.ascontiguousarray(prob)


def problem_tables(att_table, threshold, resolution, nbins, tof_range, tof_resolution):
    eref = 511
    ei = int(np.where(att_table[:, 0] == eref)[0][0])
    ratio = att_table[:, 1] / att_table[ei, 1]
    eff = efficiency_table(att_table[:, 0], threshold, resolution)
    return dict(eff=np.ascontiguousarray(eff, dtype=np.float64),
                ratio=np.ascontiguousarray(ratio, dtype=np.float64),
                tof=tof_table(nbins, tof_range, tof_resolution))


def sampled_rings(nr, nru):
    return np.floor(np.linspace(0, nr - 1, nru) + 0.5).astype(np.int64)


def sampled_detectors(nd, ndu):
    step = nd / ndu
    d = np.zeros(ndu, dtype=np.int64)
    for i in range(1, ndu):
        d[i] = int(np.floor(d[i - 1] + step))
    return d


# ---------------------------------------------------------------- tracing


def trace_batch(grid, bounds, lines, eps=1e-20, nthreads=0, allow_overrun=False):
    """Returns (counts, lengths, 1-based indices, samples) in [n, cap] layout;
    a ray whose traversal overruns Nx+Ny+Nz voxels gets count -1 when
    ``allow_overrun`` (the reference raises IndexError there)."""
    L = lib()
    grid = np.ascontiguousarray(grid, dtype=np.int64)
    bounds = np.ascontiguousarray(bounds, dtype=np.float64)
    lines = np.ascontiguousarray(lines, dtype=np.float64).reshape(-1, 6)
    n = lines.shape[0]
    cap = int(grid.sum())
    counts = np.zeros(n, np.int32)
    ln = np.zeros((n, cap))
    ix = np.zeros((n, cap), np.int32)
    sm = np.zeros((n, cap))
    bad = L.orc_trace_batch(_p(grid), _p(bounds), _p(lines), C.c_int64(n), C.c_double(eps),
                            C.c_int(cap), _p(counts), _p(ln), _p(ix), _p(sm), C.c_int(nthreads))
    if bad and not allow_overrun:
        raise RuntimeError(f"oracle trace overflow on {bad} rays")
    return counts, ln, ix, sm


class RefTracer:
    """The reference's MEX ray tracer compiled from source (oracle/_ref)."""

    def __init__(self, tof=True):
        name = "libref_raytracing3dtof.so" if tof else "libref_raytracing3d.so"
        path = os.path.join(HERE, "_ref", name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.lib.ref_trace.restype = C.c_int
        self.tof = tof

    def __call__(self, grid, bounds, line):
        grid = np.ascontiguousarray(grid, dtype=np.float64)
        bounds = np.ascontiguousarray(bounds, dtype=np.float64)
        line = np.ascontiguousarray(line, dtype=np.float64)
        cap = int(grid.sum()) + 8
        ln = np.zeros(cap)
        ix = np.zeros(cap, np.int32)
        sm = np.zeros(cap)
        n = self.lib.ref_trace(_p(grid), _p(bounds), _p(line), _p(ln), _p(ix), _p(sm), C.c_int(cap))
        if n < 0:
            raise RuntimeError("reference MEX tracer raised")
        return ln[:n].copy(), ix[:n].copy(), sm[:n].copy()


# ---------------------------------------------------------------- SSS


class _SSSProblem(C.Structure):
    _fields_ = [
        ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
        ("act", C.c_void_p), ("mu", C.c_void_p), ("image_size", C.c_void_p),
        ("nr", C.c_int64), ("nd", C.c_int64),
        ("geom", C.c_void_p), ("normals", C.c_void_p), ("det_size", C.c_void_p),
        ("nru", C.c_int64), ("ndu", C.c_int64),
        ("rings", C.c_void_p), ("dets", C.c_void_p),
        ("step", C.c_int64 * 3), ("nbins", C.c_int64),
        ("tof_table", C.c_void_p), ("eff", C.c_void_p), ("ratio", C.c_void_p),
        ("energy_ref", C.c_int64), ("sp_begin", C.c_int64), ("sp_end", C.c_int64),
        ("sp_list", C.c_void_p), ("sp_count", C.c_int64),
    ]


def _sss_struct(act, mu, image_size, geometry, normals, det_size, nru, ndu, step, tables,
                sp_begin=0, sp_end=-1, points=None):
    keep = []

    def hold(a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a

    actf = hold(np.asarray(act).flatten(order="F"), np.float32)
    muf = hold(np.asarray(mu).flatten(order="F"), np.float32)
    nx, ny, nz = act.shape
    nr, nd = geometry.shape[:2]
    s = _SSSProblem()
    s.nx, s.ny, s.nz = nx, ny, nz
    s.act, s.mu = actf.ctypes.data, muf.ctypes.data
    s.image_size = hold(image_size, np.float64).ctypes.data
    s.nr, s.nd = nr, nd
    s.geom = hold(geometry, np.float64).ctypes.data
    s.normals = hold(normals, np.float64).ctypes.data
    s.det_size = hold(det_size, np.float64).ctypes.data
    s.nru, s.ndu = nru, ndu
    s.rings = hold(sampled_rings(nr, nru), np.int64).ctypes.data
    s.dets = hold(sampled_detectors(nd, ndu), np.int64).ctypes.data
    for i in range(3):
        s.step[i] = int(step[i])
    tof = hold(tables["tof"], np.float64)
    s.nbins = tof.shape[0]
    s.tof_table = tof.ctypes.data
    s.eff = hold(tables["eff"], np.float64).ctypes.data
    s.ratio = hold(tables["ratio"], np.float64).ctypes.data
    s.energy_ref = 511
    s.sp_begin, s.sp_end = sp_begin, sp_end
    if points is not None:
        lst = hold(np.asarray(points).reshape(-1), np.int64)
        s.sp_list, s.sp_count = lst.ctypes.data, len(lst)
    return s, keep


def scatter_points(act, mu, image_size, step):
    s, keep = _sss_struct(act, mu, image_size, np.zeros((1, 2, 3)), np.zeros((1, 2, 3)),
                          np.ones(2), 1, 1, step,
                          dict(tof=np.ones((1, TOF_ENTRIES)), eff=np.ones(2000), ratio=np.ones(2000)))
    n = lib().orc_scatter_points(C.byref(s), None, None)
    xyz = np.zeros((n, 3))
    sl = np.zeros(n, np.int64)
    lib().orc_scatter_points(C.byref(s), _p(xyz), _p(sl))
    return xyz, sl


_gpu_lib = None


def gpu_lib():
    """The FP64 GPU oracle (``oracle/_build/libsssoracle_gpu.so``)."""
    global _gpu_lib
    if _gpu_lib is None:
        path = os.path.join(HERE, "_build", "libsssoracle_gpu.so")
        if not os.path.exists(path):
            from oracle import build_oracle  # noqa: WPS433

            build_oracle.build_oracle_gpu()
        _gpu_lib = C.CDLL(path)
        _gpu_lib.orc_sss_gpu.restype = C.c_int
        _gpu_lib.orc_sss_gpu.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    return _gpu_lib


def sss_compact(act, mu, image_size, geometry, normals, det_size, att_table, energy_resolution,
                energy_threshold, nru, ndu, step, tof_resolution, tof_range, nbins,
                sp_begin=0, sp_end=-1, nthreads=0, tof=None, points=None, gpu=False, leg_bytes=0):
    """FP64 SSS; returns compact [B, NRU*NRU, NDU, NDU] (pairs di1<=di2 filled).
    ``tof`` replaces the TOF table ([B, 8001], e.g. an emulation of another
    evaluation of the weights).  ``points`` (ascending scatter-point numbers
    in lattice order) restricts the sum to those points instead of the range
    [sp_begin, sp_end); each z-slice is then normalised over its listed
    points, as the engine does for the same subset.  ``gpu`` runs the same
    restatement on the current CUDA device (``orc_sss_gpu``, the FP64 GPU
    oracle), holding at most ``leg_bytes`` of voxel lists at once (0: 4 GB)."""
    tables = problem_tables(att_table, energy_threshold, energy_resolution, nbins, tof_range,
                            tof_resolution)
    if tof is not None:
        if np.shape(tof) != (nbins, TOF_ENTRIES):
            raise ValueError(f"tof table must be [{nbins}, {TOF_ENTRIES}], got {np.shape(tof)}")
        tables["tof"] = np.ascontiguousarray(tof, dtype=np.float64)
    s, keep = _sss_struct(act, mu, image_size, geometry, normals, det_size, nru, ndu, step,
                          tables, sp_begin, sp_end, points)
    out = np.zeros((nbins, nru * nru, ndu, ndu))
    if gpu:
        st = gpu_lib().orc_sss_gpu(C.addressof(s), _p(out), int(leg_bytes))
    else:
        st = lib().orc_sss(C.byref(s), _p(out), C.c_int(nthreads))
    if st != 0:
        raise RuntimeError(f"oracle SSS failed with status {st}")
    return out


def densify(compact, lor, nd, nru, ndu):
    """Compact [B, NRU^2, NDU, NDU] -> reference layout [B, ND+1, ND//2, NRU^2]."""
    nb = compact.shape[0]
    det = sampled_detectors(nd, ndu)
    out = np.zeros((nb, nd + 1, nd // 2, nru * nru), dtype=np.float32)
    a, b = np.triu_indices(ndu)
    ang = lor[det[a], det[b], 0].astype(np.int64)
    rad = lor[det[a], det[b], 1].astype(np.int64)
    for s in range(nru * nru):
        out[:, rad, ang, s] = compact[:, s, a, b]
    return out


# ---------------------------------------------------------------- mask / fit


def mask(mu, image_size, geometry, lor, sino_index, af, nthreads=0, use_activity=False, acf_below=0.0):
    """Tail mask (TailsMask.py:84-228): LORs whose attenuation factor is
    exactly 1, or with ``acf_below`` > 1 below that bound."""
    grid = np.ascontiguousarray(mu.shape, dtype=np.int64)
    muf = np.ascontiguousarray(mu.flatten(order="F"), dtype=np.float32)
    gb = np.ascontiguousarray(image_size, dtype=np.float64)
    geom = np.ascontiguousarray(geometry, dtype=np.float64)
    lor = np.ascontiguousarray(lor, dtype=np.int16)
    si = np.ascontiguousarray(sino_index, dtype=np.int16)
    nr, nd = geom.shape[:2]
    out = np.zeros((nd + 1, nd // 2, nr * nr), np.uint8)
    st = lib().orc_mask(_p(grid), _p(muf), _p(gb), C.c_int64(nr), C.c_int64(nd), _p(geom), _p(lor),
                        _p(si), C.c_int64(af), C.c_int(int(use_activity)), _p(out),
                        C.c_int(nthreads), C.c_double(acf_below))
    if st:
        raise RuntimeError(f"oracle mask failed {st}")
    return out


def fit(prompts, scatters, randoms, mask_f32, grid, bounds, geometry, lor, sino_index, af,
        nthreads=0, return_images=False):
    g = np.ascontiguousarray(grid, dtype=np.int64)
    gb = np.ascontiguousarray(bounds, dtype=np.float64)
    geom = np.ascontiguousarray(geometry, dtype=np.float64)
    nr, nd = geom.shape[:2]
    lor = np.ascontiguousarray(lor, dtype=np.int16)
    si = np.ascontiguousarray(sino_index, dtype=np.int16)
    P = np.ascontiguousarray(prompts, dtype=np.float32)
    S = np.ascontiguousarray(scatters, dtype=np.float32)
    R = np.ascontiguousarray(randoms, dtype=np.float32)
    M = np.ascontiguousarray(mask_f32, dtype=np.float32)
    scale = np.zeros(1, np.float32)
    imgs = np.zeros((4, int(np.prod(g))), np.float32)
    st = lib().orc_fit(_p(g), _p(gb), C.c_int64(nr), C.c_int64(nd), _p(geom), _p(lor), _p(si),
                       C.c_int64(af), _p(P), _p(S), _p(R), _p(M), _p(scale), _p(imgs),
                       C.c_int(nthreads))
    if st:
        raise RuntimeError(f"oracle fit failed {st}")
    return (scale, imgs) if return_images else scale


def upsample_bin(sampled_bin, nru, ndu, nr, nd, lut, ringmap, sino_index):
    """One bin of InterpolateAllBins given the nearest-source tables.
    sampled_bin: [NRU*NRU, NDU, NDU] (sino = ri1*NRU + ri2)."""
    s = np.ascontiguousarray(sampled_bin, dtype=np.float64)
    lut = np.ascontiguousarray(lut, dtype=np.int32).reshape(-1)
    rm = np.ascontiguousarray(ringmap, dtype=np.int32)
    si = np.ascontiguousarray(sino_index, dtype=np.int16)
    out = np.zeros((nd + 1, nd // 2, nr * nr), np.float32)
    lib().orc_upsample_bin(_p(s), C.c_int64(nru), C.c_int64(ndu), C.c_int64(nr), C.c_int64(nd),
                           _p(lut), _p(rm), _p(si), _p(out))
    return out


def mask_pairs(mu, image_size, geometry, lor, pairs, nslices, af, nthreads=0, use_activity=False, acf_below=0.0):
    """Span tail mask on the expanded geometry (TailsMask.py:230-377)."""
    grid = np.ascontiguousarray(mu.shape, dtype=np.int64)
    muf = np.ascontiguousarray(mu.flatten(order="F"), dtype=np.float32)
    gb = np.ascontiguousarray(image_size, dtype=np.float64)
    geom = np.ascontiguousarray(geometry, dtype=np.float64)
    lor = np.ascontiguousarray(lor, dtype=np.int16)
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    nr, nd = geom.shape[:2]
    out = np.zeros((nd + 1, nd // 2, nslices), np.uint8)
    st = lib().orc_mask_pairs(_p(grid), _p(muf), _p(gb), C.c_int64(nr), C.c_int64(nd), _p(geom), _p(lor),
                              _p(pairs), C.c_int64(pairs.shape[0]), C.c_int64(nslices), C.c_int64(af),
                              C.c_int(int(use_activity)), _p(out), C.c_int(nthreads), C.c_double(acf_below))
    if st:
        raise RuntimeError(f"oracle span mask failed {st}")
    return out


def fit_pairs(prompts, scatters, randoms, mask_f32, grid, bounds, geometry, lor, pairs, af, nthreads=0):
    """Span scale fit, length-weighted (BackProjection.py:217-393)."""
    grid = np.ascontiguousarray(grid, dtype=np.int64)
    gb = np.ascontiguousarray(bounds, dtype=np.float64)
    geom = np.ascontiguousarray(geometry, dtype=np.float64)
    lor = np.ascontiguousarray(lor, dtype=np.int16)
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    nr, nd = geom.shape[:2]
    f = [np.ascontiguousarray(a, dtype=np.float32) for a in (prompts, scatters, randoms, mask_f32)]
    nslices = f[0].shape[2]
    out = np.zeros(1, np.float32)
    st = lib().orc_fit_pairs(_p(grid), _p(gb), C.c_int64(nr), C.c_int64(nd), _p(geom), _p(lor), _p(pairs),
                             C.c_int64(pairs.shape[0]), C.c_int64(nslices), C.c_int64(af), _p(f[0]), _p(f[1]),
                             _p(f[2]), _p(f[3]), _p(out), C.c_int(nthreads))
    if st:
        raise RuntimeError(f"oracle span fit failed {st}")
    return out
