"""Host side of the TOF-SSS engine: device buffers (torch), tables and the
calls into ``libsss300.so``.

``TofSSS`` keeps the scanner, sampling and tables resident on the device;
``run`` takes the activity and attenuation volumes (numpy or CUDA tensors)
and returns the sampled scatter sinogram in the engine's leg-pair layout
``[B, NL, NL]`` (see ``include/sss300.h``) as a CUDA tensor.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib, geometry, tables

WS_BUDGET_BYTES = 24 << 30  # default cap on the leg-list workspace per run


def _require_cuda(device):
    if not torch.cuda.is_available():
        raise _lib.EngineUnavailable("no CUDA device: the engine has no CPU path")
    dev = torch.device(device)
    if dev.type != "cuda":
        raise ValueError(f"device {dev} is not a CUDA device: the engine has no CPU path")
    # "cuda" means the current device; name it, so that devices compare equal
    return dev if dev.index is not None else torch.device("cuda", torch.cuda.current_device())


def as_device(a, dtype, device):
    """numpy / tensor -> contiguous CUDA tensor of dtype."""
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=device, dtype=dtype).contiguous()


def fortran_flat(vol, device):
    """[Nx, Ny, Nz] volume -> flat float32 CUDA tensor in Fortran order (x fastest),
    the reference's ``flatten(order="F")`` (SingleScatterSimulationTOF.py:187-188)."""
    if isinstance(vol, torch.Tensor):
        return vol.to(device=device, dtype=torch.float32).permute(2, 1, 0).contiguous().reshape(-1)
    return torch.from_numpy(np.ascontiguousarray(np.asarray(vol, dtype=np.float32).transpose(2, 1, 0))
                            ).reshape(-1).to(device)


def _ptr(t: torch.Tensor | None):
    return C.c_void_p(0 if t is None else t.data_ptr())


class TofSSS:
    """A configured TOF-SSS problem with scanner, sampling and tables on the GPU."""

    def __init__(self, Geometry, NormalVectors, DetectorSize, AttenuationTable, EnergyResolution,
                 EnergyThreshold, NrRingsUsed, NrDetectorsUsed, SampleStep, TOFResolution,
                 TOFRange, NrBins, device="cuda"):
        self.device = _require_cuda(device)
        _lib.lib()
        geom = np.asarray(Geometry, dtype=np.float64)
        self.nr, self.nd = geom.shape[:2]
        self.nru, self.ndu = int(NrRingsUsed), int(NrDetectorsUsed)
        self.nl = self.nru * self.ndu
        self.nbins = int(NrBins)
        if not 1 <= self.nbins <= 64:
            raise ValueError("NrBins must be 1..64")
        self.sample_step = [int(s) for s in np.asarray(SampleStep).reshape(-1)[:3]]
        self.detector_size = [float(x) for x in np.asarray(DetectorSize).reshape(-1)[:2]]
        self.tof_resolution = float(TOFResolution)
        self.tof_range = float(TOFRange)
        att = np.asarray(AttenuationTable, dtype=np.float64)
        self.rings_np = geometry.sampled_rings(self.nr, self.nru)
        self.dets_np = geometry.sampled_detectors(self.nd, self.ndu)
        dev = self.device
        self.geometry = as_device(geom, torch.float64, dev)
        self.normals = as_device(np.asarray(NormalVectors, dtype=np.float64), torch.float64, dev)
        self.rings = as_device(self.rings_np, torch.int32, dev)
        self.dets = as_device(self.dets_np, torch.int32, dev)
        log2w = tables.tof_log2_table(self.nbins, self.tof_range, self.tof_resolution)
        # one bin whose normalised weight is exactly 1 everywhere (the non-TOF case)
        self.unit_tof = self.nbins == 1 and not np.any(log2w)
        self.tof_log2w = as_device(log2w, torch.float32, dev)
        self.eff = as_device(tables.pair_efficiency_f32(att, float(EnergyThreshold),
                                                        float(EnergyResolution)), torch.float32, dev)
        self.ratio = as_device(tables.attenuation_ratio(att), torch.float32, dev)
        self._ws = None
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        # launch shape of the kernels (0 = the library's default); set by
        # opensss_gb300.autotune.tune or by hand
        self.pair_warps = 0
        self.leg_threads = 0

    # ------------------------------------------------------------------
    def problem(self, act_flat, mu_flat, shape, image_size, kahan: bool = False,
                unit_tof: bool | None = None) -> _lib.TofProblem:
        """``unit_tof`` None: use the leg integrals when the TOF table is all
        ones (``self.unit_tof``); False forces the voxel walk."""
        p = _lib.TofProblem()
        unit = self.unit_tof if unit_tof is None else (unit_tof and self.unit_tof)
        p.flags = (_lib.SSS_FLAG_KAHAN if kahan else 0) | (_lib.SSS_FLAG_UNIT_TOF if unit else 0)
        p.nx, p.ny, p.nz = (int(s) for s in shape)
        p.activity = act_flat.data_ptr()
        p.attenuation = mu_flat.data_ptr()
        for i, v in enumerate(np.asarray(image_size, dtype=np.float64).reshape(-1)[:6]):
            p.image_size[i] = float(v)
        p.nr, p.nd = self.nr, self.nd
        p.geometry = self.geometry.data_ptr()
        p.normals = self.normals.data_ptr()
        p.detector_size[0], p.detector_size[1] = self.detector_size
        p.nru, p.ndu = self.nru, self.ndu
        p.rings = self.rings.data_ptr()
        p.detectors = self.dets.data_ptr()
        for i in range(3):
            p.sample_step[i] = self.sample_step[i]
        p.nbins = self.nbins
        p.tof_bin_width = 2 * self.tof_range / self.nbins
        p.tof_resolution = self.tof_resolution
        p.tof_log2w = self.tof_log2w.data_ptr()
        p.efficiency = self.eff.data_ptr()
        p.atten_ratio = self.ratio.data_ptr()
        p.pair_warps = int(self.pair_warps)
        p.leg_threads = int(self.leg_threads)
        return p

    def scatter_points(self, p, stream=None):
        """(points [n, 4] float64 CUDA tensor, per-slice counts numpy int64)."""
        L = _lib.lib()
        lz = -(-p.nz // self.sample_step[2])
        cap = (-(-p.nx // self.sample_step[0])) * (-(-p.ny // self.sample_step[1])) * lz
        pts = torch.empty((max(cap, 1), 4), dtype=torch.float64, device=self.device)
        count = C.c_int64(0)
        counts = np.zeros(lz, dtype=np.int64)
        st = C.c_void_p(stream.cuda_stream if stream is not None
                        else torch.cuda.current_stream(self.device).cuda_stream)
        _lib.check(L.sss_scatter_points(C.byref(p), _ptr(pts), cap, C.byref(count),
                                        counts.ctypes.data_as(C.c_void_p), st))
        return pts[:count.value], counts

    def run(self, ActivityMap, AttenuationMap, ImageSize, max_points: int | None = None,
            wave_points: int | None = None, out: torch.Tensor | None = None, stream=None,
            check: bool = True, kahan: bool = False, unit_tof: bool | None = None,
            slice_range=None, points=None) -> torch.Tensor:
        """Sampled scatter sinogram, leg-pair layout [B, NL, NL] float32 (CUDA).

        ``max_points`` restricts the run to the first scatter points in
        lattice order (a partial last slice is normalised over its points,
        like the oracle's bounded samples).  ``points`` (ascending scatter-point
        numbers in lattice order) restricts it to those points, each z-slice
        normalised over its kept points (the oracle's ``points`` sample).
        ``kahan`` selects the precision launch (``SSS_FLAG_KAHAN``): each
        pair's per-point terms summed with Kahan's compensated addition, and
        the TOF offsets formed from float-pair distances and samples."""
        dev = self.device
        shape = tuple(int(s) for s in ActivityMap.shape)
        st = stream if stream is not None else torch.cuda.current_stream(dev)
        with torch.cuda.stream(st):  # the maps' copies are ordered before the launches on st
            act = fortran_flat(ActivityMap, dev)
            mu = fortran_flat(AttenuationMap, dev)
            return self.run_flat(act, mu, shape, ImageSize, max_points, wave_points, out, st, check,
                                 kahan, unit_tof, slice_range, points)

    def run_flat(self, act, mu, shape, ImageSize, max_points: int | None = None,
                 wave_points: int | None = None, out: torch.Tensor | None = None, stream=None,
                 check: bool = True, kahan: bool = False, unit_tof: bool | None = None,
                 slice_range=None, points=None) -> torch.Tensor:
        """``run`` on device-resident maps already flattened in Fortran order
        (float32, Nx*Ny*Nz).  ``slice_range`` = (a, b) keeps the sampled
        z-slices a..b-1 only (a shard: the slice terms add up, :201)."""
        dev = self.device
        st = stream if stream is not None else torch.cuda.current_stream(dev)
        with torch.cuda.stream(st):  # buffers and the status reset belong to the launch stream
            return self._run_on(st, act, mu, shape, ImageSize, max_points, wave_points, out, check, kahan,
                                unit_tof, slice_range, points)

    def _run_on(self, st, act, mu, shape, ImageSize, max_points, wave_points, out, check, kahan, unit_tof,
                slice_range, points=None) -> torch.Tensor:
        dev = self.device
        p = self.problem(act, mu, shape, ImageSize, kahan, unit_tof)
        pts, counts = self.scatter_points(p, st)
        if slice_range is not None:
            # whole sampled z-slices [a, b): the points of the other slices are dropped
            a, b = (int(v) for v in slice_range)
            first = int(counts[:a].sum())
            keep = np.zeros_like(counts)
            keep[a:b] = counts[a:b]
            pts = pts[first:first + int(keep.sum())]
            counts = keep
        if max_points is not None:
            keep = np.minimum(counts, np.maximum(0, max_points - np.concatenate([[0], np.cumsum(counts)[:-1]])))
            counts = keep
            pts = pts[: int(counts.sum())]
        if points is not None:
            pts, counts = select_points(pts, counts, points)
        n = int(counts.sum())
        if out is None:
            out = torch.empty((self.nbins, self.nl, self.nl), dtype=torch.float32, device=dev)
        wave = self.plan_wave(p, counts, wave_points)
        L = _lib.lib()
        need = L.sss_tof_workspace_size(C.byref(p), wave)
        ws = self.workspace(need)
        self._status.zero_()
        _lib.check(L.sss_tof_run(C.byref(p), _ptr(pts), n, counts.ctypes.data_as(C.c_void_p),
                                 len(counts), wave, _ptr(ws), need, _ptr(out), _ptr(self._status),
                                 C.c_void_p(st.cuda_stream)))
        # keep the inputs alive until the stream has consumed them
        self._last = (act, mu, pts)
        if check:
            st.synchronize()
            _lib.check_status(int(self._status.item()))
        return out

    def plan_wave(self, p, counts, wave_points=None) -> int:
        if wave_points is not None:
            return int(max(wave_points, counts.max(initial=0), 1))
        L = _lib.lib()
        per_point = L.sss_tof_workspace_size(C.byref(p), 2) - L.sss_tof_workspace_size(C.byref(p), 1)
        budget = min(WS_BUDGET_BYTES, int(torch.cuda.mem_get_info(self.device)[0] * 0.5))
        fit = max(1, budget // max(per_point, 1))
        total = int(counts.sum())
        return int(max(min(fit, total), counts.max(initial=0), 1))

    def workspace(self, nbytes: int) -> torch.Tensor:
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = None
            self._ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=self.device)
        return self._ws

    # ------------------------------------------------------------------
    def densify_full(self, compact: torch.Tensor, cell_pair: torch.Tensor, out: torch.Tensor,
                     sampled_only: bool = False) -> torch.Tensor:
        """Leg-pair layout -> every element of the reference layout
        [B, ND+1, ND//2, NRU^2] float32, zeros included, into ``out``: a CUDA
        tensor or a page-locked host tensor (written by the GPU over the host
        link, no separate copy).  ``cell_pair``: CUDA int32 table of
        ``geometry.dense_cell_pairs``.  ``sampled_only``: write the cells of
        sampled pairs alone (``sss_tof_densify_cells``), the other cells of
        ``out`` holding zeros already.  Asynchronous on the current stream; a
        table entry out of range is OR-ed into the engine's status word
        (``check_status``)."""
        shape = (self.nbins, self.nd + 1, self.nd // 2, self.nru * self.nru)
        if tuple(out.shape) != shape or out.dtype != torch.float32 or not out.is_contiguous():
            raise ValueError(f"densify_full: out must be contiguous float32 {shape}")
        if not (out.is_cuda or out.is_pinned()):
            raise ValueError("densify_full: out must be a CUDA tensor or page-locked host memory")
        st = torch.cuda.current_stream(self.device)
        fn = _lib.lib().sss_tof_densify_cells if sampled_only else _lib.lib().sss_tof_densify_full
        _lib.check(fn(_ptr(compact), self.nbins, self.nru, self.ndu, self.nd, _ptr(cell_pair), _ptr(out),
                      _ptr(self._status), C.c_void_p(st.cuda_stream)))
        return out

    def densify(self, compact: torch.Tensor, lor, out: torch.Tensor | None = None) -> torch.Tensor:
        """Leg-pair layout -> reference layout [B, ND+1, ND//2, NRU^2] (CUDA).

        ``lor`` is the LORCoordinates table (checked here), or a CUDA int16
        copy of a table checked before.  ``out``: a dense buffer that this
        engine densified into before with the same table (or zeros): only
        the sampled pairs' cells are written, the others stay as they are.
        Asynchronous; a table entry out of range is OR-ed into the engine's
        status word (``check_status``)."""
        dev = self.device
        if isinstance(lor, torch.Tensor) and lor.is_cuda:
            lor_t = lor
        else:
            lor = geometry.check_dense_lor(lor, self.dets_np, self.nd)
            lor_t = as_device(np.asarray(lor, dtype=np.int16), torch.int16, dev)
        shape = (self.nbins, self.nd + 1, self.nd // 2, self.nru * self.nru)
        if out is not None and (tuple(out.shape) != shape or out.dtype != torch.float32 or out.device != dev):
            raise ValueError(f"densify: out must be float32 {shape} on {dev}")
        dense = out if out is not None else torch.zeros(shape, dtype=torch.float32, device=dev)
        st = torch.cuda.current_stream(dev)
        _lib.check(_lib.lib().sss_tof_densify(_ptr(compact), self.nbins, self.nru, self.ndu, self.nd,
                                              _ptr(lor_t), _ptr(self.dets), _ptr(dense), _ptr(self._status),
                                              C.c_void_p(st.cuda_stream)))
        return dense

    def check_status(self):
        """Wait for the current stream, then raise for any error bit of the
        engine's status word (set by ``run`` and by the densify calls since
        the last ``run``)."""
        torch.cuda.current_stream(self.device).synchronize()
        _lib.check_status(int(self._status.item()))


def select_points(pts: torch.Tensor, counts: np.ndarray, points):
    """The scatter points numbered ``points`` (ascending, lattice order) out
    of ``(pts, counts)`` from ``TofSSS.scatter_points``: their rows and the
    per-slice counts of the kept points."""
    idx = np.asarray(points, dtype=np.int64).reshape(-1)
    if len(idx) and (idx[0] < 0 or idx[-1] >= len(pts) or np.any(np.diff(idx) <= 0)):
        raise IndexError("points must be ascending scatter-point numbers below the point count")
    slice_of = np.repeat(np.arange(len(counts)), counts)
    kept = np.bincount(slice_of[idx], minlength=len(counts)).astype(np.int64)
    return pts[torch.from_numpy(idx).to(pts.device)], kept


def leg_pair_to_compact(lp: np.ndarray, nru: int, ndu: int) -> np.ndarray:
    """[B, NL, NL] leg-pair layout (leg = crystal_index*NRU + ring_index) ->
    [B, NRU*NRU, NDU, NDU] (sino = ri1*NRU + ri2, then crystal indices)."""
    b = lp.shape[0]
    x = lp.reshape(b, ndu, nru, ndu, nru).transpose(0, 2, 4, 1, 3)
    return x.reshape(b, nru * nru, ndu, ndu)


def compact_to_leg_pair(cmp: np.ndarray, nru: int, ndu: int) -> np.ndarray:
    """Inverse of ``leg_pair_to_compact``: [B, NRU*NRU, NDU, NDU] -> [B, NL, NL]."""
    b = cmp.shape[0]
    x = cmp.reshape(b, nru, nru, ndu, ndu).transpose(0, 3, 1, 4, 2)
    return np.ascontiguousarray(x.reshape(b, nru * ndu, nru * ndu))
