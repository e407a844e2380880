"""Many TOF-SSS problems in one schedule (sss_batch_* of libsss300.so).

The reference simulates one problem per SingleScatterSimulationTOF call
(Python/openSSS/SingleScatterSimulationTOF.py:46-178).  ``BatchSSS`` plans a
list of problems once -- scatter points, (problem, z-slice) items, waves that
fit a workspace -- and then runs the whole list as a fixed sequence of
launches.  Activity maps can be replaced in place between runs; the
attenuation maps fix the scatter points and therefore the plan.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .engine import WS_BUDGET_BYTES, TofSSS, _ptr, fortran_flat


def _tune_classes(jobs) -> dict:
    """One autotune per TOF class (bins, bin width, resolution) on its
    largest problem; every engine of the class gets that class's pair shape,
    all engines the leg shape of the class with the most legs."""
    from . import autotune

    classes: dict = {}
    for job in jobs:
        eng = job[0]
        shape = tuple(int(s) for s in (job[4] if len(job) > 4 else np.shape(job[1])))
        key = (eng.nbins, round(eng.tof_range, 6), round(eng.tof_resolution, 6))
        work = eng.nl * int(np.prod(shape))
        if key not in classes or work > classes[key][0]:
            classes[key] = (work, job, shape)
    results, legs_best = {}, (-1, 0)
    for key, (work, job, shape) in classes.items():
        eng, act, mu, size = job[:4]
        flat = len(job) > 4
        r = autotune.tune(eng, act, mu, size, shape=shape if flat else None)
        results[key] = r
        if work > legs_best[0]:
            legs_best = (work, int(r["leg_threads"]))
    for job in jobs:
        eng = job[0]
        key = (eng.nbins, round(eng.tof_range, 6), round(eng.tof_resolution, 6))
        eng.pair_warps = int(results[key]["pair_warps"])
        eng.leg_threads = legs_best[1]
    return {f"bins={k[0]}": {"pair_warps": v["pair_warps"], "leg_threads": v["leg_threads"],
                             "cached": v["cached"]} for k, v in results.items()}


class BatchSSS:
    """A planned batch of TOF-SSS problems.

    jobs: sequence of ``(engine, ActivityMap, AttenuationMap, ImageSize)`` with
    ``engine`` a :class:`TofSSS` (scanner, sampling, tables; engines may be
    shared between jobs).  Maps may be numpy arrays (x, y, z) or CUDA tensors
    already flattened in Fortran order with ``shape`` given as the fifth
    element of the job tuple.
    """

    def __init__(self, jobs, workspace_bytes: int | None = None, stream=None, points=None,
                 workspace: torch.Tensor | None = None, outs=None, autotune: bool = False):
        """``points``: optional per-job ``(points, slice_counts)`` from
        ``TofSSS.scatter_points`` (they depend on the attenuation map only);
        with them the plan skips the scatter-point pass.  ``workspace`` /
        ``outs``: caller-owned device buffers to plan into (otherwise
        allocated here).  ``autotune``: before planning, pick the launch
        shapes of each TOF class on its largest problem
        (:func:`opensss_gb300.autotune.tune`, cached per device and size
        class); the plan's leg launches take the shape of the class with the
        most legs."""
        if not jobs:
            raise ValueError("empty batch")
        L = _lib.lib()
        self.tuned = _tune_classes(jobs) if autotune else None
        self.engines: list[TofSSS] = []
        self.shapes = []
        self._keep = []
        probs = (_lib.TofProblem * len(jobs))()
        dev = jobs[0][0].device
        self.device = dev
        for i, job in enumerate(jobs):
            eng, act, mu, size = job[:4]
            if eng.device != dev:
                raise ValueError("all engines of a batch must be on one device")
            if len(job) > 4:
                shape = tuple(int(s) for s in job[4])
                act_f = act if isinstance(act, torch.Tensor) else fortran_flat(act, dev)
                mu_f = mu if isinstance(mu, torch.Tensor) else fortran_flat(mu, dev)
            else:
                shape = tuple(int(s) for s in np.shape(act))
                act_f, mu_f = fortran_flat(act, dev), fortran_flat(mu, dev)
            probs[i] = eng.problem(act_f, mu_f, shape, size)
            self.engines.append(eng)
            self.shapes.append(shape)
            self._keep.append((act_f, mu_f))
        self.outs = list(outs) if outs is not None else [
            torch.empty((e.nbins, e.nl, e.nl), dtype=torch.float32, device=dev) for e in self.engines]
        out_ptrs = (C.c_void_p * len(jobs))(*[o.data_ptr() for o in self.outs])
        if workspace is None:
            if workspace_bytes is None:
                workspace_bytes = min(WS_BUDGET_BYTES, int(torch.cuda.mem_get_info(dev)[0] * 0.5))
            workspace = torch.empty(int(workspace_bytes), dtype=torch.uint8, device=dev)
        self.workspace = workspace
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._probs = probs
        st = stream if stream is not None else torch.cuda.current_stream(dev)
        plan = C.c_void_p(0)
        if points is None:
            _lib.check(L.sss_batch_plan(probs, len(jobs), C.cast(out_ptrs, C.c_void_p),
                                        _ptr(self.workspace), self.workspace.numel(), _ptr(self.status),
                                        C.byref(plan), C.c_void_p(st.cuda_stream)))
        else:
            counts = [np.ascontiguousarray(c, dtype=np.int64) for _, c in points]
            self._points = (points, counts)
            pts = (C.c_void_p * len(jobs))(*[pt.data_ptr() if pt.numel() else 0 for pt, _ in points])
            cts = (C.c_void_p * len(jobs))(*[c.ctypes.data for c in counts])
            _lib.check(L.sss_batch_plan_points(probs, len(jobs), C.cast(out_ptrs, C.c_void_p),
                                               C.cast(pts, C.c_void_p), C.cast(cts, C.c_void_p),
                                               _ptr(self.workspace), self.workspace.numel(),
                                               _ptr(self.status), C.byref(plan),
                                               C.c_void_p(st.cuda_stream)))
        self._plan = plan
        info = np.zeros(4, dtype=np.int64)
        _lib.check(L.sss_batch_info(plan, info.ctypes.data_as(C.c_void_p)))
        self.waves, self.launches, self.units, self.points = (int(v) for v in info)

    def activity(self, i: int) -> torch.Tensor:
        """Problem i's resident activity map (flat, Fortran order); write into
        it in place to re-run the plan on new activity."""
        return self._keep[i][0]

    def run(self, stream=None, check: bool = True) -> list[torch.Tensor]:
        """Enqueue the whole batch; outputs are the leg-pair sinograms
        [B, NL, NL] of each problem (reused across runs)."""
        if self._plan is None:
            raise RuntimeError("batch plan was freed")
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        if check:
            with torch.cuda.stream(st):  # ordered before the batch's launches
                self.status.zero_()
        _lib.check(_lib.lib().sss_batch_run(self._plan, C.c_void_p(st.cuda_stream)))
        if check:
            st.synchronize()
            _lib.check_status(int(self.status.item()))
        return self.outs

    def run_waves(self, first: int, count: int, stream=None):
        """Enqueue waves [first, first + count) (in order; wave 0 zeroes the
        outputs).  No synchronisation, no status check."""
        if self._plan is None:
            raise RuntimeError("batch plan was freed")
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        _lib.check(_lib.lib().sss_batch_run_waves(self._plan, int(first), int(count),
                                                  C.c_void_p(st.cuda_stream)))

    def capture(self):
        """Record one run in a CUDA graph; ``replay()`` then enqueues the whole
        batch (output zeroing, every wave's leg and pair launches) as one
        graph launch on the current stream."""
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.run(stream=s, check=False)
        torch.cuda.current_stream(self.device).wait_stream(s)
        self._graph = g
        return g

    def replay(self, check: bool = True) -> list[torch.Tensor]:
        if getattr(self, "_graph", None) is None:
            raise RuntimeError("capture() first")
        if check:
            self.status.zero_()
        self._graph.replay()
        if check:
            torch.cuda.current_stream(self.device).synchronize()
            _lib.check_status(int(self.status.item()))
        return self.outs

    def close(self):
        self._graph = None
        if getattr(self, "_plan", None):
            _lib.lib().sss_batch_free(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
