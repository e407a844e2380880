"""Served scatter updates: continuous batching of TOF-SSS requests on one GPU.

No counterpart in the reference, which runs one SingleScatterSimulationTOF
call per script invocation (Python/openSSS/SingleScatterSimulationTOF.py:36).

Model.  A fixed set of *beds* (bed positions of patients under
reconstruction) stays resident on the device: scanner tables, attenuation map,
base activity map and scatter points (the points depend on the attenuation
only).  A request asks for one outer-iteration scatter update of one bed with
a new activity map (the bed's base activity times 1 +- 5% seeded noise).

``ScatterServer`` serves a stream of timed requests:

* admission: a batch is started only while the device memory of everything
  in flight (workspaces, outputs, per-request activity maps) plus the new
  batch stays under ``hbm_budget`` bytes; waiting requests keep FIFO order
  within their class;
* continuous batching on two streams: waiting small requests are planned
  together into one batch (``BatchSSS``, planned from the cached scatter
  points) and enqueued whole on a high-priority stream, while the current
  large request runs wave by wave on a low-priority stream that is kept
  ``depth`` waves deep.  A small request that arrives while large work is on
  the GPU is admitted at once (memory permitting): its kernels are queued
  beside the large waves and the block scheduler gives them the
  multiprocessors that the large kernels free, so the two overlap on the
  device instead of taking turns;
* completion times are GPU timestamps (CUDA events against one start event).

``PlainServer`` is the reference-style baseline: requests in arrival order,
each through ``TofSSS.run_flat`` (one problem per call).
"""

from __future__ import annotations

import collections
import dataclasses
import time

import numpy as np
import torch

from . import _lib
from .batch import BatchSSS
from .engine import WS_BUDGET_BYTES, TofSSS, fortran_flat


@dataclasses.dataclass
class Bed:
    """One resident problem."""
    engine: TofSSS
    mu: torch.Tensor            # flat, Fortran order
    activity: torch.Tensor      # base activity, flat, Fortran order
    shape: tuple
    image_size: np.ndarray
    points: torch.Tensor        # scatter points [n, 4]
    counts: np.ndarray          # points per sampled z-slice
    units: int                  # scatter points x detector pairs x bins
    leg_bytes: int              # leg records of all scatter points
    large: bool = False


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float              # seconds after the stream starts
    bed: int
    seed: int
    done: float = float("nan")  # completion, seconds after the stream starts
    out: torch.Tensor | None = None

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def make_bed(engine: TofSSS, activity, attenuation, image_size, large: bool = False) -> Bed:
    dev = engine.device
    shape = tuple(int(s) for s in np.shape(activity))
    act = fortran_flat(activity, dev)
    mu = fortran_flat(attenuation, dev)
    p = engine.problem(act, mu, shape, image_size)
    pts, counts = engine.scatter_points(p)
    nru, ndu, nl = engine.nru, engine.ndu, engine.nl
    pairs = nru * nru * ndu * (ndu - 1) // 2 + ndu * nru * (nru - 1)
    cap = sum(shape)
    n = int(counts.sum())
    return Bed(engine, mu, act, shape, np.asarray(image_size, dtype=np.float64), pts, counts,
               n * pairs * engine.nbins, n * nl * (48 + 8 * cap), large)


def request_activity(bed: Bed, seed: int) -> torch.Tensor:
    """The bed's base activity times (1 + u), u uniform in [-5%, +5%] per
    voxel, drawn from ``seed`` on the device."""
    g = torch.Generator(device=bed.activity.device)
    g.manual_seed(int(seed))
    u = torch.rand(bed.activity.shape, generator=g, device=bed.activity.device, dtype=torch.float32)
    return bed.activity * (1.0 + 0.05 * (2.0 * u - 1.0))


def poisson_stream(rate_hz: float, seconds: float, beds: list[Bed], small_fraction: float, seed: int):
    """Seeded Poisson arrivals; each request picks its size class (small with
    probability small_fraction) and then a bed of that class uniformly."""
    rng = np.random.default_rng(seed)
    small = [i for i, b in enumerate(beds) if not b.large]
    large = [i for i, b in enumerate(beds) if b.large]
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= seconds:
            return out
        pool = small if (rng.uniform() < small_fraction or not large) else large
        out.append(Request(len(out), t, int(pool[rng.integers(len(pool))]), int(rng.integers(1 << 31))))


class _Batch:
    def __init__(self, reqs, plan: BatchSSS, nbytes: int, large: bool):
        self.reqs = reqs
        self.plan = plan
        self.nbytes = nbytes
        self.large = large
        self.next_wave = 0
        self.done_event = None
        self.acts = None


class ScatterServer:
    def __init__(self, beds: list[Bed], hbm_budget: int = 80 << 30, depth: int = 2,
                 large_workspace: int = WS_BUDGET_BYTES, max_small_batch: int = 64):
        self.beds = beds
        self.dev = beds[0].engine.device
        self.budget = int(hbm_budget)
        self.depth = depth
        self.large_ws = int(large_workspace)
        self.max_small = max_small_batch
        # lower numbers are higher priorities; the small batches' stream gets the highest
        lo_prio, hi_prio = torch.cuda.Stream.priority_range()
        self.compute = torch.cuda.Stream(self.dev, priority=lo_prio)
        self.small = torch.cuda.Stream(self.dev, priority=hi_prio)
        self.planning = torch.cuda.Stream(self.dev)
        self.resident = sum(b.mu.numel() * 8 + b.points.numel() * 8 for b in beds)
        self.stats = collections.Counter()

    # -- sizes ---------------------------------------------------------
    def _out_bytes(self, r: Request) -> int:
        e = self.beds[r.bed].engine
        return 4 * e.nbins * e.nl * e.nl + 4 * self.beds[r.bed].activity.numel()

    def _workspace(self, reqs, large: bool) -> int:
        need = sum(self.beds[r.bed].leg_bytes for r in reqs) + (1 << 24) * len(reqs)
        return min(need, self.large_ws) if large else need

    # -- batches -------------------------------------------------------
    def _start(self, reqs, large: bool, in_flight: int, stream=None) -> _Batch | None:
        ws_bytes = self._workspace(reqs, large)
        nbytes = ws_bytes + sum(self._out_bytes(r) for r in reqs)
        if self.resident + in_flight + nbytes > self.budget:
            return None
        with torch.cuda.stream(self.planning):
            acts = [request_activity(self.beds[r.bed], r.seed) for r in reqs]
            for r in reqs:
                e = self.beds[r.bed].engine
                r.out = torch.empty((e.nbins, e.nl, e.nl), dtype=torch.float32, device=self.dev)
            ws = torch.empty(ws_bytes, dtype=torch.uint8, device=self.dev)
            jobs = [(self.beds[r.bed].engine, a, self.beds[r.bed].mu, self.beds[r.bed].image_size,
                     self.beds[r.bed].shape) for r, a in zip(reqs, acts)]
            pts = [(self.beds[r.bed].points, self.beds[r.bed].counts) for r in reqs]
            plan = BatchSSS(jobs, stream=self.planning, points=pts, workspace=ws, outs=[r.out for r in reqs])
            ready = torch.cuda.Event()
            ready.record(self.planning)
        (stream or self.compute).wait_event(ready)
        b = _Batch(reqs, plan, nbytes, large)
        b.acts = acts
        self.stats["batches_large" if large else "batches_small"] += 1
        return b

    def _enqueue_wave(self, b: _Batch, waves_in_queue: collections.deque, stream=None):
        st = stream or self.compute
        b.plan.run_waves(b.next_wave, 1, stream=st)
        b.next_wave += 1
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(st)
        waves_in_queue.append(ev)
        if b.next_wave == b.plan.waves:
            b.done_event = ev
        self.stats["waves"] += 1

    def _enqueue_all(self, b: _Batch, waves_in_queue: collections.deque, stream=None):
        st = stream or self.compute
        while b.next_wave < b.plan.waves:
            self._enqueue_wave(b, waves_in_queue, st)
        if b.done_event is None:  # no scatter points: nothing to run
            b.plan.run_waves(0, 0, stream=st)
            b.done_event = torch.cuda.Event(enable_timing=True)
            b.done_event.record(st)

    def serve(self, requests: list[Request]) -> list[Request]:
        """Serve ``requests`` (sorted by arrival) in real time; returns them
        with ``done`` and ``out`` set.  Raises on any device error."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        small_q, large_q = collections.deque(), collections.deque()
        running_small: list[_Batch] = []
        current_large: _Batch | None = None
        in_flight: list[_Batch] = []
        retired: list[torch.Tensor] = []  # status words of finished batches
        queue: collections.deque = collections.deque()        # large waves on self.compute
        small_queue: collections.deque = collections.deque()  # small batches' waves on self.small
        start = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(self.dev)
        start.record(self.compute)
        self.small.wait_event(start)
        t0 = time.perf_counter()
        i, finished = 0, 0
        while finished < len(reqs):
            now = time.perf_counter() - t0
            while i < len(reqs) and reqs[i].arrival <= now:
                (large_q if self.beds[reqs[i].bed].large else small_q).append(reqs[i])
                i += 1
            # retire finished batches (their status words are read at the end:
            # a read now would wait for the whole queue)
            for b in list(in_flight):
                if b.done_event is not None and b.done_event.query():
                    t_done = start.elapsed_time(b.done_event) / 1e3
                    for r in b.reqs:
                        r.done = t_done
                    in_flight.remove(b)
                    retired.append(b.plan.status)
                    b.plan.close()  # the workspace goes back to the allocator
                    b.plan = None
                    if current_large is b:
                        current_large = None
                    finished += len(b.reqs)
            while queue and queue[0].query():
                queue.popleft()
            while small_queue and small_queue[0].query():
                small_queue.popleft()
            used = sum(b.nbytes for b in in_flight)
            # small requests: admitted at once into the high-priority stream,
            # beside whatever large work is queued
            if small_q and len(small_queue) < self.depth:
                n = min(len(small_q), self.max_small)
                b = None
                while n >= 1:
                    take = [small_q.popleft() for _ in range(n)]
                    b = self._start(take, False, used, self.small)
                    if b is not None:
                        break
                    small_q.extendleft(reversed(take))
                    n //= 2  # a smaller batch may fit where this one does not
                if b is None:
                    if not in_flight:
                        raise MemoryError("a small request does not fit the HBM budget")
                else:
                    in_flight.append(b)
                    self._enqueue_all(b, small_queue, self.small)
                    continue
            if len(queue) < self.depth:
                if current_large is not None and current_large.next_wave < current_large.plan.waves:
                    self._enqueue_wave(current_large, queue)
                    continue
                if large_q:
                    take = [large_q.popleft()]
                    b = self._start(take, True, used)
                    if b is None:
                        if not in_flight:
                            raise MemoryError("a large request does not fit the HBM budget")
                        large_q.extendleft(take)
                    else:
                        in_flight.append(b)
                        current_large = b
                        if b.plan.waves == 0:
                            self._enqueue_all(b, queue)
                        else:
                            self._enqueue_wave(b, queue)
                        continue
            if i < len(reqs) or in_flight:
                time.sleep(5e-5)
        torch.cuda.synchronize(self.dev)
        for status in retired:
            _lib.check_status(int(status.item()))
        return reqs


class PlainServer:
    """One request at a time, in arrival order, through TofSSS.run_flat."""

    def __init__(self, beds: list[Bed]):
        self.beds = beds
        self.dev = beds[0].engine.device

    def serve(self, requests: list[Request]) -> list[Request]:
        reqs = sorted(requests, key=lambda r: r.arrival)
        st = torch.cuda.current_stream(self.dev)
        start = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(self.dev)
        start.record(st)
        t0 = time.perf_counter()
        for r in reqs:
            wait = r.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            bed = self.beds[r.bed]
            act = request_activity(bed, r.seed)
            r.out = bed.engine.run_flat(act, bed.mu, bed.shape, bed.image_size, check=True)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(st)
            ev.synchronize()
            r.done = start.elapsed_time(ev) / 1e3
            bed.engine._ws = None
        return reqs


def latency_summary(reqs: list[Request], beds: list[Bed]) -> dict:
    lat = np.array([r.latency for r in reqs])
    small = np.array([r.latency for r in reqs if not beds[r.bed].large])
    large = np.array([r.latency for r in reqs if beds[r.bed].large])
    makespan = max(r.done for r in reqs) - min(r.arrival for r in reqs)
    units = sum(beds[r.bed].units for r in reqs)

    def pct(a, q):
        return float(np.percentile(a, q) * 1e3) if len(a) else None

    return {"requests": len(reqs), "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
            "small_p50_ms": pct(small, 50), "small_p99_ms": pct(small, 99),
            "large_p50_ms": pct(large, 50), "large_p99_ms": pct(large, 99),
            "makespan_s": makespan, "requests_per_s": len(reqs) / makespan, "units_per_s": units / makespan}
