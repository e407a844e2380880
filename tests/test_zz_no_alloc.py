"""sss_scatter_points_noalloc: the scatter-point step for callers that must
not allocate device memory (code inside a fixed arena it does not own, or a
process whose device memory is capped).

Checked through the C ABI against sss_scatter_points on two calls in a row:
the second call must not see the first call's counts, because every call
shares the library's scratch array and clears it first.  Around each call
the device's free memory and the default stream-ordered pool's use (current
and high-water mark) must not move: the call allocates nothing, not even
briefly.  Kept in the last collected file so a run that stops at the first
failure has run all else."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(pr, att):
    from opensss_gb300 import TofSSS
    from opensss_gb300.engine import fortran_flat

    eng = TofSSS(pr.scanner.geometry, pr.scanner.normals, pr.scanner.detector_size_mm, att,
                 pr.energy_resolution, pr.energy_threshold, pr.nr_rings_used, pr.nr_detectors_used,
                 pr.sample_step, pr.tof_resolution, pr.tof_range, pr.nr_bins)
    act = fortran_flat(pr.activity, eng.device)
    mu = fortran_flat(pr.attenuation, eng.device)
    return eng, act, mu, eng.problem(act, mu, pr.grid, pr.image_size)


# cudaMemPoolAttr values of the CUDA runtime's public header (driver_types.h)
_RESERVED_CURRENT, _USED_CURRENT, _USED_HIGH = 0x5, 0x7, 0x8


class _DeviceMemory:
    """Free device memory (cudaMemGetInfo) and the default pool's reserved,
    used and peak-used bytes, read through the CUDA runtime the engine
    library links (libcudart.so.13, already loaded with it)."""

    def __init__(self, device_index):
        self.rt = C.CDLL("libcudart.so.13")
        self.pool = C.c_void_p()
        assert self.rt.cudaDeviceGetDefaultMemPool(C.byref(self.pool), int(device_index)) == 0

    def _attr(self, which):
        v = C.c_uint64(0)
        assert self.rt.cudaMemPoolGetAttribute(self.pool, which, C.byref(v)) == 0
        return v.value

    def reset_peak(self):
        zero = C.c_uint64(0)
        assert self.rt.cudaMemPoolSetAttribute(self.pool, _USED_HIGH, C.byref(zero)) == 0

    def snapshot(self):
        free, total = C.c_size_t(0), C.c_size_t(0)
        assert self.rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
        return {"free": free.value, "reserved": self._attr(_RESERVED_CURRENT), "used": self._attr(_USED_CURRENT),
                "peak": self._attr(_USED_HIGH)}


def _call(fn, p, cap, lz, device, memory=None):
    import torch

    pts = torch.full((cap, 4), -7.0, dtype=torch.float64, device=device)
    count = C.c_int64(-1)
    slices = np.full(lz, -1, dtype=np.int64)
    st = torch.cuda.current_stream(device)
    torch.cuda.synchronize(device)
    if memory is not None:
        memory.reset_peak()
        before = memory.snapshot()
    rc = fn(C.byref(p), C.c_void_p(pts.data_ptr()), cap, C.byref(count),
            slices.ctypes.data_as(C.c_void_p), C.c_void_p(st.cuda_stream))
    if memory is not None:
        after = memory.snapshot()
        assert after == before, (before, after)
        assert after["peak"] == after["used"]
    return rc, pts.cpu().numpy(), count.value, slices


@pytest.mark.parametrize("which", ["tiny", "tof13_64x64x48"])
def test_noalloc_matches_allocating_entry_point(cuda_ok, att_table, which):
    from opensss_gb300 import _lib, workloads as W

    pr = W.tiny_problem(3, seed=2) if which == "tiny" else W.tof13_64x64x48()
    eng, act, mu, p = _setup(pr, att_table)
    L = _lib.lib()
    lz = -(-pr.grid[2] // int(pr.sample_step[2]))
    cap = (-(-pr.grid[0] // int(pr.sample_step[0]))) * (-(-pr.grid[1] // int(pr.sample_step[1]))) * lz
    rc, ref_pts, ref_n, ref_sl = _call(L.sss_scatter_points, p, cap, lz, eng.device)
    assert rc == 0, _lib.last_error()
    memory = _DeviceMemory(eng.device.index or 0)
    for _ in range(2):  # two calls in a row share the scratch array
        rc, pts, n, sl = _call(L.sss_scatter_points_noalloc, p, cap, lz, eng.device, memory)
        assert rc == 0, _lib.last_error()
        assert n == ref_n
        assert np.array_equal(sl, ref_sl)
        assert np.array_equal(pts[:n], ref_pts[:n])  # same kernel: exact


def test_noalloc_rejects_more_slices_than_its_limit(cuda_ok, att_table):
    from opensss_gb300 import _lib, workloads as W

    pr = W.tiny_problem(1, seed=2)
    pr.activity = np.ones((1, 1, 8200), np.float32)
    pr.attenuation = np.full((1, 1, 8200), 0.1, np.float32)
    pr.image_size = np.array([-1.0, -1.0, -410.0, 1.0, 1.0, 410.0])
    pr.sample_step = np.array([1, 1, 2])  # 4100 sampled slices > 4096
    eng, act, mu, p = _setup(pr, att_table)
    rc, _, _, _ = _call(_lib.lib().sss_scatter_points_noalloc, p, 8200, 4100, eng.device)
    assert rc == 1
    assert "4096" in _lib.last_error()
