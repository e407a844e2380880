"""The C ABI library loads and exports every declared symbol (no GPU needed)."""

import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(sss_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from opensss_gb300 import _lib

    return _lib.lib()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert "sss_tof_run" in names and "sss_raytrace" in names
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    from opensss_gb300 import _lib

    assert set(_declared()) <= set(_lib.SIGNATURES)


def test_abi_version(lib):
    assert lib.sss_abi_version() == 7


def test_invalid_arguments_fail_before_any_device_work(lib):
    from opensss_gb300 import _lib

    grid = np.array([4, 4, 4], np.int32)
    bad = np.array([1.0, 0, 0, 0, 1, 1])  # xMax < xMin
    rc = lib.sss_raytrace(grid.ctypes.data_as(C.c_void_p), bad.ctypes.data_as(C.c_void_p), None, 0,
                          0, 12, C.c_void_p(8), None, None, C.c_void_p(8), None, None, None)
    assert rc == 1
    assert "bounds" in _lib.last_error()
    ok = np.array([0.0, 0, 0, 1, 1, 1])
    rc = lib.sss_raytrace(grid.ctypes.data_as(C.c_void_p), ok.ctypes.data_as(C.c_void_p), None, 0,
                          0, 11, C.c_void_p(8), None, None, C.c_void_p(8), None, None, None)
    assert rc == 8  # capacity below Nx+Ny+Nz
    rc = lib.sss_raytrace(grid.ctypes.data_as(C.c_void_p), ok.ctypes.data_as(C.c_void_p), None, 0,
                          2, 12, C.c_void_p(8), None, None, C.c_void_p(8), None, None, None)
    assert rc == 1
    # the densify calls need a status word for their table checks
    fake = C.c_void_p(8)
    assert lib.sss_tof_densify(fake, 1, 2, 2, 8, fake, fake, fake, None, None) == 1
    assert lib.sss_tof_densify_full(fake, 1, 2, 2, 8, fake, fake, None, None) == 1
    plan = C.c_void_p(0)
    rc = lib.sss_batch_plan(None, 0, None, None, 0, None, C.byref(plan), None)
    assert rc == 1 and not plan.value
    assert lib.sss_batch_run(None, None) == 1
    lib.sss_batch_free(None)


def test_status_codes(lib):
    from opensss_gb300 import _lib

    assert lib.sss_status_code(0) == 0
    assert lib.sss_status_code(1) == 3
    assert "IndexError" in _lib.last_error()
    assert lib.sss_status_code(2) == 4
    assert lib.sss_status_code(1 << 7) == 11  # a caller's index table out of range
    assert "table" in _lib.last_error()
    with pytest.raises(_lib.SSSError):
        _lib.check_status(1)


def test_problem_validation(lib):
    from opensss_gb300 import _lib

    p = _lib.TofProblem()
    assert lib.sss_tof_workspace_size(C.byref(p), 10) == 0
    rc = lib.sss_tof_run(C.byref(p), None, 0, None, 0, 1, None, 0, None, None, None)
    assert rc == 1


def _fake_problem(nx=8, ny=8, nz=4):
    """A problem that passes validation; its pointers are never dereferenced
    by the argument checks under test."""
    from opensss_gb300 import _lib

    p = _lib.TofProblem()
    p.nx, p.ny, p.nz = nx, ny, nz
    for f in ("activity", "attenuation", "geometry", "normals", "rings", "detectors", "tof_log2w", "efficiency",
              "atten_ratio"):
        setattr(p, f, 8)
    p.image_size[:] = [-1, -1, -1, 1, 1, 1]
    p.nr, p.nd, p.nru, p.ndu = 4, 16, 2, 4
    p.sample_step[:] = [2, 2, 2]
    p.nbins = 1
    return p


def test_slice_counts_are_checked_before_any_device_work(lib):
    from opensss_gb300 import _lib

    p = _fake_problem()
    fake = C.c_void_p(8)
    neg = np.array([5, -2], np.int64)
    rc = lib.sss_tof_run(C.byref(p), fake, 3, neg.ctypes.data_as(C.c_void_p), 2, 8, None, 0, fake, fake, None)
    assert rc == 1 and "negative" in _lib.last_error()
    # no point and no count array, but slices announced
    rc = lib.sss_tof_run(C.byref(p), None, 0, None, 2, 8, None, 0, fake, fake, None)
    assert rc == 1
    # a lattice slice of this problem holds 4 x 4 points
    too_many = np.array([17, 0], np.int64)
    pts = (C.c_void_p * 1)(8)
    cts = (C.c_void_p * 1)(too_many.ctypes.data)
    outs = (C.c_void_p * 1)(8)
    plan = C.c_void_p(0)
    rc = lib.sss_batch_plan_points(C.byref(p), 1, C.cast(outs, C.c_void_p), C.cast(pts, C.c_void_p),
                                   C.cast(cts, C.c_void_p), fake, 1 << 20, fake, C.byref(plan), None)
    assert rc == 1 and "slice 0 has 17 points" in _lib.last_error() and not plan.value


def test_no_cpu_fallback_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from opensss_gb300 import RayTracing3DTOF, _lib

    with pytest.raises(_lib.EngineUnavailable):
        RayTracing3DTOF(np.array([4, 4, 4]), np.array([0.0, 0, 0, 1, 1, 1]),
                        np.array([-1.0, 0.5, 0.5, 2, 0.5, 0.5]))


def test_crop_downscale_rejects_bad_arguments_without_device_work(lib):
    from opensss_gb300 import _lib

    dims = np.array([8, 8, 8], np.int32)
    zero = np.zeros(3, np.int32)
    sigma = np.zeros(3)

    def p(a):
        return a.ctypes.data_as(C.c_void_p)

    assert lib.sss_crop_downscale_workspace_size(p(np.array([0, 4, 4], np.int32))) == 0
    assert lib.sss_crop_downscale_workspace_size(p(dims)) > 0
    rc = lib.sss_crop_downscale(None, p(dims), p(zero), p(zero), p(dims), p(dims), p(sigma), 1, C.c_float(0),
                                C.c_void_p(8), C.c_void_p(8), 1 << 30, None)
    assert rc == 1 and "null" in _lib.last_error()
    rc = lib.sss_crop_downscale(C.c_void_p(8), p(dims), p(zero), p(zero), p(np.array([8, 0, 8], np.int32)), p(dims),
                                p(sigma), 1, C.c_float(0), C.c_void_p(8), C.c_void_p(8), 1 << 30, None)
    assert rc == 1 and "empty" in _lib.last_error()
    rc = lib.sss_crop_downscale(C.c_void_p(8), p(dims), p(zero), p(zero), p(dims), p(dims), p(sigma), 1,
                                C.c_float(0), C.c_void_p(8), C.c_void_p(8), 16, None)
    assert rc == 7  # workspace too small


def test_device_wrappers_reject_host_tensors():
    import torch

    from opensss_gb300.BackProjection import fit_bins_device, fit_device
    from opensss_gb300.Datafile import histogram_device
    from opensss_gb300.Interpolation import upsample_device

    host = torch.zeros(4)
    with pytest.raises(ValueError):
        upsample_device(host, (np.zeros(1, np.int64), np.zeros(1, np.int64), 1), 1, 1, 1)
    with pytest.raises(ValueError):
        fit_device(host, host, host, host, None, None, [1, 1, 1], [0, 0, 0, 1, 1, 1], np.zeros((1, 2, 3)),
                   None, None, 1)
    with pytest.raises(ValueError):
        fit_bins_device(host, host, host, host, 1, None, None, [1, 1, 1], [0, 0, 0, 1, 1, 1],
                        np.zeros((1, 2, 3)), None, None, 1)
    with pytest.raises(ValueError):
        histogram_device(host, {}, np.zeros((2, 2, 2)), np.zeros((1, 1)), 1, 1000.0)
