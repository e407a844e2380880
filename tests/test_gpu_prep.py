"""GPU image preparation (sss_crop_downscale) against the oracle: the
reference's crop window followed by skimage's resize restated on
scipy.ndimage in float64 (oracle/prep.py).  Tolerance: 2e-5 of the largest
output value (the kernels filter and interpolate in FP32)."""

import os

import numpy as np
import pytest
import torch

from conftest import ROOT
from oracle import prep as P
from opensss_gb300 import Utils

pytestmark = pytest.mark.gpu
TOL = 2e-5


def _check(got, ref):
    assert got.shape == ref.shape
    assert np.abs(got.astype(np.float64) - ref).max() <= TOL * np.abs(ref).max()


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "prep.npz"))


@pytest.mark.parametrize("case", range(4))
def test_crop_and_downscale_golden_cases(cuda_ok, golden, case):
    img = golden[f"case{case}_image"]
    a = golden[f"case{case}_args"]
    vox, crop, dims = a[:3], a[3:6], a[6:9].astype(int)
    got = Utils.CropAndDownscale(img, vox, crop, dims)
    ref = P.resize(golden[f"case{case}_cropped"].astype(np.float64), tuple(dims))
    _check(got, ref)


@pytest.mark.parametrize("shape,vox,crop,dims", [
    ((128, 128, 80), (2.0, 2.0, 2.5), (256.0, 220.0, 200.0), (32, 28, 20)),   # factor 4: sigma 1.5
    ((160, 150, 90), (1.0, 1.0, 2.0), (160.0, 150.0, 180.0), (20, 25, 45)),   # factors 8, 6, 2
    ((64, 70, 33), (3.0, 3.0, 3.0), (300.0, 120.0, 99.0), (50, 40, 11)),      # padded x, sliced y, odd z
])
def test_crop_and_downscale_against_oracle(cuda_ok, shape, vox, crop, dims):
    rng = np.random.default_rng(sum(shape))
    img = (rng.gamma(2.0, 1.0, size=shape) - 0.3).astype(np.float32)
    got = Utils.CropAndDownscale(img, vox, crop, dims)
    ref = P.crop_and_downscale(img.astype(np.float64), vox, crop, dims)
    _check(got, ref)
    # the tensor path gives the same result on the device
    t = Utils.CropAndDownscale(torch.from_numpy(img).cuda(), vox, crop, dims)
    assert t.is_cuda and np.array_equal(t.cpu().numpy(), got)


def test_without_antialiasing_and_clipping(cuda_ok):
    rng = np.random.default_rng(5)
    img = (rng.random((48, 40, 36)) * 2 - 1).astype(np.float32)
    got = Utils.CropAndDownscale(img, (1, 1, 1), (48, 40, 36), (12, 20, 9), anti_aliasing=False, clip=False)
    ref = P.resize(img.astype(np.float64), (12, 20, 9), anti_aliasing=False, clip=False)
    _check(got, ref)


def test_prepare_images_matches_oracle(cuda_ok, golden, tmp_path):
    act, atn, scale = golden["prep_act"], golden["prep_atn"], golden["prep_scale"]
    names = []
    for name, img in (("act", act), ("atn", atn)):
        with open(tmp_path / f"{name}.hdr", "w") as f:
            f.write(f"name of data file := {name}.img\n")
            for i, (n, s) in enumerate(zip(img.shape, scale)):
                f.write(f"matrix size [{i + 1}] := {n}\nscaling factor (mm/pixel) [{i + 1}] := {s}\n")
        img.transpose(2, 1, 0).tofile(tmp_path / f"{name}.img")
        names.append(str(tmp_path / f"{name}.hdr"))
    size_in = [float(v) if np.isfinite(v) else None for v in golden["prep_size_desired_in"]]
    a, m, sd, dd = Utils.PrepareImages(names[0], names[1], size_in, golden["prep_scale_desired"])
    assert np.array_equal(dd, golden["prep_dims_desired"]) and np.allclose(sd, golden["prep_size_desired"])
    _check(a, P.resize(golden["prep_act_cropped"].astype(np.float64), tuple(dd)))
    ref_m = P.resize(P.crop(atn, scale, sd).astype(np.float64), tuple(dd))
    ref_m[ref_m < 0.001] = 0
    # values within the tolerance of the 0.001 threshold may land on either side
    near = np.abs(ref_m - 0.001) <= TOL * np.abs(ref_m).max()
    assert np.abs(np.where(near, 0, m - ref_m)).max() <= TOL * np.abs(ref_m).max()
