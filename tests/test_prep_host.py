"""Image preparation on the host: the crop window and PrepareImages' sizes
against the reference's own outputs (tests/golden/prep.npz, made by running
Utils.CropAndDownscale / PrepareImages with a recording identity resize), and
the resize algorithm of the GPU kernels — 12 edge samples, a mirror-started
recursive spline filter, unclamped grid-mode coordinates — in float64 numpy
against scipy.ndimage as the oracle calls it."""

import os

import numpy as np
import pytest

from conftest import ROOT
from oracle import prep as P
from opensss_gb300 import Utils


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "prep.npz"))


def _apply_window(img, win):
    """The crop kernel's rule: out[i] = img[i - before + start] inside the image, else 0."""
    out = np.zeros(tuple(w[2] for w in win), dtype=img.dtype)
    idx = []
    for d, (start, before, length) in enumerate(win):
        src = np.arange(length) - before + start
        idx.append(src)
    ok = [(s >= 0) & (s < img.shape[d]) for d, s in enumerate(idx)]
    sub = img[np.ix_(*[s[o] for s, o in zip(idx, ok)])]
    out[np.ix_(*[np.nonzero(o)[0] for o in ok])] = sub
    return out


@pytest.mark.parametrize("case", range(4))
def test_crop_window_matches_reference(golden, case):
    img = golden[f"case{case}_image"]
    a = golden[f"case{case}_args"]
    vox, crop, dims = a[:3], a[3:6], a[6:9]
    ref = golden[f"case{case}_cropped"]
    win = Utils.crop_window(img.shape, vox, crop)
    assert tuple(w[2] for w in win) == ref.shape
    assert np.array_equal(_apply_window(img, win), ref)
    assert np.array_equal(P.crop(img, vox, crop), ref)  # the oracle's own restatement
    assert tuple(golden[f"case{case}_out_shape"]) == tuple(int(d) for d in dims)


def test_reference_resize_options(golden):
    # the options the reference passes to skimage.transform.resize, which the
    # GPU path and the oracle implement
    for case in range(4):
        kw = set(golden[f"case{case}_resize_kwargs"])
        assert kw == {"anti_aliasing=True", "clip=True", "mode=edge", "order=3", "preserve_range=True"}


def test_prepare_images_sizes_and_loading(golden, tmp_path):
    size_in = [float(v) if np.isfinite(v) else None for v in golden["prep_size_desired_in"]]
    act = golden["prep_act"]
    sd, dd = Utils.desired_size(size_in, golden["prep_scale_desired"], np.array(act.shape), golden["prep_scale"])
    assert np.array_equal(dd, golden["prep_dims_desired"])
    assert np.allclose(sd, golden["prep_size_desired"], rtol=0, atol=0)
    assert size_in[2] == act.shape[2] * golden["prep_scale"][2]  # the caller's list is filled in
    for shp in golden["prep_resize_shapes"]:
        assert tuple(shp) == tuple(dd)
    # LoadImage on an interfile pair written as the reference reads it
    nx, ny, nz = act.shape
    with open(tmp_path / "a.hdr", "w") as f:
        f.write("name of data file := a.img\n")
        for i, (n, s) in enumerate(zip(act.shape, golden["prep_scale"])):
            f.write(f"matrix size [{i + 1}] := {n}\nscaling factor (mm/pixel) [{i + 1}] := {s}\n")
    act.transpose(2, 1, 0).tofile(tmp_path / "a.img")
    img, size, scale = Utils.LoadImage(str(tmp_path / "a.hdr"))
    assert np.array_equal(img, act) and tuple(size) == act.shape and np.allclose(scale, golden["prep_scale"])
    # the reference's crop + threshold of the same maps, by the oracle's crop
    win_a = P.crop(act, golden["prep_scale"], golden["prep_size_desired"])
    assert np.array_equal(win_a, golden["prep_act_cropped"])
    atn = P.crop(golden["prep_atn"], golden["prep_scale"], golden["prep_size_desired"]).copy()
    atn[atn < 0.001] = 0
    assert np.array_equal(atn, golden["prep_atn_cropped_thresholded"])


# ---- the kernels' resize algorithm in float64 (the arithmetic prep.cu does in FP32)

_Z = np.sqrt(3.0) - 2.0


def _spline_line(s):
    n = len(s)
    c = 6.0 * s
    k = min(n, 28)
    cp = np.empty(n)
    cp[0] = np.dot(_Z ** np.arange(k), c[:k])
    for i in range(1, n):
        cp[i] = c[i] + _Z * cp[i - 1]
    cm = np.empty(n)
    cm[-1] = _Z / (_Z * _Z - 1.0) * (cp[-1] + _Z * cp[-2])
    for i in range(n - 2, -1, -1):
        cm[i] = _Z * (cm[i + 1] - cp[i])
    return cm


def _kernel_resize(img, out_shape, anti_aliasing=True):
    f = img.astype(np.float64)
    if anti_aliasing:
        sig = Utils.antialias_sigma(img.shape, out_shape)
        for d in range(3):
            if sig[d] <= 1e-15:
                continue
            r = int(4.0 * sig[d] + 0.5)
            x = np.arange(-r, r + 1)
            w = np.exp(-0.5 / sig[d] ** 2 * x * x)
            w /= w.sum()
            idx = np.clip(np.arange(img.shape[d])[:, None] + x[None, :], 0, img.shape[d] - 1)
            f = np.moveaxis(np.tensordot(np.moveaxis(f, d, 0)[idx], w, axes=([1], [0])), 0, d)
    c = np.pad(f, 12, mode="edge")
    for d in range(3):
        c = np.apply_along_axis(_spline_line, d, c)
    taps = []
    for d in range(3):
        n, m = img.shape[d], out_shape[d]
        x = (np.arange(m) + 0.5) * (n / m) - 0.5
        fl = np.floor(x)
        t = x - fl
        w = np.stack([(1 - t) ** 3, 3 * t ** 3 - 6 * t ** 2 + 4, -3 * t ** 3 + 3 * t ** 2 + 3 * t + 1, t ** 3], 1) / 6
        taps.append(((fl.astype(int) - 1)[:, None] + np.arange(4) + 12, w))
    (i0, w0), (i1, w1), (i2, w2) = taps
    g = c[i0[:, None, None, :, None, None], i1[None, :, None, None, :, None], i2[None, None, :, None, None, :]]
    out = np.einsum("ai,bj,ck,abcijk->abc", w0, w1, w2, g)
    return np.clip(out, img.min(), img.max())


@pytest.mark.parametrize("shape,out_shape", [((30, 26, 20), (8, 7, 5)), ((16, 12, 10), (16, 24, 5)),
                                             ((9, 9, 9), (20, 4, 9)), ((1, 10, 8), (4, 5, 3)),
                                             ((40, 36, 31), (5, 9, 31))])
def test_kernel_algorithm_matches_oracle(shape, out_shape):
    rng = np.random.default_rng(sum(shape))
    img = (rng.random(shape) * 3.0).astype(np.float64)
    ref = P.resize(img, out_shape)
    got = _kernel_resize(img, out_shape)
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_unsupported_options_raise_before_device_work():
    img = np.zeros((4, 4, 4), np.float32)
    with pytest.raises(NotImplementedError):
        Utils.CropAndDownscale(img, (1, 1, 1), (4, 4, 4), (2, 2, 2), mode="constant")
    with pytest.raises(NotImplementedError):
        Utils.CropAndDownscale(img, (1, 1, 1), (4, 4, 4), (2, 2, 2), order=1)


def test_crop_window_matches_oracle_on_random_windows():
    """The host window rule against the oracle's literal numpy slicing/padding
    for windows that crop, pad, overhang one end or start at a negative index."""
    rng = np.random.default_rng(21)
    for _ in range(200):
        shape = tuple(int(v) for v in rng.integers(1, 23, size=3))
        vox = rng.uniform(0.5, 4.0, size=3).round(2)
        crop = rng.uniform(0.0, 2.5, size=3) * np.array(shape) * vox
        img = rng.random(shape).astype(np.float32)
        win = Utils.crop_window(shape, vox, crop)
        ref = P.crop(img, vox, crop)
        assert tuple(w[2] for w in win) == ref.shape
        if ref.size:
            assert np.array_equal(_apply_window(img, win), ref)


def test_host_tensors_are_rejected_before_device_work():
    import torch

    with pytest.raises(ValueError):
        Utils.CropAndDownscale(torch.zeros((4, 4, 4)), (1, 1, 1), (4, 4, 4), (2, 2, 2))
    with pytest.raises(ValueError):
        Utils.crop_downscale_device(torch.zeros((4, 4, 4)), Utils.crop_window((4, 4, 4), (1, 1, 1), (4, 4, 4)),
                                    (2, 2, 2))
