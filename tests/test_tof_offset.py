"""The precision launch's TOF offset (floor_pair in csrc/pair.cuh), emulated
in numpy float32: the floor of u + sigma * rho from float-pair parts is the
floor of the FP64 value (the reference's column, SingleScatterSimulationTOF.py
:520, :526) except within about 1e-9 ps of an integer, where the plain FP32
offset errs within about 1e-3 ps."""

import numpy as np

F = np.float32


def _pair(x):
    hi = x.astype(F)
    return hi, (x - hi.astype(np.float64)).astype(F)


def floor_pair(uh, ul, sigma, rh, rl):
    """Operation for operation as the kernel: a two-sum of uh and sigma*rh,
    the low parts added to its error, floor(s) moved by one where they carry
    the sum across an integer (compared against 1 - f and -f, both exact)."""
    b = (sigma * rh).astype(F)
    s = (uh + b).astype(F)
    bb = (s - uh).astype(F)
    e = ((uh - (s - bb).astype(F)).astype(F) + (b - bb).astype(F)).astype(F)
    low = (e + (sigma * rl + ul).astype(F)).astype(F)
    t = np.floor(s.astype(np.float64))  # the round-down add of 1.5 * 2^23, exact below 2^22
    f = (s - t.astype(F)).astype(F)
    return t.astype(np.int64) + (low >= (F(1) - f).astype(F)).astype(np.int64) - (low < -f).astype(np.int64)


def _cases(n, seed):
    rng = np.random.default_rng(seed)
    sigma = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    rho = rng.uniform(0.0, 5000.0, n)
    # the offset lies within delta of an integer k in 700..7300
    k = rng.integers(700, 7300, n).astype(np.float64)
    delta = np.where(rng.random(n) < 0.5, -1.0, 1.0) * 10.0 ** rng.uniform(-11, -3, n)
    u = k + delta - sigma * rho
    return u, sigma, rho, np.floor(u + sigma * rho), delta


def test_floor_pair_takes_the_fp64_column():
    u, sigma, rho, ref, delta = _cases(400_000, 5)
    uh, ul = _pair(u)
    rh, rl = _pair(rho)
    got = floor_pair(uh, ul, sigma.astype(F), rh, rl)
    # the float pairs hold u and rho to ~2e-11 ps; beyond 1e-9 of an integer the column is sure
    sure = np.abs(delta) > 1e-9
    assert np.array_equal(got[sure], ref[sure])


def test_plain_fp32_offset_takes_the_neighbouring_column_near_boundaries():
    """The plain launch's offset, fmaf(sigma, rho, u) in FP32 from the high
    floats, errs by up to ~8e-4 ps (u reaches 12,000): within 1e-4 ps of a
    boundary it takes the neighbouring column in a good fraction of cases,
    where the float-pair offset never does beyond 1e-9 ps."""
    u, sigma, rho, ref, delta = _cases(400_000, 6)
    x = (u.astype(F) + (sigma * rho.astype(F)).astype(F)).astype(F)  # fmaf(sigma, rho, u) in FP32
    plain = np.floor(x.astype(np.float64))
    near = (np.abs(delta) < 1e-4) & (np.abs(delta) > 1e-9)
    assert (plain[near] != ref[near]).mean() > 0.1
    uh, ul = _pair(u)
    rh, rl = _pair(rho)
    assert np.array_equal(floor_pair(uh, ul, sigma.astype(F), rh, rl)[near], ref[near])
