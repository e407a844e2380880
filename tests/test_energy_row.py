"""The pair kernel's scattered-energy row (``walk_task`` and
``energy_row_pair`` in ``opensss_gb300/csrc/pair.cuh``), emulated in numpy
float32, against the reference's FP64 evaluation (law of cosines,
``SingleScatterSimulationTOF.py:442-444, :216-235, :495-501``) on seeded legs of
the 760-crystal ring: every row the FP32 stage or the float-pair stage
decides equals the FP64 row; the FP32 stage leaves about one pair in 500 to
the float pairs, and they defer to FP64 for about one in a million."""

import numpy as np

F = np.float32


def _fma(a, b, c):
    # a*b is exact in float64 for float32 inputs; one rounding to float32 after
    # the add (double rounding only matters for terms far below the result)
    return F(np.float64(a) * np.float64(b) + np.float64(c))


def _split(u):
    hi = u.astype(F)
    return hi, (u - hi.astype(np.float64)).astype(F)


def _row_pair(bw, cw, bp, cp):
    """Operation for operation as energy_row_pair (vectorised over pairs)."""
    with np.errstate(all="ignore"):
        p = [bw[:, k] * bp[:, k] for k in range(3)]
        r = (_fma(bw[:, 0], bp[:, 0], -p[0]) + _fma(bw[:, 1], bp[:, 1], -p[1])) + _fma(bw[:, 2], bp[:, 2], -p[2])
        s = p[0] + p[1]
        v = s - p[0]
        t = (p[0] - (s - v)) + (p[1] - v)
        s2 = s + p[2]
        v = s2 - s
        t = t + ((s - (s2 - v)) + (p[2] - v))
        cross = _fma(bw[:, 0], cp[:, 0], _fma(cw[:, 0], bp[:, 0], _fma(bw[:, 1], cp[:, 1], _fma(
            cw[:, 1], bp[:, 1], _fma(bw[:, 2], cp[:, 2], cw[:, 2] * bp[:, 2])))))
        ql = (t + r) + cross
        qc = np.clip(s2 + ql, F(-1), F(1))
        dh = F(2) + s2
        v = dh - F(2)
        dl = ((F(2) - (dh - v)) + (s2 - v)) + ql
        d1 = dh + dl
        dl = dl - (d1 - dh)
        dh = d1
        y = (np.float64(511) / dh.astype(np.float64)).astype(F)
        el = ((_fma(-y, dh, F(511)) - y * dl).astype(np.float64) / dh).astype(F)
        n0 = np.floor(y + F(0.5))
        f = (y - (n0 - F(0.5))) + el
        defer = ~((f > F(1e-6)) & (f < F(1) - F(1e-6))) | (np.abs(qc) > F(1) - F(1e-6))
    return np.where(defer, -2, 2 * n0.astype(np.int64) - 1), y.astype(np.float64) + el.astype(np.float64)


def _row_fp32(b1, b2):
    """The first stage of the kernel's row: FP32 from the legs' high floats,
    undecided (-3) within 1e-3 keV of a rounding boundary or near collinear
    legs (the hardware's fast division is within 2 ulps of this one)."""
    with np.errstate(all="ignore"):
        qc = _fma(b1[:, 0], b2[:, 0], _fma(b1[:, 1], b2[:, 1], b1[:, 2] * b2[:, 2]))
        qc = np.clip(qc, F(-1), F(1))
        e = (np.float64(511) / (F(2) + qc).astype(np.float64)).astype(F)
        eh = e + F(0.5)
        fr = eh - np.floor(eh)
        undecided = (fr < F(1e-3)) | (fr > F(1) - F(1e-3)) | (np.abs(qc) > F(1) - F(1e-5))
    return np.where(undecided, -3, 2 * np.floor(eh).astype(np.int64) - 1)


def test_fp32_pair_row_matches_fp64_row():
    rng = np.random.default_rng(5)
    n = 400_000
    phi = 2 * np.pi * rng.integers(0, 760, size=(n, 2)) / 760
    z = (rng.integers(0, 80, size=(n, 2)) - 39.5) * 0.32
    crys = np.stack([41 * np.cos(phi), 41 * np.sin(phi), z], axis=-1)  # [n, 2, 3]
    pts = np.concatenate([rng.uniform(-20, 20, size=(n, 2)), rng.uniform(-12, 12, size=(n, 1))], axis=1)
    # the FP64 row as the reference forms it
    v1, v2 = crys[:, 0] - pts, crys[:, 1] - pts
    sv1, sv2 = np.sqrt((v1 * v1).sum(1)), np.sqrt((v2 * v2).sum(1))
    lor = ((crys[:, 0] - crys[:, 1]) ** 2).sum(1)
    a, b = sv1 * sv1, sv2 * sv2
    q = (a + b - lor) / (2 * np.sqrt(a * b))
    ok = np.abs(q) < 1 - 1e-9
    ref = (np.floor(511 / (1 + (1 + q)) + 0.5) * 2).astype(np.int64) - 1
    # the pair kernel's float pairs of the legs' FP64 unit vectors
    u1, u2 = v1 / sv1[:, None], v2 / sv2[:, None]
    (b1, c1), (b2, c2) = _split(u1), _split(u2)
    got, e = _row_pair(b1, c1, b2, c2)
    decided = (got != -2) & ok
    assert np.array_equal(got[decided], ref[decided])
    assert (got[ok] == -2).mean() < 2e-5
    # the float-pair energy is within 1e-8 keV of the FP64 one: a hundredth of
    # the 1e-6 band inside which the kernel defers to FP64
    assert np.abs(e - 511 / (2 + q))[ok].max() < 1e-8
    # the kernel's first stage, FP32 from the high floats: every row it decides
    # is the FP64 row, and it leaves about one pair in 500 to the float pairs
    first = _row_fp32(b1, b2)
    decided32 = (first != -3) & ok
    assert np.array_equal(first[decided32], ref[decided32])
    assert (first[ok] == -3).mean() < 5e-3
