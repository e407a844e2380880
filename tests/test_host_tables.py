"""Host-side set-up tables of the engine against the reference's outputs."""

import hashlib

import numpy as np
import pytest

from conftest import golden
from opensss_gb300 import geometry as G
from opensss_gb300 import tables as T


@pytest.mark.parametrize("tag", ["b1", "b6", "b13", "b33"])
def test_tof_table_matches_reference(tag):
    g = golden("tables")
    nb, rng, res = g[f"tof_{tag}_params"]
    ref = g[f"tof_{tag}"]
    assert np.array_equal(T.tof_table(int(nb), rng, res)[:, ::3], ref)


@pytest.mark.parametrize("tag", ["b1", "b6", "b13", "b33"])
def test_kernel_tof_weights_reproduce_table(tag):
    """The per-bin weights the kernel rebuilds from (log2 max weight, bin)
    agree with the reference table to FP32 storage precision."""
    g = golden("tables")
    nb, rng, res = g[f"tof_{tag}_params"]
    ref = g[f"tof_{tag}"]
    l2 = T.tof_log2_table(int(nb), rng, res)
    w = T.tof_weights_from_log2(l2, int(nb), rng, res)[:, ::3]
    assert np.abs(w - ref).max() < 5e-8
    assert np.array_equal(w == 0, ref == 0) or np.abs(w[ref == 0]).max() < 1e-30


def test_efficiency_zero_set_matches_reference():
    g = golden("tables")
    att = g["att_table"]
    eff = T.efficiency(att[:, 0], 435.0, 0.12)
    assert np.array_equal(eff, g["eff_435_012"])
    pe = T.pair_efficiency_f32(att, 435.0, 0.12)
    ref_prod = g["eff_435_012"] * g["eff_435_012"][1021]
    assert np.array_equal(pe == 0, ref_prod == 0)


@pytest.mark.parametrize("nd,nr,lk,sk", [(48, 6, "lor48", "sino6"), (64, 10, "lor64", "sino10")])
def test_sinogram_coordinates_small(nd, nr, lk, sk):
    g = golden("sinogram")
    lor, si, shift = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    assert lor.dtype == np.int16 and si.dtype == np.int16 and shift == 0
    assert np.array_equal(lor, g[lk])
    assert np.array_equal(si, g[sk])


def test_sinogram_coordinates_760():
    g = golden("sinogram")
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, 760, 80, ID_Shidt=False)
    assert hashlib.sha256(lor.tobytes()).hexdigest() == str(g["lor760_sha256"])
    assert np.array_equal(lor[0], g["lor760_row0"])
    assert np.array_equal(lor[379], g["lor760_row379"])
    assert np.array_equal(si, g["sino80"])


@pytest.mark.parametrize("ndu", [32, 48, 96])
def test_upsample_source_matches_reference(ndu):
    lut = golden("upsample_lut760")[f"src_ndu{ndu}"]
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, 760, 80, ID_Shidt=False)
    det = G.sampled_detectors(760, ndu)
    src = G.upsample_source(lor, det)
    a, b = np.divmod(src, ndu)
    code = lor[det[a], det[b], 1].astype(np.int64) * 1000 + lor[det[a], det[b], 0]
    assert np.array_equal(code, lut)


def test_ring_nearest_ties_to_lower():
    rings = G.sampled_rings(80, 8)
    m = G.ring_nearest(80, rings)
    assert m[0] == 0 and m[79] == 7
    for r in range(80):
        d = np.abs(rings - r)
        best = np.where(d == d.min())[0]
        assert m[r] == best.min()


def test_sampled_detectors_reference_rule():
    assert G.sampled_detectors(760, 32)[:4].tolist() == [0, 23, 46, 69]
    assert G.sampled_detectors(760, 96)[-1] == 665
    assert G.sampled_rings(80, 16)[[0, -1]].tolist() == [0, 79]


def _legpair_from_compact(cmp, nru, ndu):
    """[B, NRU^2, NDU, NDU] (sino = ri1*NRU + ri2) -> leg-pair [B, NL, NL]."""
    b = cmp.shape[0]
    x = cmp.reshape(b, nru, nru, ndu, ndu).transpose(0, 3, 1, 4, 2)
    return x.reshape(b, ndu * nru, ndu * nru)


@pytest.mark.parametrize("case", range(2))
@pytest.mark.parametrize("layout", ["dense", "legpair"])
def test_upsample_gather_tables_reproduce_reference(case, layout):
    """The gather tables the upsampling kernel reads, applied with numpy,
    reproduce the reference's InterpolateAllBins output exactly."""
    from oracle import oracle as O

    g = golden("upsample")
    nd, nr, nru, ndu, nb = (int(v) for v in g[f"case{case}_dims"])
    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    cmp = g[f"case{case}_compact"]
    if layout == "dense":
        src = O.densify(cmp.astype(np.float64), lor, nd, nru, ndu).astype(np.float32)
    else:
        src = _legpair_from_compact(cmp, nru, ndu)
    t = G.upsample_tables(lor, si, nru, ndu, layout)
    cell, ring, stride = t
    assert np.array_equal(t.ring_off[t.ring_idx], ring)  # the kernel's staged form
    assert len(t.ring_off) <= nru * nru
    flat = src.reshape(-1)
    idx = cell[:, None] + ring[None, :]
    total = np.zeros(idx.shape, np.float32)
    for b in range(nb):
        vb = np.maximum(flat[b * stride + idx], 0)
        assert np.array_equal(vb.reshape(nd + 1, nd // 2, nr * nr), g[f"case{case}_bins"][b])
        total += vb
    assert np.array_equal(total.reshape(nd + 1, nd // 2, nr * nr), g[f"case{case}_sum"])


def test_unit_tof_table_detection():
    """One bin with a 1e6 ps kernel: every normalised weight is exactly 1, so
    the table is all (0, 0) and the engine may use the leg integrals; a real
    timing kernel or more bins never give that form."""
    from opensss_gb300 import tables

    assert not np.any(tables.tof_log2_table(1, 1000.0, 1.0e6))
    assert np.any(tables.tof_log2_table(1, 1000.0, 214.0))
    assert np.any(tables.tof_log2_table(3, 1000.0, 1.0e6))


# ---- the factored TOF weights of the pair kernel, emulated in float32

def _pack_bin(a, n, mask):
    ai = int(np.float32(a).view(np.int32))
    if ai == 0:
        return np.float32(0)
    p = ai - ((ai - n) & mask)
    if ai - p > (mask + 1) // 2 or p < 0:
        p += mask + 1
    return np.int32(p).view(np.float32)


def _factored_weights(nb, rng, res, ca=1.0):
    """The pair kernel's terms ca * w_b, operation for operation in float32,
    divided by ca: the table set-up of load_pair_tables (A with the bin in its
    low bits, r, G rows) and the FFMA2 / FMUL2 chain of accumulate_loaded,
    which starts from ca * A."""
    f32 = np.float32
    ca = f32(ca)
    w = 2 * rng / nb
    kappa = 4.0 / (res * res)
    s0, W, k2w, gam = f32((1.0 - (nb + 1) / 2.0) * w), f32(w), f32(2 * kappa * w), f32(kappa * w * w)
    bits = 1
    while (1 << bits) < nb:
        bits += 1
    mask = (1 << bits) - 1
    l2 = T.tof_log2_table(nb, rng, res).astype(np.float32)
    G = np.array([[np.exp2(f32(f32(-gam * f32(n - b)) * f32(n - b))) for b in range(nb)] for n in range(nb)],
                 np.float32)
    out = np.zeros((nb, 8001))
    with np.errstate(all="ignore"):
        for i in range(8001):
            Y, n = l2[i, 0], int(l2[i, 1])
            beta = f32(k2w * f32(f32(i - 4000) - f32(np.float64(n) * np.float64(W) + np.float64(s0))))
            e = np.float64(Y) - np.float64(n) * np.float64(beta)
            a = f32(0)
            if e > -1000.0:
                k = np.floor(e)
                a = f32(np.ldexp(np.float64(np.exp2(f32(e - k))), int(k)))
            A = _pack_bin(a, n, mask)
            row = int(A.view(np.int32)) & mask
            r = np.exp2(beta)
            px = f32(ca * A)
            py, r2 = f32(px * r), f32(r * r)
            for kk in range((nb + 1) // 2):
                out[2 * kk, i] = f32(px * G[row, 2 * kk])
                if 2 * kk + 1 < nb:
                    out[2 * kk + 1, i] = f32(py * G[row, 2 * kk + 1])
                px, py = f32(px * r2), f32(py * r2)
    return out / np.float64(ca)


def _valid_limit(nb, rng, res, ca=1.0):
    """Largest offset (ps) up to which the chain's first term ca * A, A =
    2^(Y - n beta), stays a normal float on the high side (n = B-1, Y ~ 0):
    (B-1) beta <= 126 + log2(ca)."""
    w = 2 * rng / nb
    return (nb - 1) / 2.0 * w + (126.0 + np.log2(ca)) / ((nb - 1) * 2 * (4.0 / res ** 2) * w)


_C = 0.0299792458
_FACTORED = [(13, 13 * 3.9 / _C, 214.0), (33, 33 * 1.5 / _C, 214.0), (64, 64 * 1.5 / _C, 214.0)]


# ca = (pair factor) x (activity x length) of one voxel term; 2^-27 is about the
# largest in a 41 cm ring with 3.2 mm crystals (geometry factor ~8e-4 / d1^2 d2^2)
@pytest.mark.parametrize("ca", [1.0, 2.0 ** -27])
@pytest.mark.parametrize("nb,rng,res", _FACTORED)
def test_factored_weights_match_table_within_their_range(nb, rng, res, ca):
    ref = T.tof_table(nb, rng, res)
    got = _factored_weights(nb, rng, res, ca)
    t = np.arange(-4000, 4001)
    ok = t <= _valid_limit(nb, rng, res, ca)
    # rounding of the FP32 power chain (up to B-1 products) and of the packed A:
    # measured 1.9e-6 / 4.6e-6 / 6.5e-6 absolute and 3.8e-6 / 7.9e-6 / 1.4e-5
    # relative on weights above 1e-3 for 13 / 33 / 64 bins
    assert np.abs(got[:, ok] - ref[:, ok]).max() < 1e-5
    big = (ref > 1e-3) & ok[None, :]
    assert (np.abs(got - ref)[big] / ref[big]).max() < 3e-5


@pytest.mark.parametrize("nb,rng,res", _FACTORED[:1])
def test_factored_chain_alone_fails_far_past_the_last_bin(nb, rng, res):
    """Why the kernel splits the table: run at every offset, the factored
    chain's start ca * A underflows past its range (weights of about 1 become
    0) and r^2 overflows further out (NaN)."""
    ref = T.tof_table(nb, rng, res)
    got = _factored_weights(nb, rng, res)
    assert not (np.isfinite(got).all() and np.abs(got - ref).max() < 1e-5)


def _largest_tof_offset(pr):
    """Largest positive TOF offset (ps) any (scatter point, pair, voxel) term
    of a problem reaches, from the oracle tracer.  A pair (l1, l2) with l1 on
    the smaller crystal (or the same crystal on another ring, both orders)
    puts leg-1 voxels at (d1 - d2 - 2s)/c and leg-2 voxels at (d1 - d2 + 2s)/c,
    s the voxel's distance from the point; only voxels with activity count."""
    from oracle import oracle as O

    xyz, _ = O.scatter_points(pr.activity, pr.attenuation, pr.image_size, pr.sample_step)
    g = pr.scanner.geometry
    rings = O.sampled_rings(g.shape[0], pr.nr_rings_used)
    dets = O.sampled_detectors(g.shape[1], pr.nr_detectors_used)
    crys = np.array([[g[r, d, 0], g[r, d, 1], g[r, 0, 2]] for d in dets for r in rings])
    cid = np.repeat(np.arange(len(dets)), len(rings))
    nl = len(crys)
    lines = np.concatenate([np.repeat(xyz, nl, 0), np.tile(crys, (len(xyz), 1))], 1)
    cnt, _, ix, sm = O.trace_batch(np.array(pr.activity.shape), np.asarray(pr.image_size).reshape(-1)[:6], lines,
                                   allow_overrun=True)
    act = np.asarray(pr.activity, np.float32).flatten("F")
    hot = (np.arange(sm.shape[1])[None, :] < cnt[:, None]) & (act[np.maximum(ix - 1, 0)] > 0)
    s_hi = np.where(hot, sm, -np.inf).max(1).reshape(len(xyz), nl)
    s_lo = np.where(hot, sm, np.inf).min(1).reshape(len(xyz), nl)
    d = np.linalg.norm(lines[:, 3:] - lines[:, :3], axis=1).reshape(len(xyz), nl)
    first = (cid[:, None] < cid[None, :]) | ((cid[:, None] == cid[None, :]) & ~np.eye(nl, dtype=bool))
    base = d[:, :, None] - d[:, None, :]                                   # [point, l1, l2]
    walk1 = np.where(first[None] & np.isfinite(s_lo)[:, :, None], base - 2 * s_lo[:, :, None], -np.inf)
    walk2 = np.where(first[None] & np.isfinite(s_hi)[:, None, :], base + 2 * s_hi[:, None, :], -np.inf)
    return max(walk1.max(), walk2.max()) / _C


@pytest.mark.parametrize("name", ["sss_tiny_far", "sss_wide_body_tof13"])
def test_far_goldens_need_the_per_bin_split(att_table, name):
    """The far-offset fixtures reach past the kernel's split offset: 5 bins
    of 1 cm at 60 ps (into the factored chain's NaN region, beta >= 64) and a
    50 cm wide body at the benchmark's 13 bins of 3.9 cm.  Both stay inside
    the reference's +-4000 ps table.  The FP64 oracle run with the kernel's
    emulated weights (factored below the split, per-bin from it on) matches
    the reference; on the 5-bin case the factored chain at every offset gives
    NaN."""
    from conftest import golden, problem_from_golden, rel_l2
    from oracle import oracle as O

    g = golden(name)
    pr = problem_from_golden(g)
    top = _largest_tof_offset(pr)
    nb, rng, res = pr.nr_bins, pr.tof_range, pr.tof_resolution
    assert _kernel_split_offset(nb, rng, res) < _valid_limit(nb, rng, res, 2.0 ** -27) < top < 4000, top

    def run(tof=None):
        return O.sss_compact(pr.activity, pr.attenuation, pr.image_size, pr.scanner.geometry, pr.scanner.normals,
                             pr.scanner.detector_size_mm, att_table, pr.energy_resolution, pr.energy_threshold,
                             pr.nr_rings_used, pr.nr_detectors_used, pr.sample_step, pr.tof_resolution,
                             pr.tof_range, pr.nr_bins, tof=tof)

    assert rel_l2(run(), g["compact"]) < 1e-6
    kernel = run(_kernel_weights(nb, rng, res))
    assert np.isfinite(kernel).all() and rel_l2(kernel, g["compact"]) < 1e-5
    if name == "sss_tiny_far":
        assert np.isnan(run(_factored_weights(nb, rng, res))).any()


def _kernel_split_offset(nb, rng, res):
    """First TOF offset (ps) whose weights the pair kernel takes per bin
    instead of from the factored chain (tof_const's tsafe, less 4000): past
    t_safe = s_{B-1} + 62 / ((B-1) 2 kappa w) the chain's start ca * A falls
    below 2^-126 for voxel terms ca < 2^-64."""
    w = 2 * rng / nb
    t_safe = (nb - 1) / 2.0 * w + 62.0 / ((nb - 1) * 2 * (4.0 / res ** 2) * w)
    return min(np.floor(t_safe) + 1, 4001)


def _per_bin_weights(nb, rng, res):
    """The per-bin evaluation 2^(Y - d (beta + gamma d)), d = n - b, in float32
    (the non-factored path of the pair kernel, with exp2 for its ex2)."""
    f32 = np.float32
    w = 2 * rng / nb
    kappa = 4.0 / (res * res)
    l2 = T.tof_log2_table(nb, rng, res).astype(np.float32)
    Y, n = l2[:, 0], l2[:, 1]
    k2w, gam = f32(2 * kappa * w), f32(kappa * w * w)
    s0, W = f32((1.0 - (nb + 1) / 2.0) * w), f32(w)
    beta = (k2w * (np.arange(-4000, 4001).astype(np.float32) - (n * W + s0))).astype(np.float32)
    d = (n[None, :] - np.arange(nb, dtype=np.float32)[:, None]).astype(np.float32)
    with np.errstate(all="ignore"):
        out = np.exp2((Y[None, :] - d * (beta[None, :] + gam * d)).astype(np.float32)).astype(np.float64)
    out[:, ~np.isfinite(Y)] = 0
    return out


def _kernel_weights(nb, rng, res, ca=1.0):
    """The pair kernel's weights in float32 emulation: the factored chain
    below the split offset, per-bin 2^x from it on."""
    t = np.arange(-4000, 4001)
    far = (t >= _kernel_split_offset(nb, rng, res))[None, :]
    return np.where(far, _per_bin_weights(nb, rng, res), _factored_weights(nb, rng, res, ca))


@pytest.mark.parametrize("nb,rng,res", _FACTORED + [(5, 5 * 1.0 / _C, 60.0), (2, 2 * 4.0 / _C, 214.0),
                                                    (7, 7 * 1.4 / _C, 100.0)])
def test_kernel_weights_match_table_at_every_offset(nb, rng, res):
    """Factored weights below the split, per-bin weights from it on: in
    float32 emulation that matches the FP64 table at all 8001 offsets, with
    no NaN, for voxel terms ca down to 2^-64."""
    ref = T.tof_table(nb, rng, res)
    for ca in (1.0, 2.0 ** -27, 2.0 ** -64):
        got = _kernel_weights(nb, rng, res, ca)
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() < 1e-5, ca


def test_dense_lor_check_accepts_reference_tables_and_rejects_bad_ones():
    from opensss_gb300 import geometry as G

    for args in ((1, 1, 1, 1, 48, 6), (38, 8, 1, 1, 20, 10), (1, 1, 1, 1, 64, 8)):
        for shift in (False, True):
            lor, _, _ = G.SinogramCoordinates(*args, ID_Shidt=shift)
            nd = lor.shape[0]
            for ndu in (1, 8, nd // 2, nd):
                G.check_dense_lor(lor, G.sampled_detectors(nd, ndu), nd)
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, 48, 6, ID_Shidt=False)
    dets = G.sampled_detectors(48, 8)
    with pytest.raises(ValueError):
        G.check_dense_lor(lor[:40, :40], dets, 48)
    for bad in ((dets[1], dets[3], 0, 24), (dets[0], dets[5], 1, 49), (dets[2], dets[2], 1, -1)):
        d1, d2, k, v = bad
        t = lor.copy()
        t[d1, d2, k] = v
        with pytest.raises(IndexError):
            G.check_dense_lor(t, dets, 48)
    t = lor.copy()
    t[dets[3], dets[1], 0] = 99  # di1 > di2: never read
    G.check_dense_lor(t, dets, 48)


def test_slice_table_check_accepts_reference_tables_and_rejects_bad_ones():
    from opensss_gb300 import geometry as G

    for args in ((1, 1, 1, 1, 48, 6), (38, 8, 1, 1, 20, 10), (1, 1, 1, 1, 64, 8)):
        _, si, _ = G.SinogramCoordinates(*args, ID_Shidt=False)
        nr = si.shape[0]
        assert np.array_equal(G.check_slice_table(si, nr), si)
    _, si, _ = G.SinogramCoordinates(1, 1, 1, 1, 48, 6, ID_Shidt=False)
    with pytest.raises(ValueError):
        G.check_slice_table(si[:4, :4], 6)
    for v in (-1, 36):
        t = si.copy()
        t[2, 3] = v
        with pytest.raises(IndexError):
            G.check_slice_table(t, 6)


@pytest.mark.parametrize("nd,nr,ndu,nru", [(48, 6, 8, 4), (64, 8, 10, 2), (760, 80, 48, 16)])
def test_dense_cell_pairs_rebuild_the_dense_layout(nd, nr, ndu, nru):
    """The cell table of the full densify, read the way its kernel reads it
    (every element: the cell's pair, or zero), rebuilds the oracle's dense
    layout of a random compact result exactly."""
    from oracle import oracle as O

    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, nd, nr, ID_Shidt=False)
    dets = G.sampled_detectors(nd, ndu)
    cells = G.dense_cell_pairs(lor, dets, nd)
    rng = np.random.default_rng(nd)
    nb = 2
    cmp = rng.random((nb, nru * nru, ndu, ndu))
    for ri in range(nru):  # a crystal with itself on one ring is no pair: zero in every result
        cmp[:, ri * nru + ri, np.arange(ndu), np.arange(ndu)] = 0.0
    ref = O.densify(cmp, lor, nd, nru, ndu)
    pair = cells.reshape(nd + 1, nd // 2)
    di1, di2 = np.where(pair >= 0, pair // ndu, 0), np.where(pair >= 0, pair % ndu, 0)
    ri1, ri2 = np.divmod(np.arange(nru * nru), nru)
    valid = (pair >= 0)[:, :, None] & ((di1 < di2)[:, :, None] | (ri1 != ri2)[None, None, :])
    got = cmp[:, (ri1 * nru + ri2)[None, None, :], di1[:, :, None], di2[:, :, None]] * valid[None]
    assert np.array_equal(got.astype(np.float32), ref)
