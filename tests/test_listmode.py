"""CASToR list-mode rows: the host decoding and a plain-Python histogram of
the same events against the reference's ExportPrompts / InjectScatters
outputs (tests/golden/listmode.npz), then the GPU kernels against the same
goldens, bit for bit."""

import os
import struct

import numpy as np
import pytest

from conftest import golden


def _tables(ncr, nr, mash, span, mrd):
    from opensss_gb300 import DataReduction as D, geometry as G

    lor, si, _ = G.SinogramCoordinates(1, 1, 1, 1, ncr // mash, nr, ID_Shidt=False)
    if span > 0:
        msi, _, lut, _ = D.SinogramLUT(nr, span, mrd)
        return lor, si, msi, lut, lut
    return lor, si, si, np.array([]), si


def _write_case(g, ci, d):
    from opensss_gb300 import Headerfile, workloads as W

    ev = g[f"case{ci}_events"]
    n = ev.size // 24
    name = f"case{ci}_df"
    ev.tofile(os.path.join(d, f"{name}.Cdf"))
    Headerfile.WriteHeaderFile(W.listmode_header(name, n), os.path.join(d, f"{name}.Cdh"))
    return f"{name}.Cdh"


@pytest.mark.parametrize("ci", range(4))
def test_host_decoding_reproduces_reference_histogram(ci, tmp_path):
    """Python restatement of the event layout and ParseCASToRIDs, looped over
    the events: the oracle for this row."""
    from opensss_gb300 import Coincidence, Headerfile

    g = golden("listmode")
    ncr, nr, mash, shift, span, mrd = (int(v) for v in g[f"case{ci}_args"])
    lor, si, msi, lut, table = _tables(ncr, nr, mash, span, mrd)
    hdr = Headerfile.ReadHeaderFile(os.path.join(tmp_path, _write_case(g, ci, str(tmp_path))))
    fmt, pos = Coincidence.GenerateEventClass(hdr)
    prompts = np.zeros(g[f"case{ci}_prompts"].shape, np.uint16)
    randoms = np.zeros(g[f"case{ci}_randoms"].shape, np.float32)
    norm = np.ones(g[f"case{ci}_norm"].shape, np.float32)
    bins, rng_ps = 5, 1000.0
    for ev in struct.iter_unpack(fmt, g[f"case{ci}_events"].tobytes()):
        d1, r1, d2, r2, tof = Coincidence.ParseCASToRIDs(ev, pos, ncr, shift)
        ang, rad = lor[d1 // mash, d2 // mash]
        s = table[r1, r2]
        if s == -1 or rad == -1 or ang == -1:
            continue
        randoms[rad, ang, s] = ev[0] * hdr["duration"] / bins
        norm[rad, ang, s] = ev[1]
        if abs(tof) > rng_ps:
            continue
        t = (tof + rng_ps) / (2 * rng_ps / bins)
        if 0 <= t < bins:
            prompts[rad, ang, s, int(t)] += 1
    assert np.array_equal(prompts, g[f"case{ci}_prompts"])
    assert np.array_equal(randoms, g[f"case{ci}_randoms"])
    assert np.array_equal(norm, g[f"case{ci}_norm"])


def _numpy_histogram(ev, duration, ncr, lor, table, bins, rng_ps, mash, shift):
    """The same histogram as the loop above (ExportPrompts, Datafile.py:29-115,
    with ParseCASToRIDs, Coincidence.py:97-159), vectorised over a structured
    event array with fields time, c0.. (corrections; the last is the TOF
    difference), id1, id2: (prompts uint16, randoms, norm), the last event of
    each cell giving its randoms and normalisation values."""
    names = ev.dtype.names
    a, b = ev["id1"].astype(np.int64), ev["id2"].astype(np.int64)
    tof = ev[names[-3]].astype(np.float64)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    tof_t = np.where(a < b, tof, -tof)
    c1, c2 = lo % ncr, hi % ncr
    d1, d2 = np.minimum(c1, c2), np.maximum(c1, c2)
    s1, s2 = (c1 - shift) % ncr, (c2 - shift) % ncr
    first = s1 < s2
    r1 = np.where(first, lo // ncr, hi // ncr)
    r2 = np.where(first, hi // ncr, lo // ncr)
    tof = np.where(first, tof_t, -tof_t)
    ang = lor[d1 // mash, d2 // mash, 0].astype(np.int64)
    rad = lor[d1 // mash, d2 // mash, 1].astype(np.int64)
    sino = table[r1, r2].astype(np.int64)
    nrad, nang, nsl = int(lor[:, :, 1].max()) + 1, int(lor[:, :, 0].max()) + 1, int(table.max()) + 1
    ok = (sino != -1) & (rad != -1) & (ang != -1)
    cell = (rad * nang + ang) * nsl + sino
    t = (tof + rng_ps) / (2 * rng_ps / bins)
    inb = ok & (np.abs(tof) <= rng_ps) & (t >= 0) & (t < bins)
    counts = np.bincount(cell[inb] * bins + t[inb].astype(np.int64), minlength=nrad * nang * nsl * bins)
    prompts = (counts & 0xFFFF).astype(np.uint16).reshape(nrad, nang, nsl, bins)
    # the last event of each cell: events in file order, so the last occurrence
    idx = np.nonzero(ok)[0]
    cells = cell[idx]
    last = np.full(nrad * nang * nsl, -1, np.int64)
    np.maximum.at(last, cells, idx)
    has = last >= 0
    randoms = np.zeros(nrad * nang * nsl, np.float32)
    norm = np.ones(nrad * nang * nsl, np.float32)
    randoms[has] = (ev["time"][last[has]].astype(np.float64) * duration / bins).astype(np.float32)
    norm[has] = ev[names[1]][last[has]]
    return prompts, randoms.reshape(nrad, nang, nsl), norm.reshape(nrad, nang, nsl)


@pytest.mark.parametrize("ci", range(4))
def test_numpy_histogram_reproduces_reference(ci, tmp_path):
    """The vectorised restatement against the reference's outputs."""
    from opensss_gb300 import Headerfile, workloads as W

    g = golden("listmode")
    ncr, nr, mash, shift, span, mrd = (int(v) for v in g[f"case{ci}_args"])
    lor, si, msi, lut, table = _tables(ncr, nr, mash, span, mrd)
    hdr = Headerfile.ReadHeaderFile(os.path.join(tmp_path, _write_case(g, ci, str(tmp_path))))
    n = g[f"case{ci}_events"].size // 24
    ev = g[f"case{ci}_events"].view(W.synthetic_events(W.listmode_header("x", 1), 2, 1).dtype)[:n]
    p, r, nm = _numpy_histogram(ev, hdr["duration"], ncr, lor, np.asarray(table), 5, 1000.0, mash, shift)
    assert np.array_equal(p, g[f"case{ci}_prompts"])
    assert np.array_equal(r, g[f"case{ci}_randoms"])
    assert np.array_equal(nm, g[f"case{ci}_norm"])


def test_header_round_trip(tmp_path):
    from opensss_gb300 import Headerfile, workloads as W

    h = W.listmode_header("x_df", 123, random_flag=False)
    Headerfile.WriteHeaderFile(h, tmp_path / "x.Cdh")
    back = Headerfile.ReadHeaderFile(tmp_path / "x.Cdh")
    assert back == h


@pytest.mark.gpu
@pytest.mark.parametrize("ci", range(4))
def test_gpu_export_prompts_matches_reference(cuda_ok, ci, tmp_path):
    from opensss_gb300.Datafile import ExportPrompts

    g = golden("listmode")
    ncr, nr, mash, shift, span, mrd = (int(v) for v in g[f"case{ci}_args"])
    lor, si, msi, lut, table = _tables(ncr, nr, mash, span, mrd)
    hdr = _write_case(g, ci, str(tmp_path))
    p, r, n = ExportPrompts(str(tmp_path), hdr, lor, table, 5, 1000.0, mash=mash, Shift=shift)
    assert p.dtype == np.uint16 and np.array_equal(p, g[f"case{ci}_prompts"])
    assert np.array_equal(r, g[f"case{ci}_randoms"])
    assert np.array_equal(n, g[f"case{ci}_norm"])


@pytest.mark.gpu
@pytest.mark.parametrize("ci", range(4))
def test_gpu_inject_scatters_matches_reference(cuda_ok, ci, tmp_path):
    from opensss_gb300.Datafile import InjectScatters

    g = golden("listmode")
    ncr, nr, mash, shift, span, mrd = (int(v) for v in g[f"case{ci}_args"])
    lor, si, msi, lut, table = _tables(ncr, nr, mash, span, mrd)
    hdr = _write_case(g, ci, str(tmp_path))
    np.save(tmp_path / "ScaleFactors.npy", g[f"case{ci}_scale"])
    for b in range(5):
        np.savez_compressed(tmp_path / f"SSS_mashed_bin{b}", g[f"case{ci}_scatters"][b])
    InjectScatters(str(tmp_path), hdr, lor, msi, str(tmp_path), lut, span > 0, 1000.0, mash=mash, Shift=shift)
    dname = f"case{ci}_df.Cdf"
    got = np.fromfile(tmp_path / (dname[:-6] + "scatter_" + dname[-6:]), dtype=np.uint8)
    assert np.array_equal(got, g[f"case{ci}_injected"])
    text = (tmp_path / (hdr[:-6] + "scatter_" + hdr[-6:])).read_text()
    assert text == g[f"case{ci}_injected_header"].tobytes().decode()


def test_generate_prompts_cache_rule(tmp_path, monkeypatch):
    """GeneratePrompts histograms once per SavePath and span setting (the
    reference's file names); a later call finds the prompts file and skips
    the histogram.  The histogram itself is replaced by a recording fake."""
    from opensss_gb300 import IO

    calls = []

    def fake_export(DataPath, DataHeader, lor, table, bins, rng, mash=1, Shift=0, device="cuda"):
        calls.append((table, mash, Shift))
        return np.zeros((2, 2, 2, bins), np.uint16), np.zeros((2, 2, 2), np.float32), np.ones((2, 2, 2), np.float32)

    monkeypatch.setattr(IO.Datafile, "ExportPrompts", fake_export)
    si, lut = np.zeros((2, 2)), np.ones((2, 2))
    assert IO.GeneratePrompts(str(tmp_path), "d", "h", None, si, lut, 3, 1000.0, 1, 2, 5)
    assert calls[-1][0] is si and calls[-1][1:] == (2, 5)
    assert not IO.GeneratePrompts(str(tmp_path), "d", "h", None, si, lut, 3, 1000.0, 1, 2, 5)
    assert IO.GeneratePrompts(str(tmp_path), "d", "h", None, si, lut, 3, 1000.0, 3, 1)  # span: its own file
    assert calls[-1][0] is lut and len(calls) == 2
    assert not IO.GeneratePrompts(str(tmp_path), "d", "h", None, si, lut, 3, 1000.0, 3, 1)
    assert not IO.GeneratePrompts(str(tmp_path / "x"), "d", "h", None, si, lut, 3, 1000.0, 0, 1)
    names = sorted(os.listdir(tmp_path))
    assert names == ["NormSinogram.npz", "PromptsSinogram.npz", "PromptsSinogramMashed.npz", "RandomsSinogram.npz"]
    assert np.load(tmp_path / "PromptsSinogram.npz")["arr_0"].shape == (2, 2, 2, 3)


def test_create_directories(tmp_path, capsys):
    from opensss_gb300 import IO

    params = tmp_path / "p.txt"
    params.write_text("TOFbins = 6\n")
    IO.CreateDirectories(str(tmp_path / "out"), "Images", "Scatters", str(params))
    assert (tmp_path / "out" / "Images").is_dir() and (tmp_path / "out" / "Scatters").is_dir()
    assert (tmp_path / "out" / "parameters_backup.txt").read_text() == "TOFbins = 6\n"
    IO.CreateDirectories(str(tmp_path / "out"), "Images", "Scatters", str(tmp_path / "missing.txt"))
    assert "Unable to copy file" in capsys.readouterr().out


@pytest.mark.gpu
def test_gpu_generate_prompts_writes_the_reference_histogram(cuda_ok, tmp_path):
    from opensss_gb300 import IO

    g = golden("listmode")
    ncr, nr, mash, shift, span, mrd = (int(v) for v in g["case1_args"])
    lor, si, msi, lut, table = _tables(ncr, nr, mash, span, mrd)
    hdr = _write_case(g, 1, str(tmp_path))
    assert IO.GeneratePrompts(str(tmp_path), str(tmp_path), hdr, lor, si, lut, 5, 1000.0, 1, mash, shift)
    assert np.array_equal(np.load(tmp_path / "PromptsSinogram.npz")["arr_0"], g["case1_prompts"])
    assert np.array_equal(np.load(tmp_path / "RandomsSinogram.npz")["arr_0"], g["case1_randoms"])
    assert np.array_equal(np.load(tmp_path / "NormSinogram.npz")["arr_0"], g["case1_norm"])


@pytest.mark.gpu
def test_gpu_histogram_of_a_large_sinogram_matches_numpy(cuda_ok):
    """The demo's reduced sinogram (760 x 80 scanner, mash 2, span 19: 381 x
    190 x 815 cells x 6 TOF bins, 1.4 GB of counters), which the GPU fills in
    L2-sized buckets of cells: 3 million seeded events against the vectorised
    restatement, bit for bit."""
    import torch

    from opensss_gb300 import DataReduction as D, Datafile, geometry as G, workloads as W

    header = W.listmode_header("big_df", 3_000_000)
    ev = W.synthetic_events(header, 760, 80, seed=4)
    lor, _, _ = G.SinogramCoordinates(1, 1, 1, 1, 380, 80, ID_Shidt=False)
    _, _, lut, _ = D.SinogramLUT(80, 19, 79)
    ref = _numpy_histogram(ev, header["duration"], 760, lor, np.asarray(lut), 6, 1000.0, 2, 0)
    dev = torch.from_numpy(ev.view(np.uint8).reshape(-1)).cuda()
    got = Datafile.histogram_device(dev, header, lor, lut, 6, 1000.0, mash=2, Shift=0)
    for g_, r_ in zip(got, ref):
        assert np.array_equal(g_.cpu().numpy().view(r_.dtype), r_)
