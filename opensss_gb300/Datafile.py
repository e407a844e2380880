"""CASToR list-mode data on the GPU (drop-in for ``Timber.Datafile``).

``ExportPrompts`` histograms the events of a list-mode file into the
(radial, angular, slice, TOF bin) prompt sinogram plus the randoms and
normalisation sinograms, and ``InjectScatters`` writes a copy of the file with
each kept event's scatter rate inserted; both with the reference's arguments
and results (``Python/Timber/Datafile.py:29-240``).  The file is read once
into device memory and every event is decoded by one GPU thread
(``csrc/listmode.cu``); the reference decodes them one at a time in Python.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from . import Coincidence, Headerfile, _lib
from .engine import as_device


def _ptr(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def layout_of(header: dict, for_injection: bool = False) -> _lib.ListmodeLayout:
    fmt, pos = Coincidence.GenerateEventClass(header)
    if pos[3] is None:
        raise TypeError("the list-mode events carry no TOF field")
    L = _lib.ListmodeLayout()
    L.record_bytes = Coincidence.record_bytes(fmt)
    L.id_offset = 4 * pos[4]
    L.tof_offset = 4 * pos[3]
    L.scatter_offset = 4 * (1 + int(header["attenuation_flag"]))
    return L


def sino_map(lor_t: torch.Tensor, nd_lor: int, mash: int, shift: int, slices_t: torch.Tensor,
             nrad: int, nang: int, nslices: int, tof_bins: int, tof_range: float) -> _lib.SinoMap:
    M = _lib.SinoMap()
    M.lor = lor_t.data_ptr()
    M.nd_lor, M.mash, M.shift = int(nd_lor), int(mash), int(shift)
    M.slices = slices_t.data_ptr()
    M.nr_table = int(slices_t.shape[0])
    M.nrad, M.nang, M.nslices = int(nrad), int(nang), int(nslices)
    M.tof_bins, M.tof_range = int(tof_bins), float(tof_range)
    return M


def read_events(path: str, header: dict, device) -> torch.Tensor:
    """The event records of a data file as a flat uint8 device tensor."""
    fmt, _ = Coincidence.GenerateEventClass(header)
    size = os.path.getsize(path)
    if size / Coincidence.record_bytes(fmt) != header["nb_events"]:
        raise ValueError("The number of events in the file is not consistent with the header")
    raw = np.fromfile(path, dtype=np.uint8)
    return torch.from_numpy(raw).to(device)


def histogram_device(events: torch.Tensor, header: dict, LORCoordinates, SinogramIndex, TOF_bins: int,
                     TOF_range: float, mash: int = 1, Shift: int = 0, device="cuda"):
    """(prompts uint16, randoms float32 or None, norm float32 or None) as
    device tensors of the reference's shapes."""
    _lib.require_cuda(events=events)
    lor = np.asarray(LORCoordinates)
    table = np.asarray(SinogramIndex)
    nrad = int(lor[:, :, 1].max()) + 1
    nang = int(lor[:, :, 0].max()) + 1
    nslices = int(table.max()) + 1
    lor_t = as_device(lor.astype(np.int16), torch.int16, device)
    slices_t = as_device(table.astype(np.int16), torch.int16, device)
    L = layout_of(header)
    M = sino_map(lor_t, lor.shape[0], mash, Shift, slices_t, nrad, nang, nslices, TOF_bins, TOF_range)
    n = events.numel() // L.record_bytes
    counts = torch.zeros((nrad, nang, nslices, TOF_bins), dtype=torch.int32, device=device)
    want = header["random_flag"] or header["normalization_flag"]
    last = torch.zeros((nrad, nang, nslices), dtype=torch.int64, device=device) if want else None
    status = torch.zeros(1, dtype=torch.int32, device=device)
    st = C.c_void_p(torch.cuda.current_stream(device).cuda_stream)
    lib = _lib.lib()
    _lib.check(lib.sss_histogram_prompts(_ptr(events), n, C.byref(L), C.byref(M), _ptr(counts), _ptr(last),
                                         _ptr(status), st))
    prompts = torch.empty((nrad, nang, nslices, TOF_bins), dtype=torch.int16, device=device)
    randoms = (torch.zeros((nrad, nang, nslices), dtype=torch.float32, device=device)
               if header["random_flag"] else None)
    norm = (torch.ones((nrad, nang, nslices), dtype=torch.float32, device=device)
            if header["normalization_flag"] else None)
    _lib.check(lib.sss_histogram_finish(_ptr(events), n, C.byref(L), C.byref(M), _ptr(counts), _ptr(last),
                                        float(header["duration"]), _ptr(prompts), _ptr(randoms), _ptr(norm), st))
    torch.cuda.current_stream(device).synchronize()
    _lib.check_status(int(status.item()))
    return prompts, randoms, norm


def ExportPrompts(DataPath: str, DataHeader: str, LORCoordinates, SinogramIndex, TOF_bins: int,
                  TOF_range: float = None, mash: int = 1, Shift: int = 0, device="cuda"):
    """Prompts (uint16), randoms and normalisation sinograms of a CASToR
    list-mode file, as the reference's ExportPrompts (``Datafile.py:29-115``)."""
    if not torch.cuda.is_available():
        raise _lib.EngineUnavailable("no CUDA device: the engine has no CPU path")
    header = Headerfile.ReadHeaderFile(os.path.join(DataPath, DataHeader))
    events = read_events(os.path.join(DataPath, header["data_filename"]), header, device)
    if TOF_range is None:
        TOF_range = header["tof_range"]
    p, r, n = histogram_device(events, header, LORCoordinates, SinogramIndex, TOF_bins, TOF_range, mash,
                               Shift, device)
    prompts = p.cpu().numpy().view(np.uint16)
    return (prompts, None if r is None else r.cpu().numpy(), None if n is None else n.cpu().numpy())


def inject_device(events: torch.Tensor, header: dict, LORCoordinates, slice_table, nslices: int,
                  scatters: torch.Tensor, factor: np.ndarray, TOF_range: float, mash: int = 1, Shift: int = 0,
                  device="cuda"):
    """(out records uint8 device tensor, kept events): the injection on
    device-resident events and scatter sinograms [bins, rad, ang, slice]."""
    _lib.require_cuda(events=events, scatters=scatters)
    lor = np.asarray(LORCoordinates)
    nrad = int(lor[:, :, 1].max()) + 1
    nang = int(lor[:, :, 0].max()) + 1
    bins = int(scatters.shape[0])
    lor_t = as_device(lor.astype(np.int16), torch.int16, device)
    slices_t = as_device(np.asarray(slice_table).astype(np.int16), torch.int16, device)
    L = layout_of(header)
    M = sino_map(lor_t, lor.shape[0], mash, Shift, slices_t, nrad, nang, nslices, bins, TOF_range)
    n = events.numel() // L.record_bytes
    lib = _lib.lib()
    ws = torch.empty(int(lib.sss_inject_workspace_size(n)), dtype=torch.uint8, device=device)
    out = torch.empty(n * (L.record_bytes + 4), dtype=torch.uint8, device=device)
    count = torch.zeros(1, dtype=torch.int64, device=device)
    status = torch.zeros(1, dtype=torch.int32, device=device)
    fac = torch.from_numpy(np.ascontiguousarray(factor, dtype=np.float32)).to(device)
    st = C.c_void_p(torch.cuda.current_stream(device).cuda_stream)
    _lib.check(lib.sss_inject_scatters(_ptr(events), n, C.byref(L), C.byref(M), _ptr(scatters), _ptr(fac),
                                       _ptr(out), _ptr(count), _ptr(ws), ws.numel(), _ptr(status), st))
    torch.cuda.current_stream(device).synchronize()
    _lib.check_status(int(status.item()))
    kept = int(count.item())
    return out[: kept * (L.record_bytes + 4)], kept


def InjectScatters(DataPath: str, DataHeader: str, LORCoordinates, SinogramIndex, ScatterPath: str,
                   LookUpTable, SpanFlag: bool, TOF_range: float = None, NewPath: str = None, mash: int = 1,
                   Shift: int = 0, device="cuda"):
    """Writes ``<name>scatter_<ext>`` next to (or in NewPath instead of) the
    original data file and header, as the reference (``Datafile.py:117-240``)."""
    if not torch.cuda.is_available():
        raise _lib.EngineUnavailable("no CUDA device: the engine has no CPU path")
    header = Headerfile.ReadHeaderFile(os.path.join(DataPath, DataHeader))
    if header["scatter_flag"]:
        raise ValueError("the data file already carries scatter rates")
    duration = header["duration"]
    scale = np.load(os.path.join(ScatterPath, "ScaleFactors.npy"))
    bins = scale.shape[0]
    events = read_events(os.path.join(DataPath, header["data_filename"]), header, device)
    new = dict(header)
    new["scatter_flag"] = True
    name = header["data_filename"]
    new["data_filename"] = name[:-6] + "scatter_" + name[-6:]
    new_header_name = DataHeader[:-6] + "scatter_" + DataHeader[-6:]
    if TOF_range is None:
        TOF_range = header["tof_range"]
    else:
        new["tof_range"] = TOF_range
    NewPath = DataPath if NewPath is None else NewPath
    # float32 arithmetic as the reference rounds it (:165, :228)
    scale = (scale / (2 * TOF_range / bins)).astype(scale.dtype)
    sf = 1.0 / (0.299792458 / 2)
    factor = np.array([(scale[b] * sf) / duration for b in range(bins)], dtype=np.float32)
    lor = np.asarray(LORCoordinates)
    si = np.asarray(SinogramIndex)
    if SpanFlag:
        nslices = si.shape[0]
    else:
        nslices = int(np.max(si)) + 1
    table = si if si.shape[0] == si.shape[1] else np.asarray(LookUpTable)
    nrad, nang = int(lor[:, :, 1].max()) + 1, int(lor[:, :, 0].max()) + 1
    sino = torch.empty((bins, nrad, nang, nslices), dtype=torch.float32, device=device)
    for b in range(bins):
        arr = np.load(os.path.join(ScatterPath, f"SSS_mashed_bin{b}.npz"))["arr_0"]
        sino[b].copy_(torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float32).reshape(nrad, nang, nslices)))
    out, kept = inject_device(events, header, lor, table, nslices, sino, factor, TOF_range, mash, Shift, device)
    out.cpu().numpy().tofile(os.path.join(NewPath, new["data_filename"]))
    new["nb_events"] = kept
    Headerfile.WriteHeaderFile(new, os.path.join(NewPath, new_header_name))
