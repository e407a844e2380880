"""Drop-in ``GeneratePrompts`` and ``CreateDirectories`` (Python/openSSS/IO.py:44-133).

``GeneratePrompts`` is the pipeline's prompt cache: it histograms the CASToR
list-mode file once (``Datafile.ExportPrompts``, on the GPU) and saves the
prompts, randoms and normalisation sinograms under ``SavePath``.  A later run
that finds the prompts file skips the histogram.  The file names are the
reference's:
- ``PromptsSinogram.npz`` without span (Span == 1, slices from SinogramIndex);
- ``PromptsSinogramMashed.npz`` with span (Span > 1, slices from LookUpTable);
- ``RandomsSinogram.npz`` and ``NormSinogram.npz`` in both cases.
"""

from __future__ import annotations

import os
import shutil

import numpy as np

from . import Datafile


def CreateDirectories(targetFolder: str, folderImages: str, folderScatters: str, parameters: str):
    """Creates the image and scatter folders under targetFolder and keeps a
    copy of the parameter file there as ``parameters_backup.txt``; a copy that
    fails is reported, not raised (IO.py:44-75)."""
    for sub in (folderImages, folderScatters):
        os.makedirs(os.path.join(targetFolder, sub), exist_ok=True)
    try:
        shutil.copy(parameters, os.path.join(targetFolder, "parameters_backup.txt"))
        print(f"Used parameters saved to {targetFolder}")
    except OSError as e:
        print(f"Unable to copy file. {e}")


def prompt_files(SavePath: str, Span: int) -> dict:
    """Paths of the cached sinograms for this span setting."""
    name = "PromptsSinogram.npz" if Span == 1 else "PromptsSinogramMashed.npz"
    return {"prompts": os.path.join(SavePath, name), "randoms": os.path.join(SavePath, "RandomsSinogram.npz"),
            "norm": os.path.join(SavePath, "NormSinogram.npz")}


def GeneratePrompts(SavePath: str, DataPath: str, DataHeader: str, LORCoordinates, SinogramIndex, LookUpTable,
                    TOFbins: int, TOFRange: float, Span: int, Mash: int, Shift: int = 0, device="cuda") -> bool:
    """Histograms the list-mode file into the cache unless its prompts file
    exists.  Returns True when it histogrammed, False on a cache hit.
    Span < 1 writes nothing, as in the reference."""
    if Span < 1:
        return False
    files = prompt_files(SavePath, Span)
    if os.path.isfile(files["prompts"]):
        return False
    table = SinogramIndex if Span == 1 else LookUpTable
    prompts, randoms, norm = Datafile.ExportPrompts(DataPath, DataHeader, LORCoordinates, table, TOFbins,
                                                    TOFRange, mash=Mash, Shift=Shift, device=device)
    np.savez_compressed(files["prompts"], prompts)
    np.savez_compressed(files["randoms"], randoms)
    np.savez_compressed(files["norm"], norm)
    return True
