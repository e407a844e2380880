"""The ray walk's integer-pipe arithmetic (``opensss_gb300/csrc/trace.cuh``):
``add_nonneg_bits`` and ``div_bits`` against the host's IEEE binary64
addition and division, ``ceil_clear`` against ceil of the host's division.
``tests/native/add_bits_check.cu`` is compiled for the host with nvcc (no GPU
needed) and run on seeded random operands."""

import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_integer_fp64_arithmetic_matches_ieee(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "add_bits_check"
    src = os.path.join(ROOT, "tests", "native", "add_bits_check.cu")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "opensss_gb300", "csrc"),
                        "-I" + os.path.join(ROOT, "include"), src, "-o", str(exe)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe), "3000000"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-3000:]
    assert "mismatches 0" in out.stdout
    assert "divisions" in out.stdout and "deferred to FP64 0" in out.stdout
