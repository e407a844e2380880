"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/libsssoracle.so`` — the FP64 C restatement
  (``oracle/sss_oracle.c``), built with OpenMP and ``-ffp-contract=off`` so
  that no multiply-add is fused, matching the reference's IEEE FP64 numerics.
* ``oracle/_build/libsssoracle_gpu.so`` — the FP64 GPU oracle
  (``oracle/sss_oracle_gpu.cu``): the same restatement's SSS on an sm_103a GPU,
  built with ``-fmad=false`` so that no multiply-add is fused there either.
* ``oracle/_ref/libref_rt3dtof.so`` and ``oracle/_ref/libref_rt3d.so`` — the
  reference's own MEX ray tracers (``Matlab/RayTracing3DTOF.cpp``,
  ``Matlab/RayTracing3D.cpp``) compiled unmodified from the reference checkout
  against the build-owned ``mex.h`` shim.  Built only where the reference
  checkout exists; their outputs never enter the repository history.

Run ``python oracle/build_oracle.py`` (``__graft_entry__.build()`` calls it).
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_MATLAB = os.environ.get("OPENSSS_REFERENCE_MATLAB", "/root/reference/Matlab")

CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: " + " ".join(cmd) + "\n" + r.stderr[-4000:])


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(HERE, "sss_oracle.c")
    out = os.path.join(out_dir, "libsssoracle.so")
    if force or _stale(out, [src, os.path.join(HERE, "orc_core.h")]):
        _run(["gcc", "-std=gnu11", *CFLAGS, "-fopenmp", src, "-o", out + ".tmp", "-lm"])
        os.replace(out + ".tmp", out)
    return out


def build_oracle_gpu(force=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(HERE, "sss_oracle_gpu.cu")
    out = os.path.join(out_dir, "libsssoracle_gpu.so")
    if force or _stale(out, [src, os.path.join(HERE, "orc_core.h")]):
        nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
        _run([nvcc if os.path.exists(nvcc) else "nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
              "-fmad=false", "-lineinfo", "-Xcompiler", "-fPIC", "-shared", src, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def build_ref(force=False):
    """Compile the reference's MEX tracers; returns [] if the checkout is absent."""
    outs = []
    if not os.path.isdir(REFERENCE_MATLAB):
        return outs
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    shim = os.path.join(HERE, "mex_shim")
    entry = os.path.join(shim, "mex_entry.c")
    for name, nout in (("RayTracing3DTOF", 3), ("RayTracing3D", 2)):
        cpp = os.path.join(REFERENCE_MATLAB, name + ".cpp")
        out = os.path.join(out_dir, f"libref_{name.lower()}.so")
        if not os.path.exists(cpp):
            continue
        if force or _stale(out, [cpp, entry, os.path.join(shim, "mex.h")]):
            obj_c = os.path.join(out_dir, f"{name}_entry.o")
            obj_cpp = os.path.join(out_dir, f"{name}.o")
            # -O0 as well as no contraction: the reference's own build flags are
            # MATLAB's; plain IEEE evaluation keeps it comparable to the Python tracer.
            _run(["gcc", "-O0", "-fPIC", "-ffp-contract=off", f"-DREF_NOUT={nout}",
                  f"-I{shim}", "-c", entry, "-o", obj_c])
            _run(["g++", "-O0", "-fPIC", "-ffp-contract=off", f"-I{shim}", "-c", cpp,
                  "-o", obj_cpp])
            _run(["g++", "-shared", obj_c, obj_cpp, "-o", out + ".tmp"])
            os.replace(out + ".tmp", out)
            for o in (obj_c, obj_cpp):
                os.remove(o)
        outs.append(out)
    return outs


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_oracle_gpu(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
