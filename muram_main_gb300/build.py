"""Compile the gpumhd CUDA library in-tree for sm_103a.

Five translation units are compiled in parallel and linked into
``muram_main_gb300/_build/libgpumhd.so``:

* ``kernels_f64.cu`` with ``--fmad=false`` (every product and sum rounds
  separately, like the reference's no-FMA builds);
* ``kernels_f32.cu`` with FMA contraction;
* ``gpumhd.cu`` (host side of the C ABI), host code with -ffp-contract=off;
* ``adjoint.cu`` (the FP64 adjoint kernels) and ``noalloc.cu`` (the
  allocation-free CFL entry point), both with ``--fmad=false``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgpumhd.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh"))] + [
        os.path.join(INCLUDE, "gpumhd.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False):
    """Build the library if any source is newer than it; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = nvcc_path()
    common = [nvcc, "-std=c++17", ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I", INCLUDE, "-c"]
    # FP32: contraction, approximate division and square root (within the
    # FP32 mode's error budget); FP64: every operation IEEE-rounded.
    units = [("kernels_f64.cu", ["--fmad=false"]),
             ("kernels_f32.cu", ["--fmad=true", "-prec-div=false", "-prec-sqrt=false"]),
             ("gpumhd.cu", ["--fmad=false"]),
             ("adjoint.cu", ["--fmad=false"]),
             ("noalloc.cu", ["--fmad=false"])]
    procs = []
    objs = []
    for src, extra in units:
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = common + extra + [os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"--- {s}\n{o}" for s, o in failed))
    tmp = LIB + ".tmp"
    link = [nvcc, ARCH, "-shared", "-o", tmp] + objs + ["-lcudart"]
    res = subprocess.run(link, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
