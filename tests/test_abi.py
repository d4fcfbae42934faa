"""The C ABI: the library builds, loads and exports every function the header
declares, and the Python mirror of gpumhd_params has the C layout.  No
compute calls (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

import helpers as H
from muram_main_gb300 import build, gpumhd

HEADER = os.path.join(H.ROOT, "include", "gpumhd.h")


def header_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(gpumhd_[A-Za-z_0-9]+)\s*\(", txt)))


def test_library_builds_and_exports_header():
    lib = build.build()
    assert os.path.exists(lib)
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (gpumhd_\w+)", out))
    declared = header_functions()
    assert declared, "no declarations parsed"
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    assert set(declared) == set(gpumhd.EXPORTS)


def test_library_loads_with_ctypes():
    L = gpumhd.load()
    for f in header_functions():
        assert hasattr(L, f)


def test_params_layout_matches_header():
    fields = [f[0] for f in gpumhd.Params._fields_ if not f[0].startswith("pad")]
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "gpumhd.h"', "int main(void){",
           'printf("%zu\\n", sizeof(gpumhd_params));']
    for f in fields:
        src.append(f'printf("%zu\\n", offsetof(gpumhd_params, {f}));')
    src.append("return 0;}")
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "t.c")
        open(c, "w").write("\n".join(src))
        exe = os.path.join(td, "t")
        subprocess.run(["gcc", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        vals = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == C.sizeof(gpumhd.Params)
    for f, off in zip(fields, vals[1:]):
        assert getattr(gpumhd.Params, f).offset == off, f


def test_default_params_match_reference_defaults():
    p = gpumhd.default_params(8, 8, 8, 3.2e6)
    assert p.CFL == 0.8 and p.CFL_tvd == 0.95          # src/run.C:24-25
    assert p.va_max == 1e7 and p.va_adjust == 0.0       # include/physics.H:124-125
    assert list(p.tvd_h) == [2.0] * 4 and list(p.tvd_cs) == [0.2] * 4
    assert list(p.tchk) == [1.0e11, 1.0e-16, 4.0e15, 100.0e5]
    assert p.precision == 64


def test_create_rejects_bad_grid_without_gpu_work():
    L = gpumhd.load()
    p = gpumhd.default_params(2, 8, 8, 3.2e6)
    h = C.c_void_p()
    assert L.gpumhd_create(C.byref(p), 0, C.byref(h)) == gpumhd.E_INVALID
    assert b">= 4" in L.gpumhd_last_error(None)


def test_dropin_links_in_place_of_reference_routines():
    """The MURaM-side shim, linked with the reference's non-hot-path objects and
    the harness that calls the routines by their reference names, resolves every
    hot-path routine to the shim (link-level drop-in; needs the reference sources)."""
    from oracle import refrun
    if not os.path.isdir(refrun.REF_ROOT):
        pytest.skip("reference sources not available")
    build.build()
    assert refrun.build_dropin()
    out = subprocess.run(["nm", "-C", refrun.DROPIN_BIN], capture_output=True, text=True, check=True).stdout
    shim_obj = os.path.join(os.path.dirname(refrun.DROPIN_BIN), "obj", "gpumhd_muram_shim.o")
    shim_syms = subprocess.run(["nm", "-C", "--defined-only", shim_obj], capture_output=True, text=True,
                               check=True).stdout
    for fn in ("SaveCons(", "ConsToPrim(", "Adjust_Valf_Max(", "MHD_Residual(", "Source_Integrate_Tcheck(",
               "TVDlimit(", "TCheck(", "exchange_grid_acc(", "SetBoundaryConditions("):
        assert fn in shim_syms, fn
        assert out.count(" T " + fn) == 1, fn
    ldd = subprocess.run(["ldd", refrun.DROPIN_BIN], capture_output=True, text=True, check=True).stdout
    assert "libgpumhd.so" in ldd


def test_shim_single_precision_build_moves_float_cstate():
    """Compiled as a SINGLE_PRECISION build of MURaM compiles it, the shim moves
    GridData's cState arrays (floats there) through the float entry points and
    the double arrays through the double ones (needs the reference headers)."""
    from oracle import refrun
    if not os.path.isdir(refrun.REF_ROOT):
        pytest.skip("reference sources not available")
    here = os.path.dirname(os.path.abspath(refrun.__file__))
    subprocess.run(["make", "-s", "-C", here, "shim_sp", f"REF={refrun.REF_ROOT}"], check=True)
    obj = os.path.join(here, "_ref", "obj", "gpumhd_muram_shim_sp.o")
    und = subprocess.run(["nm", "-u", obj], capture_output=True, text=True, check=True).stdout.split()
    for fn in ("gpumhd_upload_f32", "gpumhd_download_f32", "gpumhd_upload", "gpumhd_download"):
        assert fn in und, fn


def test_shim_drive_program_builds():
    """The MURaM-side shim compiled against the stand-in MURaM headers and
    linked with libgpumhd.so, in both cState precisions (no GPU needed to
    build; tests/test_gpu_shim_drive.py runs them)."""
    build.build()
    here = os.path.join(H.ROOT, "tests", "shim_drive")
    subprocess.run(["make", "-s", "-C", here, f"GPULIB={os.path.dirname(build.LIB)}"], check=True)
    for exe in ("shim_drive", "shim_drive_sp"):
        path = os.path.join(here, "_build", exe)
        assert os.access(path, os.X_OK), path
        und = subprocess.run(["nm", "-u", path], capture_output=True, text=True, check=True).stdout
        assert "gpumhd_mhd_residual" in und and "gpumhd_tvdlimit" in und
        if exe == "shim_drive_sp":
            assert "gpumhd_upload_f32" in und and "gpumhd_download_f32" in und
