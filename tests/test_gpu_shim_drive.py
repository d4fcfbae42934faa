"""The MURaM-side shim on a GPU, driven in ComputeSolution's order.

`tests/shim_drive/drive.C` calls the hot-path routines by their MURaM names
and signatures (SaveCons, ConsToPrim, Adjust_Valf_Max, MHD_Residual,
Source_Integrate_Tcheck, exchange_grid_acc, SetBoundaryConditions, TVDlimit,
Clean_divB, TCheck; src/solver.C:109-365) over GridData / RunData /
PhysicsData, declared by stand-in headers (`tests/shim_drive/standin/`)
because MURaM's own sources are not part of this repository.  What runs is
the shim itself (`muram_main_gb300/shim/gpumhd_muram_shim.C`) and
libgpumhd.so: the eos_init wrapper (the linker's --wrap) creates the context,
Run.dt and Run.time changes push the parameters, Run.need_diagnostics
switches the diagnostics, and ACCH::UpdateGPU / UpdateCPU move GridData's
arrays.  Results: the reference's own (golden fixtures) to 1e-12 in FP64, and
a SINGLE_PRECISION build (cState of floats) equal, bit for bit, to the
per-routine Python path run on the same float-rounded state.
"""
import os
import subprocess

import numpy as np
import pytest

import helpers as H
from muram_main_gb300 import build, gpumhd

pytestmark = pytest.mark.gpu

DRIVE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "shim_drive")
CASES = ["periodic", "two_half_tvd", "open_bottom", "spitzer", "va_adjust", "diagnostics_two_half",
         "diagnostics_spitzer"]


@pytest.fixture(scope="module")
def drive_programs(gpu_lib):
    build.build()
    subprocess.run(["make", "-s", "-C", DRIVE, f"GPULIB={os.path.dirname(build.LIB)}"], check=True)
    return {64: os.path.join(DRIVE, "_build", "shim_drive"), 32: os.path.join(DRIVE, "_build", "shim_drive_sp")}


def run_drive(exe, hp, U, steps, diag_step, tmp):
    p = H.gpu_params(hp, 64)
    with open(os.path.join(tmp, "params.bin"), "wb") as f:
        f.write(bytes(p))
    with open(os.path.join(tmp, "run.txt"), "w") as f:
        f.write(f"{H.EOS_SMALL} {p.dt_rad!r} {steps} {diag_step}\n")
    np.ascontiguousarray(np.moveaxis(U, 0, -1), dtype=np.float64).tofile(os.path.join(tmp, "input.bin"))
    subprocess.run([exe, tmp], check=True, timeout=600)
    box = U.shape[1:]
    final = np.moveaxis(np.fromfile(os.path.join(tmp, "final.bin")).reshape(box + (8,)), -1, 0)
    dts = np.loadtxt(os.path.join(tmp, "dts.txt")).reshape(-1, 2)
    diag = np.fromfile(os.path.join(tmp, "diag.bin")).reshape((10,) + box) if diag_step else None
    pres = np.fromfile(os.path.join(tmp, "pres.bin")).reshape(box)
    return final, dts, diag, pres


@pytest.mark.parametrize("name", CASES)
def test_shim_in_compute_solution_order_matches_reference(drive_programs, name, tmp_path):
    d, hp = H.load_case(name)
    steps = int(d["steps"])
    ds = int(hp.get("diag_step", 0))
    final, dts, diag, _ = run_drive(drive_programs[64], hp, d["input_U"], steps, ds, str(tmp_path))
    assert np.allclose(dts[:, 0], d["dts"].reshape(-1, 3)[:steps, 0], rtol=1e-12, atol=0)
    e = H.rel_linf(final, d["final_U"])
    print(f"shim [{name}]: rel Linf per field {np.array2string(e, precision=2)}")
    assert np.all(e <= 1e-12), e
    if ds:
        assert np.all(H.rel_linf(diag, d["diag"]) <= 1e-12)


@pytest.mark.parametrize("name", ["periodic", "open_bottom"])
def test_shim_single_precision_build(drive_programs, name, tmp_path):
    """cState of floats (MURaM built with SINGLE_PRECISION) through the float
    transfers, FP64 on the device: the per-routine path on the same
    float-rounded state gives the same float results."""
    d, hp = H.load_case(name)
    steps = int(d["steps"])
    U32 = d["input_U"].astype(np.float32).astype(np.float64)
    final, dts, _, pres = run_drive(drive_programs[32], hp, U32, steps, 0, str(tmp_path))
    g = gpumhd.MuramGPU(H.gpu_params(hp, 64), eos_path=H.EOS_SMALL)
    g.upload_state(U32)
    g.exchange_grid(True)
    ref_dts = [g.step_reference_order()[0] for _ in range(steps)]
    assert np.array_equal(dts[:, 0], np.array(ref_dts))
    assert np.array_equal(final, g.download_state().astype(np.float32).astype(np.float64))
    assert np.array_equal(pres, g.download_field(gpumhd.FIELD_PRES))
    g.close()
