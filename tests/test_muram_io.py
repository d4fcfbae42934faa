"""Result / restart files in the reference's format (src/io_xysl.C:39-48,
99-209, 278-411; src/boundary_pdmp_1_fftw3.C:44-62)."""
import os

import numpy as np
import pytest

from helpers import EOS_SMALL, rel_linf
from muram_main_gb300 import muram_io
from muram_main_gb300.initial import EosTable, periodic_box
from oracle import refrun

REF_TEST3D = os.path.join(refrun.REF_ROOT, "TEST", "Test_3D")


def _box(nx=12, ny=10, nz=8, seed=5):
    return periodic_box(EosTable(EOS_SMALL), nx, ny, nz, seed=seed)


def test_write_read_round_trip(tmp_path):
    U = _box()
    muram_io.write_result(U, str(tmp_path), 7, (3.2e6, 3.2e6, 3.2e6), time=12.5, dt=0.25, inv_va2max=1e-12,
                          p_bc=1.5e5, s_bc=-2e9)
    names = sorted(os.listdir(tmp_path))
    assert names == sorted([f"result_prim_{v}.000007" for v in range(8)] + ["Header.000007", "backup.dat"])
    for v in range(8):
        assert os.path.getsize(tmp_path / f"result_prim_{v}.000007") == 12 * 10 * 8 * 4
    # the files hold OutputSolution's float64 primitives cast to float32
    P = muram_io.read_prims(str(tmp_path), 7, (12, 10, 8))
    assert np.array_equal(P, muram_io.conserved_to_output(U).astype(np.float32))
    # restoring gives the conserved state to float32 precision
    R = muram_io.read_result(str(tmp_path), 7)
    Ui, Ri = U[:, 2:-2, 2:-2, 2:-2], R[:, 2:-2, 2:-2, 2:-2]
    assert np.all(rel_linf(Ri, Ui) < 2e-6)
    assert np.all(R[:, :2] == 0)  # ghosts are left for the boundary fill
    h = muram_io.read_header(str(tmp_path), 7)
    assert (h["nx"], h["ny"], h["nz"]) == (12, 10, 8)
    assert h["dx"] == (3.2e6, 3.2e6, 3.2e6)
    assert h["time"] == 12.5 and h["dt"] == 0.25
    assert abs(h["va_max"] - 1e6) < 1e-6
    b = muram_io.read_backup(str(tmp_path))
    assert b == dict(iter=7, time=12.5, p_bc=1.5e5, s_bc=-2e9)


def test_header_and_backup_text_format(tmp_path):
    """Byte layout of WriteHeaderFile's "%d  %d  %d  %f ..." and
    WriteBackupFile's "%d  %.16lg  %lg  %lg"."""
    muram_io.write_header(str(tmp_path), 3, (192, 64, 64), (3.2e6, 9.6e6, 9.6e6), 1.35429, 0.135432, 1.0 / 28726091.32118 ** 2)
    txt = (tmp_path / "Header.000003").read_text()
    assert txt == "192  64  64  3200000.000000  9600000.000000  9600000.000000  1.354290  0.135432  28726091.321180"
    muram_io.write_backup(str(tmp_path), 20, 2.708284890110555, 6.19644e+06, 9.78209e+08)
    assert (tmp_path / "backup.dat").read_text() == "20  2.708284890110555  6.19644e+06  9.78209e+08"


def test_sflx_variable(tmp_path):
    U = _box(seed=9)
    s = np.random.default_rng(1).standard_normal(U.shape[1:])
    muram_io.write_result(U, str(tmp_path), 0, (1.0, 1.0, 1.0), sflx=s)
    R, S = muram_io.read_result(str(tmp_path), 0, with_sflx=True)
    assert np.array_equal(S[2:-2, 2:-2, 2:-2], s[2:-2, 2:-2, 2:-2].astype(np.float32).astype(np.float64))
    with pytest.raises(ValueError):
        muram_io.read_prims(str(tmp_path), 0, (13, 10, 8))


def test_output_of_restored_state_is_stable(tmp_path):
    """write -> read -> write reproduces the files: the density, velocity and
    field exactly, the internal energy to float32 rounding."""
    U = _box(seed=11)
    a, b = tmp_path / "a", tmp_path / "b"
    muram_io.write_result(U, str(a), 1, (1.0, 1.0, 1.0))
    muram_io.write_result(muram_io.read_result(str(a), 1), str(b), 1, (1.0, 1.0, 1.0))
    Pa = muram_io.read_prims(str(a), 1, (12, 10, 8))
    Pb = muram_io.read_prims(str(b), 1, (12, 10, 8))
    for v in (0, 1, 2, 3, 5, 6, 7):
        assert np.array_equal(Pa[v], Pb[v]), v
    assert rel_linf(Pb[4:5], Pa[4:5])[0] < 1e-6


@pytest.mark.skipif(not os.path.isdir(REF_TEST3D), reason="reference TEST fixtures not present")
@pytest.mark.parametrize("it", [0, 10, 20])
def test_reads_reference_test3d_outputs(tmp_path, it):
    """The reference's own 3-D test outputs (192x64x64, Spitzer on: 9
    variables) read back, and written again, byte for byte where the
    conversion is exact."""
    d = os.path.join(REF_TEST3D, "3D")
    h = muram_io.read_header(d, it)
    assert (h["nx"], h["ny"], h["nz"]) == (192, 64, 64)
    assert h["dx"] == (3.2e6, 9.6e6, 9.6e6)
    U, S = muram_io.read_result(d, it, with_sflx=True)
    Ui = U[:, 2:-2, 2:-2, 2:-2]
    assert np.all(np.isfinite(Ui)) and np.all(Ui[0] > 0)
    raw = np.fromfile(os.path.join(d, f"result_prim_0.{it:06d}"), dtype="<f4").reshape(64, 64, 192)
    assert np.array_equal(Ui[0], raw.astype(np.float64))
    # x (dim 0, the vertical) is the fastest file axis: the mean density falls with height
    prof = raw.mean(axis=(0, 1))
    assert prof[0] > 100 * prof[-1]
    out = tmp_path / "out"
    muram_io.write_result(U, str(out), it, h["dx"], time=h["time"], dt=h["dt"],
                          inv_va2max=1.0 / max(h["va_max"], 1.0) ** 2, sflx=S, backup=False)
    for v in (0, 1, 2, 3, 5, 6, 7, 8):
        a = open(os.path.join(d, f"result_prim_{v}.{it:06d}"), "rb").read()
        b = (out / f"result_prim_{v}.{it:06d}").read_bytes()
        assert a == b, v
    P0 = muram_io.read_prims(d, it, (192, 64, 64), nvar=5)[4].astype(np.float64)
    P1 = muram_io.read_prims(str(out), it, (192, 64, 64), nvar=5)[4].astype(np.float64)
    assert np.max(np.abs(P1 - P0)) <= 1e-6 * np.max(np.abs(P0))
    if it > 0:
        h2 = muram_io.read_header(str(out), it)
        assert abs(h2["time"] - h["time"]) < 1e-6 and abs(h2["va_max"] - h["va_max"]) < 1e-3


@pytest.mark.skipif(not os.path.isdir(REF_TEST3D), reason="reference TEST fixtures not present")
def test_reads_reference_backup_file():
    b = muram_io.read_backup(REF_TEST3D)
    assert b["iter"] == 20
    assert abs(b["time"] - 2.708284890110555) < 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_output_restore_through_gpu_context(gpu_lib, tmp_path, precision):
    """OutputSolution after fused steps writes the downloaded state;
    RestoreSolution uploads it again, with ghosts filled and the time set."""
    from helpers import gpu_params, load_case
    from muram_main_gb300 import gpumhd
    from muram_main_gb300.initial import fill_ghosts
    d, hp = load_case("periodic")
    p = gpu_params(hp, precision)
    g = gpumhd.MuramGPU(p, eos_path=EOS_SMALL)
    g.upload_state(d["input_U"])
    dts = g.run_steps(3)
    U = g.download_state()
    g.OutputSolution(str(tmp_path), 3)
    P = muram_io.read_prims(str(tmp_path), 3, (p.nx, p.ny, p.nz))
    assert np.array_equal(P, muram_io.conserved_to_output(U).astype(np.float32))
    h = muram_io.read_header(str(tmp_path), 3)
    assert abs(h["time"] - float(np.sum(dts))) <= 1e-6 * max(1.0, h["time"])
    g.close()
    g2 = gpumhd.MuramGPU(gpu_params(hp, precision), eos_path=EOS_SMALL)
    t = g2.RestoreSolution(str(tmp_path), 3)
    assert abs(t - float(np.sum(dts))) <= 1e-12 * max(1.0, t)
    R = g2.download_state()
    expect = fill_ghosts(muram_io.read_result(str(tmp_path), 3), periodic_x=True)
    tol = 0.0 if precision == 64 else 1e-6
    assert np.all(rel_linf(R, expect) <= tol)
    assert g2.step_info()[2] == t
    g2.close()
