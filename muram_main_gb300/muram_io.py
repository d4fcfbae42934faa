"""MURaM result / restart files: read and write the reference's format.

Files of one output at iteration ``it`` in directory ``path``:

* ``{resfile}_prim_{v}.{it:06d}``: float32 interior arrays, x (dim 0, vertical)
  fastest, then y, then z.  v = 0..7 hold rho, v_x, v_y, v_z, e_int (per
  volume), B_x, B_y, B_z; with Spitzer conduction on, v = 8 holds the heat
  flux ``sflx`` (src/io_xysl.C:99-209; the primitive conversion is at
  :149-154, the ninth variable at :163-165);
* ``Header.{it:06d}``: ``nx ny nz dx dy dz time dt va_max`` as text
  (WriteHeaderFile, src/io_xysl.C:39-48, va_max = 1/sqrt(inv_va2max));
* ``backup.dat``: ``iter time p_bc s_bc`` (WriteBackupFile / ReadBackupFile,
  src/boundary_pdmp_1_fftw3.C:44-62).

Writing forms the primitives in float64 and casts each value to float32, as
OutputSolution does.  Reading converts back to conserved variables in
RestoreSolution's order (src/io_xysl.C:401-406): e += 0.5*|v|^2*rho, then
M = rho*v.

States are this package's (8, nz+4, ny+4, nx+4) float64 arrays with two ghost
layers (array axis order z, y, x, so x is fastest in memory as in the files);
only the interior is written or read.
"""
from __future__ import annotations

import os

import numpy as np

G = 2


def prim_name(path, resfile, var, it):
    return os.path.join(path, f"{resfile}_prim_{var}.{it:06d}")


def conserved_to_output(U):
    """Interior primitives as OutputSolution forms them in float64 before the
    cast: v = M / rho, e_int = e - 0.5*rho*|v|^2 (src/io_xysl.C:149-154)."""
    Ui = np.asarray(U, dtype=np.float64)[:, G:-G, G:-G, G:-G]
    d = Ui[0]
    v = Ui[1:4] / d
    sqr = v[0] * v[0] + v[1] * v[1] + v[2] * v[2]
    ei = Ui[4] - 0.5 * d * sqr
    return np.stack([d, v[0], v[1], v[2], ei, Ui[5], Ui[6], Ui[7]])


def output_to_conserved(P):
    """Inverse of conserved_to_output on float64 interior arrays, in
    RestoreSolution's operation order (src/io_xysl.C:401-406)."""
    Q = np.array(P[:8], dtype=np.float64)
    d = Q[0]
    sqr = Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]
    Q[4] += 0.5 * sqr * d
    Q[1:4] *= d
    return Q


def write_header(path, it, shape_xyz, dx, time, dt, inv_va2max):
    nx, ny, nz = shape_xyz
    with open(os.path.join(path, f"Header.{it:06d}"), "w") as fh:
        fh.write("%d  %d  %d  %f  %f  %f  %f  %f  %f" % (nx, ny, nz, dx[0], dx[1], dx[2], time, dt,
                                                          1.0 / np.sqrt(inv_va2max)))


def write_backup(path, it, time, p_bc=0.0, s_bc=0.0, name="backup.dat"):
    """``%d  %.16lg  %lg  %lg`` as WriteBackupFile prints it."""
    with open(os.path.join(path, name), "w") as fh:
        fh.write("%d  %.16g  %g  %g" % (it, time, p_bc, s_bc))


def write_result(U, path, it, dx, time=0.0, dt=0.0, inv_va2max=1e-14, resfile="result", sflx=None,
                 p_bc=0.0, s_bc=0.0, backup=True):
    """Write the result_prim files, the Header and (optionally) backup.dat of
    one output.  ``sflx``: optional (nz+4, ny+4, nx+4) heat flux, written as
    variable 8 as the reference does when Spitzer conduction is on."""
    os.makedirs(path, exist_ok=True)
    P = conserved_to_output(U).astype(np.float32)
    for v in range(8):
        P[v].astype("<f4").tofile(prim_name(path, resfile, v, it))
    if sflx is not None:
        s = np.asarray(sflx, dtype=np.float64)[G:-G, G:-G, G:-G].astype(np.float32)
        s.astype("<f4").tofile(prim_name(path, resfile, 8, it))
    nz, ny, nx = P.shape[1:]
    write_header(path, it, (nx, ny, nz), dx, time, dt, inv_va2max)
    if backup:
        write_backup(path, it, time, p_bc, s_bc)


def read_header(path, it):
    with open(os.path.join(path, f"Header.{it:06d}")) as fh:
        parts = fh.read().split()
    nx, ny, nz = (int(float(p)) for p in parts[:3])
    dx = tuple(float(p) for p in parts[3:6])
    time, dt, va_max = (float(p) for p in parts[6:9])
    return dict(nx=nx, ny=ny, nz=nz, dx=dx, time=time, dt=dt, va_max=va_max)


def read_backup(path, name="backup.dat"):
    """(iter, time, p_bc, s_bc) as ReadBackupFile reads them."""
    with open(os.path.join(path, name)) as fh:
        parts = fh.read().split()
    return dict(iter=int(parts[0]), time=float(parts[1]), p_bc=float(parts[2]), s_bc=float(parts[3]))


def read_prims(path, it, shape_xyz, resfile="result", nvar=8):
    """The float32 interior arrays, shape (nvar, nz, ny, nx)."""
    nx, ny, nz = shape_xyz
    n = nx * ny * nz
    out = np.empty((nvar, nz, ny, nx), dtype=np.float32)
    for v in range(nvar):
        a = np.fromfile(prim_name(path, resfile, v, it), dtype="<f4")
        if a.size != n:
            raise ValueError(f"{prim_name(path, resfile, v, it)}: {a.size} values, expected {n}")
        out[v] = a.reshape(nz, ny, nx)
    return out


def read_result(path, it, resfile="result", shape_xyz=None, with_sflx=False):
    """Read one output into a conserved float64 state with (unfilled) ghosts.

    Returns U, or (U, sflx) when ``with_sflx`` (variable 8 present)."""
    if shape_xyz is None:
        h = read_header(path, it)
        shape_xyz = (h["nx"], h["ny"], h["nz"])
    nx, ny, nz = shape_xyz
    P = read_prims(path, it, shape_xyz, resfile, nvar=9 if with_sflx else 8).astype(np.float64)
    U = np.zeros((8, nz + 2 * G, ny + 2 * G, nx + 2 * G))
    U[:, G:-G, G:-G, G:-G] = output_to_conserved(P)
    if not with_sflx:
        return U
    s = np.zeros((nz + 2 * G, ny + 2 * G, nx + 2 * G))
    s[G:-G, G:-G, G:-G] = P[8]
    return U, s
