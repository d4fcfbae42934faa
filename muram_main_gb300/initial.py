"""Seeded synthetic initial states for the benchmark boxes.

The reference starts runs only from restart files (src/driver.C:57-67), so the
benchmark states are generated here, identically for the CPU oracle and the
GPU path.  Layout: float64 array of shape (8, nz+4, ny+4, nx+4) holding the
conserved variables (rho, M_x, M_y, M_z, e, B_x, B_y, B_z) with two ghost
layers on each side; MURaM's dimension 0 (x, vertical) is the fastest index
(src/grid.C:197-199).  B is in code units, B_code = B_gauss / sqrt(4 pi)
(src/boundary_pdmp_1_fftw3.C:95).

e holds internal + kinetic energy; magnetic energy is not included
(src/cons_to_prim.C:157).
"""
from __future__ import annotations

import math
import struct

import numpy as np

GHOSTS = 2
B_UNIT = math.sqrt(4.0 * math.pi)


class EosTable:
    """Host copy of an EOS table, pre-scaled exactly as eos_init does.

    Follows src/eos_init.C:80-198: the axes are built in double precision from
    the float header; each float table entry is divided by del_eps*del_lr in
    double precision and stored back as float32.
    """

    def __init__(self, path):
        with open(path, "rb") as fh:
            raw = fh.read()
        h = struct.unpack("<14f", raw[:56])
        self.N_eps, self.N_lr, self.N_lp3, self.N_s3 = (int(h[0]), int(h[1]), int(h[2]), int(h[3]))
        eps0, eps1, lr0, lr1, lp0, lp1, s0, s1 = (float(v) for v in h[4:12])
        self.eps_off = float(h[12])
        self.ss_off = float(h[13])
        self.header = h
        ne, nr = self.N_eps, self.N_lr
        self.del_eps = (eps1 - eps0) / float(ne - 1)
        self.del_lr = (lr1 - lr0) / float(nr - 1)
        self.inv_del_eps = 1.0 / self.del_eps
        self.inv_del_lr = 1.0 / self.del_lr
        self.xeps = eps0 + self.del_eps * np.arange(ne, dtype=np.float64)
        self.xlr = lr0 + self.del_lr * np.arange(nr, dtype=np.float64)
        self.del_lp3 = (lp1 - lp0) / float(self.N_lp3 - 1)
        self.del_s3 = (s1 - s0) / float(self.N_s3 - 1)
        self.xlp3 = lp0 + self.del_lp3 * np.arange(self.N_lp3, dtype=np.float64)
        self.xs3 = s0 + self.del_s3 * np.arange(self.N_s3, dtype=np.float64)
        off = 56
        tabs = np.frombuffer(raw, dtype="<f4", count=6 * ne * nr, offset=off).reshape(6, nr, ne)
        off += 6 * ne * nr * 4
        inv = np.frombuffer(raw, dtype="<f4", count=2 * self.N_lp3 * self.N_s3, offset=off)
        inv = inv.reshape(2, self.N_s3, self.N_lp3)
        scale = self.del_eps * self.del_lr
        # [table][i_eps][j_rho] like p_eostab[i][j]
        self.tables = (tabs.astype(np.float64) / scale).astype(np.float32).transpose(0, 2, 1).copy()
        scale3 = self.del_lp3 * self.del_s3
        self.inv_tables = (inv.astype(np.float64) / scale3).astype(np.float32).transpose(0, 2, 1).copy()

    def T_interp(self, ee, dd):
        """Scalar temperature lookup restated from src/eos_init.C:292-316."""
        ee1 = math.log(ee + self.eps_off)
        logr = math.log(dd)
        i = int((ee1 - self.xeps[0]) * self.inv_del_eps)
        i = min(max(i, 0), self.N_eps - 2)
        j = int((logr - self.xlr[0]) * self.inv_del_lr)
        j = min(max(j, 0), self.N_lr - 2)
        T = self.tables[1]
        x = self.xeps
        y = self.xlr
        v = ((logr - y[j]) * (ee1 - x[i]) * float(T[i + 1, j + 1])
             + (logr - y[j]) * (x[i + 1] - ee1) * float(T[i, j + 1])
             + (y[j + 1] - logr) * (ee1 - x[i]) * float(T[i + 1, j])
             + (y[j + 1] - logr) * (x[i + 1] - ee1) * float(T[i, j]))
        return math.exp(v)

    def p_interp(self, ee, dd):
        """Scalar pressure lookup restated from src/eos_init.C:319-343."""
        ee1 = math.log(ee + self.eps_off)
        logr = math.log(dd)
        i = int((ee1 - self.xeps[0]) * self.inv_del_eps)
        i = min(max(i, 0), self.N_eps - 2)
        j = int((logr - self.xlr[0]) * self.inv_del_lr)
        j = min(max(j, 0), self.N_lr - 2)
        P = self.tables[0]
        x = self.xeps
        y = self.xlr
        v = ((logr - y[j]) * (ee1 - x[i]) * float(P[i + 1, j + 1])
             + (logr - y[j]) * (x[i + 1] - ee1) * float(P[i, j + 1])
             + (y[j + 1] - logr) * (ee1 - x[i]) * float(P[i + 1, j])
             + (y[j + 1] - logr) * (x[i + 1] - ee1) * float(P[i, j]))
        return math.exp(v)

    def eint_for_T(self, T, rho, lo=1.0e10, hi=1.0e15):
        """Specific internal energy giving temperature T at density rho (bisection on T_interp)."""
        for _ in range(200):
            mid = 0.5 * (lo + hi)
            if self.T_interp(mid, rho) < T:
                lo = mid
            else:
                hi = mid
            if hi - lo <= 1e-13 * hi:
                break
        return 0.5 * (lo + hi)


def _shell_field(shape_zyx, kmin, kmax, rng):
    """Real random field with integer wavenumbers kmin <= |k| <= kmax and random phases."""
    nz, ny, nx = shape_zyx
    kz = np.fft.fftfreq(nz, 1.0 / nz)[:, None, None]
    ky = np.fft.fftfreq(ny, 1.0 / ny)[None, :, None]
    kx = np.fft.rfftfreq(nx, 1.0 / nx)[None, None, :]
    kk = np.sqrt(kx * kx + ky * ky + kz * kz)
    mask = (kk >= kmin) & (kk <= kmax)
    ph = rng.uniform(0.0, 2.0 * np.pi, size=mask.shape)
    amp = rng.standard_normal(size=mask.shape) ** 2 + 0.5
    spec = np.where(mask, amp * np.exp(1j * ph), 0.0)
    return np.fft.irfftn(spec, s=(nz, ny, nx), axes=(0, 1, 2))


def _d4(f, axis, dx):
    """4th-order central derivative on a periodic array (the residual's stencil)."""
    w1 = 8.0 / (12.0 * dx)
    w2 = -1.0 / (12.0 * dx)
    return (w1 * (np.roll(f, -1, axis) - np.roll(f, 1, axis))
            + w2 * (np.roll(f, -2, axis) - np.roll(f, 2, axis)))


def fill_ghosts(U, periodic_x=True):
    """Fill the two ghost layers: periodic in y and z, periodic or mirrored in x.

    The mirror ("closed") rule flips M_x, B_y, B_z, like the reference's closed
    top boundary (src/boundary_pdmp_1_fftw3.C:415-447) applied at both ends."""
    g = GHOSTS
    # x (last axis)
    if periodic_x:
        U[..., :g] = U[..., -2 * g:-g]
        U[..., -g:] = U[..., g:2 * g]
    else:
        sign = np.array([1, -1, 1, 1, 1, 1, -1, -1], dtype=U.dtype)[:, None, None, None]
        for gg in range(1, g + 1):
            U[..., g - gg] = U[..., g - 1 + gg] * sign[..., 0]
            U[..., -g - 1 + gg] = U[..., -g - gg] * sign[..., 0]
    # y
    U[:, :, :g, :] = U[:, :, -2 * g:-g, :]
    U[:, :, -g:, :] = U[:, :, g:2 * g, :]
    # z
    U[:, :g, :, :] = U[:, -2 * g:-g, :, :]
    U[:, -g:, :, :] = U[:, g:2 * g, :, :]
    return U


def periodic_box(eos, nx, ny, nz, dx=3.2e6, rho0=3e-7, T0=6000.0, v_rms=1.0e5,
                 b_rms_gauss=100.0, kmin=1, kmax=8, seed=1234, dy=None, dz=None):
    """Uniform-density periodic box with a random solenoidal-plus-compressive velocity
    and a divergence-free random field (curl of a random vector potential)."""
    dy = dx if dy is None else dy
    dz = dx if dz is None else dz
    rng = np.random.default_rng(seed)
    shp = (nz, ny, nx)
    v = np.stack([_shell_field(shp, kmin, kmax, rng) for _ in range(3)])
    v *= v_rms / math.sqrt(float(np.mean(np.sum(v * v, axis=0))))
    A = np.stack([_shell_field(shp, kmin, kmax, rng) for _ in range(3)])
    # B = curl A with the residual's 4th-order central operator; axis 2 = x, 1 = y, 0 = z
    Ax, Ay, Az = A
    Bx = _d4(Az, 1, dy) - _d4(Ay, 0, dz)
    By = _d4(Ax, 0, dz) - _d4(Az, 2, dx)
    Bz = _d4(Ay, 2, dx) - _d4(Ax, 1, dy)
    B = np.stack([Bx, By, Bz])
    B *= (b_rms_gauss / B_UNIT) / math.sqrt(float(np.mean(np.sum(B * B, axis=0))))
    eint = eos.eint_for_T(T0, rho0)
    U = np.zeros((8, nz + 4, ny + 4, nx + 4), dtype=np.float64)
    s = (slice(GHOSTS, -GHOSTS),) * 3
    rho = np.full(shp, rho0)
    U[(0,) + s] = rho
    for c in range(3):
        U[(1 + c,) + s] = rho * v[c]
        U[(5 + c,) + s] = B[c]
    U[(4,) + s] = rho * eint + 0.5 * rho * np.sum(v * v, axis=0)
    return fill_ghosts(U, periodic_x=True)


def stratified_box(eos, nx, ny, nz, dx=1.6e6, rho_bot=3e-7, T0=1.0e4, grav=2.74e4,
                   v_rms=0.5e5, b_vert_gauss=50.0, b_rms_gauss=20.0, kmin=1, kmax=8, seed=4321):
    """Vertically stratified box (x vertical): rho decreases upward in near
    hydrostatic balance at temperature T0 under gravity grav, a uniform vertical
    field plus a random divergence-free component, and a random velocity.

    The density profile integrates dp/dh = -rho g with the tabulated pressure at
    fixed T0, cell by cell from the bottom."""
    rng = np.random.default_rng(seed)
    shp = (nz, ny, nx)
    # hydrostatic profile along x
    rho_x = np.empty(nx)
    e_x = np.empty(nx)
    rho = rho_bot
    for i in range(nx):
        eint = eos.eint_for_T(T0, rho)
        rho_x[i] = rho
        e_x[i] = eint
        p = eos.p_interp(eint, rho)
        # next cell: p_next = p - rho*g*dx with rho_next from p_next at fixed T (secant on rho)
        target = p - rho * grav * dx
        r_lo, r_hi = rho * 0.2, rho
        for _ in range(80):
            r_mid = math.sqrt(r_lo * r_hi)
            if eos.p_interp(eos.eint_for_T(T0, r_mid), r_mid) > target:
                r_hi = r_mid
            else:
                r_lo = r_mid
            if r_hi / r_lo - 1.0 < 1e-12:
                break
        rho = math.sqrt(r_lo * r_hi)
    v = np.stack([_shell_field(shp, kmin, kmax, rng) for _ in range(3)])
    # taper the vertical velocity to zero at the closed boundaries
    taper = np.sin(np.pi * (np.arange(nx) + 0.5) / nx)[None, None, :]
    v[0] *= taper
    v *= v_rms / math.sqrt(float(np.mean(np.sum(v * v, axis=0))))
    A = np.stack([_shell_field(shp, kmin, kmax, rng) for _ in range(3)])
    Ax, Ay, Az = A
    Bx = _d4(Az, 1, dx) - _d4(Ay, 0, dx)
    By = _d4(Ax, 0, dx) - _d4(Az, 2, dx)
    Bz = _d4(Ay, 2, dx) - _d4(Ax, 1, dx)
    B = np.stack([Bx, By, Bz])
    B *= (b_rms_gauss / B_UNIT) / math.sqrt(float(np.mean(np.sum(B * B, axis=0))))
    B[0] += b_vert_gauss / B_UNIT
    U = np.zeros((8, nz + 4, ny + 4, nx + 4), dtype=np.float64)
    s = (slice(GHOSTS, -GHOSTS),) * 3
    rho3 = np.broadcast_to(rho_x[None, None, :], shp)
    U[(0,) + s] = rho3
    for c in range(3):
        U[(1 + c,) + s] = rho3 * v[c]
        U[(5 + c,) + s] = B[c]
    U[(4,) + s] = rho3 * e_x[None, None, :] + 0.5 * rho3 * np.sum(v * v, axis=0)
    return fill_ghosts(U, periodic_x=False)


def soa_to_aos(U):
    """(8, sz, sy, sx) -> contiguous cState array (sz, sy, sx, 8)."""
    return np.ascontiguousarray(np.moveaxis(U, 0, -1))


def aos_to_soa(A, shape_zyx):
    """Inverse of soa_to_aos for a flat float64 buffer."""
    sz, sy, sx = shape_zyx
    return np.ascontiguousarray(np.moveaxis(A.reshape(sz, sy, sx, 8), -1, 0))
