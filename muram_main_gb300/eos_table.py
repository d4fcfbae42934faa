"""Tabulated equation of state in the binary layout MURaM's ``eos_init`` reads.

MURaM looks up p, T, s, n_e, rho_i and the ion-neutral collision frequency in
float tables over (ln eps, ln rho), where eps = e_int/rho + eps_off
(src/eos_init.C:57-212).  The file layout is:

* 14 float32 header words: N_eps, N_lr, N_lp3, N_s3, eps0, eps1, lr0, lr1,
  lp0, lp1, s0, s1, eps_off, ss_off            (src/eos_init.C:80-101)
* 6 float32 tables of N_eps*N_lr values, eps index fastest
  (index j*N_eps + i): ln p, ln T, s + ss_off, ln n_e, ln rho_i, ln nu_in
                                               (src/eos_init.C:155-177)
* 2 float32 inverse tables of N_lp3*N_s3 values, ln p index fastest:
  ln(eps) and ln(rho) as functions of (ln p, s + ss_off)
                                               (src/eos_init.C:181-198)

The reference's production tables (Uppsala / Wittmann) are large binary
inputs that are not part of the source tree, so this module computes a table
of its own from a published textbook model: an ideal gas of hydrogen
(mass fraction X) and helium (Y), with hydrogen ionisation in Saha
equilibrium and a small fully ionised metal electron background
(fraction ``EPS_METAL`` of n_H).  Entropy is the Sackur-Tetrode sum over
species, which is the thermodynamically consistent partner of the Saha
equation.  The physics only has to be smooth, monotonic and realistic near
the photosphere (rho ~ 3e-7 g/cm^3, T ~ 6000 K gives c_s ~ 8 km/s); the hot
path only interpolates.
"""
from __future__ import annotations

import hashlib
import os
import struct

import numpy as np

# cgs constants
K_B = 1.380649e-16
M_H = 1.6735575e-24
M_U = 1.66053907e-24
M_HE = 4.002602 * M_U
M_E = 9.1093837e-28
H_PL = 6.62607015e-27
CHI_H = 13.598434 * 1.602176634e-12
X_H = 0.7
Y_HE = 0.3
EPS_METAL = 1.0e-4
SIGMA_IN = 5.0e-15


def _species(rho, T):
    """Number densities for given rho [g/cm^3] and T [K] (broadcasting)."""
    nH = X_H * rho / M_H
    nHe = Y_HE * rho / M_HE
    lam = (2.0 * np.pi * M_E * K_B * T / H_PL**2) ** 1.5
    a = lam * np.exp(-CHI_H / (K_B * T)) / nH
    b = EPS_METAL + a
    x = 2.0 * a / (b + np.sqrt(b * b + 4.0 * a))
    x = np.clip(x, 0.0, 1.0)
    return nH, nHe, x


def state_rho_T(rho, T):
    """Return dict of e (erg/g), p, s (erg/g/K), ne, rhoi, nu_in at (rho, T)."""
    nH, nHe, x = _species(rho, T)
    ne = (x + EPS_METAL) * nH
    n_tot = nH * (1.0 + x) + nHe + EPS_METAL * nH
    p = n_tot * K_B * T
    e = (1.5 * n_tot * K_B * T + x * nH * CHI_H) / rho

    lnT = np.log(T)

    def st(n, m, g):
        n = np.maximum(n, 1e-300)
        lnq = np.log(g) + 1.5 * (np.log(2.0 * np.pi * m * K_B / H_PL**2) + lnT) - np.log(n)
        return n * K_B * (lnq + 2.5)

    s = (st((1.0 - x) * nH, M_H, 2.0) + st(x * nH, M_H, 1.0)
         + st(ne, M_E, 2.0) + st(nHe, M_HE, 1.0)) / rho
    rhoi = np.maximum(x * nH * M_H, 1e-40)
    n_n = (1.0 - x) * nH + nHe
    nu_in = np.maximum(n_n * SIGMA_IN * np.sqrt(8.0 * K_B * T / (np.pi * 0.5 * M_H)), 1e-30)
    return {"e": e, "p": p, "s": s, "ne": ne, "rhoi": rhoi, "nu_in": nu_in}


def _e_rho_T(rho, T):
    """Specific internal energy only (the quantity bisected on)."""
    nH, nHe, x = _species(rho, T)
    n_tot = nH * (1.0 + x) + nHe + EPS_METAL * nH
    return (1.5 * n_tot * K_B * T + x * nH * CHI_H) / rho


def _T_from_e(rho, e_target, lnT_lo=np.log(500.0), lnT_hi=np.log(5.0e7), iters=34):
    """Invert e(rho, T) = e_target for T by bisection in ln T (e is monotone in T).

    34 halvings of the 11.5-wide ln T bracket resolve ln T to 7e-10, far below
    the float32 resolution of the stored table values."""
    lo = np.full(np.broadcast(rho, e_target).shape, lnT_lo)
    hi = np.full_like(lo, lnT_hi)
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        em = _e_rho_T(rho, np.exp(mid))
        up = em < e_target
        lo = np.where(up, mid, lo)
        hi = np.where(up, hi, mid)
    return np.exp(0.5 * (lo + hi))


def generate(n_eps=3000, n_lr=3000, n_lp3=400, n_s3=300,
             e_min=1.5e11, e_max=2.0e15, eps_off=5.0e10,
             rho_min=1.0e-16, rho_max=1.0e-3, ss_off=None):
    """Compute the table arrays.  Returns (header list, tables dict)."""
    eps0 = float(np.float32(np.log(e_min + eps_off)))
    eps1 = float(np.float32(np.log(e_max + eps_off)))
    lr0 = float(np.float32(np.log(rho_min)))
    lr1 = float(np.float32(np.log(rho_max)))
    xeps = np.linspace(eps0, eps1, n_eps)
    xlr = np.linspace(lr0, lr1, n_lr)
    E, LR = np.meshgrid(np.exp(xeps) - eps_off, np.exp(xlr), indexing="xy")  # shape (n_lr, n_eps)
    T = _T_from_e(LR, E)
    st = state_rho_T(LR, T)
    if ss_off is None:
        ss_off = float(np.float32(-np.median(st["s"])))
    tabs = {
        "p": np.log(st["p"]),
        "T": np.log(T),
        "s": st["s"] + ss_off,
        "ne": np.log(st["ne"]),
        "rhoi": np.log(st["rhoi"]),
        "amb": np.log(st["nu_in"]),
    }
    # inverse tables over (ln p, s+ss_off): find (rho, T) by damped Newton in (ln rho, ln T)
    lp_lo, lp_hi = np.percentile(tabs["p"], [5, 95])
    s_lo, s_hi = np.percentile(tabs["s"], [5, 95])
    lp0, lp1 = float(np.float32(lp_lo)), float(np.float32(lp_hi))
    s0, s1 = float(np.float32(s_lo)), float(np.float32(s_hi))
    xlp = np.linspace(lp0, lp1, n_lp3)
    xs = np.linspace(s0, s1, n_s3)
    LP, S = np.meshgrid(xlp, xs, indexing="xy")  # (n_s3, n_lp3)
    s_target = S - ss_off
    lnT = np.full(LP.shape, np.log(8000.0))
    lnr = LP - np.log(K_B * 8000.0 / (1.3 * M_H))
    for _ in range(60):
        def f(lr_, lt_):
            q = state_rho_T(np.exp(lr_), np.exp(lt_))
            return np.log(q["p"]) - LP, (q["s"] - s_target) * 1e-8
        f0p, f0s = f(lnr, lnT)
        h = 1e-6
        fr_p, fr_s = f(lnr + h, lnT)
        ft_p, ft_s = f(lnr, lnT + h)
        a11, a12 = (fr_p - f0p) / h, (ft_p - f0p) / h
        a21, a22 = (fr_s - f0s) / h, (ft_s - f0s) / h
        det = a11 * a22 - a12 * a21
        det = np.where(np.abs(det) < 1e-300, 1e-300, det)
        dr = (a22 * f0p - a12 * f0s) / det
        dt_ = (-a21 * f0p + a11 * f0s) / det
        lnr = np.clip(lnr - np.clip(dr, -1.0, 1.0), np.log(rho_min), np.log(rho_max))
        lnT = np.clip(lnT - np.clip(dt_, -0.5, 0.5), np.log(500.0), np.log(5e7))
    e_inv = state_rho_T(np.exp(lnr), np.exp(lnT))["e"]
    inv = {"eps3": np.log(np.maximum(e_inv + eps_off, 1.0)), "d3": lnr}
    header = [n_eps, n_lr, n_lp3, n_s3, eps0, eps1, lr0, lr1, lp0, lp1, s0, s1, eps_off, ss_off]
    return header, tabs, inv


def generate_ideal(n_eps=256, n_lr=256, n_lp3=64, n_s3=64, e_min=1.0e11, e_max=2.0e15, rho_min=1.0e-16,
                   rho_max=1.0e-3, gamma=5.0 / 3.0, mu=0.62):
    """An ideal-gas table (fixed mean molecular weight mu, eps_off = 0):
    p = (gamma-1) rho eps and T = (gamma-1) mu m_H eps / k_B, so ln p and ln T
    are linear in (ln eps, ln rho) and the bilinear lookup is exact and
    smooth -- no kinks at table nodes (used to check derivatives)."""
    eps_off = 0.0
    eps0 = float(np.float32(np.log(e_min)))
    eps1 = float(np.float32(np.log(e_max)))
    lr0 = float(np.float32(np.log(rho_min)))
    lr1 = float(np.float32(np.log(rho_max)))
    xeps = np.linspace(eps0, eps1, n_eps)
    xlr = np.linspace(lr0, lr1, n_lr)
    LE, LR = np.meshgrid(xeps, xlr, indexing="xy")
    lnp = np.log(gamma - 1.0) + LR + LE
    lnT = np.log((gamma - 1.0) * mu * M_H / K_B) + LE
    s_phys = K_B / (mu * M_H) * (1.5 * lnT - LR)  # Sackur-Tetrode up to a constant
    ss_off = float(np.float32(-np.median(s_phys)))
    tabs = {"p": lnp, "T": lnT, "s": s_phys + ss_off, "ne": LR - np.log(1.2 * M_H),
            "rhoi": LR, "amb": np.zeros_like(LR)}
    lp0, lp1 = float(np.float32(np.percentile(lnp, 5))), float(np.float32(np.percentile(lnp, 95)))
    s0, s1 = float(np.float32(np.percentile(tabs["s"], 5))), float(np.float32(np.percentile(tabs["s"], 95)))
    LP, S = np.meshgrid(np.linspace(lp0, lp1, n_lp3), np.linspace(s0, s1, n_s3), indexing="xy")
    # invert: ln p = c1 + ln rho + ln eps, s' = a (1.5 (c2 + ln eps) - ln rho)
    a = K_B / (mu * M_H)
    c1 = np.log(gamma - 1.0)
    c2 = np.log((gamma - 1.0) * mu * M_H / K_B)
    q = (S - ss_off) / a  # 1.5 (c2 + le) - lr
    le = (q + (LP - c1) - 1.5 * c2) / 2.5
    lr = LP - c1 - le
    inv = {"eps3": le, "d3": lr}
    header = [n_eps, n_lr, n_lp3, n_s3, eps0, eps1, lr0, lr1, lp0, lp1, s0, s1, eps_off, ss_off]
    return header, tabs, inv


def write_table(path, ideal=False, **kw):
    """Generate a table and write it in the eos_init binary layout; returns SHA-256."""
    header, tabs, inv = generate_ideal(**kw) if ideal else generate(**kw)
    blob = bytearray(struct.pack("<14f", *[float(h) for h in header]))
    for name in ("p", "T", "s", "ne", "rhoi", "amb"):
        blob += np.ascontiguousarray(tabs[name], dtype="<f4").tobytes()
    for name in ("eps3", "d3"):
        blob += np.ascontiguousarray(inv[name], dtype="<f4").tobytes()
    tmp = path + ".tmp"
    with open(tmp, "wb") as fh:
        fh.write(blob)
    os.replace(tmp, path)
    return hashlib.sha256(bytes(blob)).hexdigest()


def small_table_kwargs():
    """Parameters of the compact table used by the test fixtures."""
    return dict(n_eps=160, n_lr=128, n_lp3=40, n_s3=30,
                e_min=1.5e11, e_max=2.0e13, rho_min=1.0e-12, rho_max=1.0e-4)


def bench_table_kwargs():
    """Parameters of the full-resolution table (3000 x 3000 like the reference's tables)."""
    return dict(n_eps=3000, n_lr=3000, n_lp3=400, n_s3=300)


def ensure_table(path, kind="bench"):
    """Create the table at ``path`` if it does not exist yet (kind: "bench",
    "small" or "ideal")."""
    if not os.path.exists(path):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        if kind == "ideal":
            write_table(path, ideal=True)
        else:
            write_table(path, **(bench_table_kwargs() if kind == "bench" else small_table_kwargs()))
    return path


if __name__ == "__main__":
    import sys
    out = sys.argv[1] if len(sys.argv) > 1 else "eos_table.dat"
    kind = sys.argv[2] if len(sys.argv) > 2 else "bench"
    kw = bench_table_kwargs() if kind == "bench" else small_table_kwargs()
    print(write_table(out, **kw))
