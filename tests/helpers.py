"""Shared helpers of the test suite (fixtures, parameter mapping, error norms)."""
from __future__ import annotations

import os
import sys

import numpy as np

TESTS = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(TESTS)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(TESTS, "golden")
EOS_SMALL = os.path.join(GOLDEN, "eos_small.dat")
CASES = ["periodic", "closed_gravity", "two_half_tvd"]


def load_case(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    hp = {k[6:]: d[k].item() for k in d if k.startswith("param_")}
    return d, hp


def oracle_params(hp):
    from oracle import oracle as O
    return O.params_from_harness(hp)


def gpu_params(hp, precision=64):
    from muram_main_gb300 import gpumhd
    kw = {}
    for k in ("CFL", "CFL_tvd", "grav", "eta", "divB_err", "bnd_bcrit", "bnd_eps_top", "p_bc", "s_bc", "spitzer",
              "va_max", "va_adjust", "max_fill"):
        if k in hp:
            kw[k] = float(hp[k])
    for k in ("divB_switch", "divB_itmax", "xbnd", "bnd_top"):
        if k in hp:
            kw[k] = int(hp[k])
    dx = float(hp.get("dx", 3.2e6))
    kw["dy"] = float(hp.get("dy", dx))
    kw["dz"] = float(hp.get("dz", dx))
    p = gpumhd.default_params(int(hp["nx"]), int(hp["ny"]), int(hp["nz"]), dx, precision=precision,
                              periodic_x=int(hp.get("periodic_x", 1)), **kw)
    for i, k in enumerate(("tchk_eps_min", "tchk_rho_min", "tchk_eps_max", "tchk_vmax")):
        if k in hp:
            p.tchk[i] = float(hp[k])
    return p


def rel_linf(a, b, axis_fields=True):
    """max |a-b| / max |b| per leading field (array of shape (F, ...))."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if not axis_fields:
        a, b = a[None], b[None]
    out = []
    for f in range(b.shape[0]):
        den = np.max(np.abs(b[f]))
        num = np.max(np.abs(a[f] - b[f]))
        out.append(0.0 if num == 0 else num / (den if den > 0 else 1.0))
    return np.array(out)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    out = []
    for f in range(b.shape[0]):
        den = np.sqrt(np.sum(b[f] ** 2))
        num = np.sqrt(np.sum((a[f] - b[f]) ** 2))
        out.append(0.0 if num == 0 else num / (den if den > 0 else 1.0))
    return np.array(out)


def interior(U):
    return U[..., 2:-2, 2:-2, 2:-2]
