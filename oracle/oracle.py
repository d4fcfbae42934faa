"""ctypes binding of the C restatement (oracle/muram_oracle.c).

Test infrastructure: the checker the GPU path is compared against.  Only
tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this module.  ``build()`` compiles the shared library with the
oracle's Makefile (gcc, -O2 -ffp-contract=off).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmuram_oracle.so")


class MoParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("periodic_x", C.c_int),
        ("dx", C.c_double * 3),
        ("CFL", C.c_double), ("CFL_tvd", C.c_double), ("dt", C.c_double), ("time", C.c_double),
        ("outcad", C.c_double), ("autostep", C.c_int),
        ("grav", C.c_double), ("va_max", C.c_double), ("va_adjust", C.c_double), ("max_fill", C.c_double),
        ("tvd_h", C.c_double * 4), ("tvd_cs", C.c_double * 4), ("tvd", C.c_double * 10),
        ("tvd_h_bnd", C.c_double * 2), ("tvd_visc_bnd", C.c_double * 2), ("tvd_eta_bnd", C.c_double * 2),
        ("tvd_coeff", C.c_double * 4), ("tchk", C.c_double * 4),
        ("rt_cfl", C.c_double), ("rt_tstep", C.c_double), ("rt_update", C.c_double),
        ("tau0", C.c_double), ("dt_rad", C.c_double),
        ("inv_va2max", C.c_double), ("v_lim", C.c_double), ("e_lim", C.c_double), ("va_max_old", C.c_double),
        ("va_ini_flag", C.c_int), ("last_cfl", C.c_double), ("tvd_two_half_steps", C.c_int),
        ("eta", C.c_double),
        ("divB_switch", C.c_int), ("divB_itmax", C.c_int), ("divB_err", C.c_double),
        ("divB_next_iter", C.c_int), ("divB_last_iters", C.c_int),
        ("divB_err0", C.c_double), ("divB_err1", C.c_double),
        ("xbnd", C.c_int), ("bnd_top", C.c_int),
        ("bnd_bcrit", C.c_double), ("bnd_eps_top", C.c_double), ("p_bc", C.c_double), ("s_bc", C.c_double),
        ("bnd_ini", C.c_int),
        ("spitzer", C.c_double),
        ("need_diagnostics", C.c_int), ("diagnostics_next_step", C.c_int), ("diag", C.c_void_p),
    ]


class MoFields(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in ("phi", "divB", "sflx", "sflx0", "Rflx", "BgradT")]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        P = C.POINTER(MoParams)
        L.mo_default_params.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_double]
        L.mo_eos_load.restype = C.c_void_p
        L.mo_eos_load.argtypes = [C.c_char_p]
        L.mo_eos_free.argtypes = [C.c_void_p]
        L.mo_save_cons.argtypes = [P, dp, dp]
        L.mo_cons_to_prim.argtypes = [P, C.c_void_p, dp, dp, dp, dp, dp, dp]
        L.mo_adjust_valf_max.argtypes = [P, dp, dp, dp]
        L.mo_mhd_residual.restype = C.c_double
        L.mo_mhd_residual.argtypes = [P, dp, dp, dp]
        L.mo_sync_timestep.restype = C.c_int
        L.mo_sync_timestep.argtypes = [P, C.c_double, C.c_double, C.POINTER(C.c_double)]
        L.mo_source_integrate_tcheck.argtypes = [P, dp, dp, dp, C.c_int]
        L.mo_boundaries.argtypes = [P, dp]
        L.mo_exchange_only.argtypes = [P, dp]
        L.mo_tvdlimit.argtypes = [P, dp, dp, C.c_double]
        L.mo_tcheck.argtypes = [P, dp]
        L.mo_step.restype = C.c_int
        L.mo_step.argtypes = [P, C.c_void_p, dp, dp, dp, dp]
        L.mo_clean_divB.argtypes = [P, dp, dp, dp]
        L.mo_boundaries_eos.argtypes = [P, C.c_void_p, dp]
        L.mo_step_ex.restype = C.c_int
        L.mo_step_ex.argtypes = [P, C.c_void_p, dp, dp, dp, dp, C.POINTER(MoFields)]
        L.mo_step_divb.restype = C.c_int
        L.mo_step_divb.argtypes = [P, C.c_void_p, dp, dp, dp, dp, dp, dp]
        _lib = L
    return _lib


class Eos:
    def __init__(self, path):
        self.ptr = lib().mo_eos_load(path.encode())
        if not self.ptr:
            raise OSError(f"cannot load EOS table {path}")

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.mo_eos_free(self.ptr)
            self.ptr = None


def make_params(nx, ny, nz, dx=3.2e6, dy=None, dz=None, periodic_x=True, **kw):
    p = MoParams()
    lib().mo_default_params(C.byref(p), nx, ny, nz, dx)
    p.dx[1] = dx if dy is None else dy
    p.dx[2] = dx if dz is None else dz
    p.periodic_x = 1 if periodic_x else 0
    for k, v in kw.items():
        if isinstance(v, (list, tuple)):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, k, v)
    return p


def params_from_harness(hp):
    """Build MoParams from the harness key/value dict used by oracle.refrun."""
    kw = {}
    simple = {"CFL": "CFL", "CFL_tvd": "CFL_tvd", "grav": "grav", "va_max": "va_max",
              "va_adjust": "va_adjust", "max_fill": "max_fill", "tau0": "tau0", "dt_rad": "dt_rad", "eta": "eta",
              "divB_err": "divB_err", "bnd_bcrit": "bnd_bcrit", "bnd_eps_top": "bnd_eps_top",
              "p_bc": "p_bc", "s_bc": "s_bc", "spitzer": "spitzer"}
    for k, a in simple.items():
        if k in hp:
            kw[a] = float(hp[k])
    for k in ("divB_switch", "divB_itmax", "xbnd", "bnd_top"):
        if k in hp:
            kw[k] = int(float(hp[k]))
    for k in ("tvd_h", "tvd_cs", "tvd_coeff", "tvd_h_bnd", "tvd_visc_bnd", "tvd_eta_bnd"):
        if k in hp:
            kw[k] = [float(x) for x in hp[k]]
    p = make_params(int(hp["nx"]), int(hp["ny"]), int(hp["nz"]), float(hp.get("dx", 3.2e6)),
                    float(hp.get("dy", hp.get("dx", 3.2e6))), float(hp.get("dz", hp.get("dx", 3.2e6))),
                    periodic_x=bool(int(hp.get("periodic_x", 1))), **kw)
    tvd_keys = ["tvd_rholev", "tvd_rholog", "tvd_qrho", "tvd_Bpar", "tvd_vhyp", "tvd_Qdiff_bnd",
                "tvd_pm_v", "tvd_pm_B", "tvd_vmax_lim", "tvd_CME_thresh"]
    for i, k in enumerate(tvd_keys):
        if k in hp:
            p.tvd[i] = float(hp[k])
    tchk_keys = ["tchk_eps_min", "tchk_rho_min", "tchk_eps_max", "tchk_vmax"]
    for i, k in enumerate(tchk_keys):
        if k in hp:
            p.tchk[i] = float(hp[k])
    return p


class State:
    """Scratch buffers for full steps on the oracle.  With divB cleaning on
    (p.divB_switch > 0), ``phi`` carries the cleaning potential from step to
    step, ``divB`` holds the last divergence and ``divb_log`` one entry
    (iterations, max|divB| before, after) per step.  ``limits_log`` holds
    Adjust_Valf_Max's (inv_va2max, v_lim, e_lim) after each step."""

    def __init__(self, p, U, eos=None):
        self.p = p
        self.U = np.ascontiguousarray(U, dtype=np.float64).copy()
        self.U0 = np.zeros_like(self.U)
        self.R = np.zeros_like(self.U)
        self.aux = np.zeros((5,) + self.U.shape[1:])
        self.phi = np.zeros(self.U.shape[1:])
        self.divB = np.zeros(self.U.shape[1:])
        self.sflx = np.zeros(self.U.shape[1:])
        self.sflx0 = np.zeros(self.U.shape[1:])
        self.Rflx = np.zeros(self.U.shape[1:])
        self.BgradT = np.zeros(self.U.shape[1:])
        ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._f = MoFields(ptr(self.phi), ptr(self.divB), ptr(self.sflx), ptr(self.sflx0), ptr(self.Rflx),
                           ptr(self.BgradT))
        self.divb_log = []
        self.limits_log = []
        # tvar1..tvar8, Qres, Qvis of the last step run with diagnostics
        self.diag = np.zeros((10,) + self.U.shape[1:])
        self.p.diag = self.diag.ctypes.data
        if p.xbnd == 1 and not p.periodic_x:
            if eos is None:
                raise ValueError("the physical x boundaries need the EOS (State(p, U, eos))")
            lib().mo_boundaries_eos(C.byref(p), eos.ptr, self.U)
        else:
            lib().mo_boundaries(C.byref(p), self.U)

    def step(self, eos, n=1, diagnostics_at=None):
        """n steps; diagnostics_at: the 1-based step among them whose
        diagnostics (an output step's) fill self.diag."""
        dts = []
        for s in range(n):
            self.p.diagnostics_next_step = 1 if diagnostics_at == s + 1 else 0
            rc = lib().mo_step_ex(C.byref(self.p), eos.ptr, self.U, self.U0, self.R, self.aux, C.byref(self._f))
            if rc:
                raise RuntimeError(f"oracle step failed: {rc}")
            dts.append((self.p.dt, self.p.last_cfl))
            self.limits_log.append((self.p.inv_va2max, self.p.v_lim, self.p.e_lim))
            if self.p.divB_switch > 0:
                self.divb_log.append((self.p.divB_last_iters, self.p.divB_err0, self.p.divB_err1))
        return dts
