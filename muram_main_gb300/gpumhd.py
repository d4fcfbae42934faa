"""Python host layer over the gpumhd C ABI (include/gpumhd.h).

``MuramGPU`` mirrors the MURaM routines on the time-step path: each method has
the reference routine's name and meaning, operating on the device-resident
GridData of one context.  Host arrays use the reference's cState layout
(float64 records of 8 values, x fastest, two ghost layers), or the package's
structure-of-arrays view (8, sz, sy, sx) which ``upload_state`` /
``download_state`` convert.

The CUDA library must be built (``muram_main_gb300.build.build()``); loading
fails loudly when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

OK = 0
E_INVALID = -1
E_CUDA = -2
E_EOS = -3
E_BAD_DT = -4
E_CFL = -5
E_ORDER = -6
E_NOMEM = -7

(FIELD_U, FIELD_U0, FIELD_RES, FIELD_PRES, FIELD_TEMP, FIELD_NE, FIELD_RHOI, FIELD_AMB, FIELD_PHI, FIELD_DIVB,
 FIELD_SFLX) = range(11)
# an output step's diagnostics: tvar1..tvar8, Qres, Qvis
FIELD_DIAG = 11
DIAG_NAMES = ("tvar1", "tvar2", "tvar3", "tvar4", "tvar5", "tvar6", "tvar7", "tvar8", "Qres", "Qvis")


class GpumhdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gpumhd error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    """ctypes mirror of ``gpumhd_params``."""
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("periodic_x", C.c_int),
        ("precision", C.c_int), ("stage_kernel", C.c_int),
        ("dx", C.c_double * 3),
        ("CFL", C.c_double), ("CFL_tvd", C.c_double), ("dt", C.c_double), ("time", C.c_double),
        ("outcad", C.c_double), ("autostep", C.c_int), ("compensated", C.c_int),
        ("grav", C.c_double), ("va_max", C.c_double), ("va_adjust", C.c_double), ("max_fill", C.c_double),
        ("tvd_h", C.c_double * 4), ("tvd_cs", C.c_double * 4), ("tvd", C.c_double * 10),
        ("tvd_h_bnd", C.c_double * 2), ("tvd_visc_bnd", C.c_double * 2), ("tvd_eta_bnd", C.c_double * 2),
        ("tvd_coeff", C.c_double * 4), ("tchk", C.c_double * 4),
        ("rt_cfl", C.c_double), ("rt_tstep", C.c_double), ("rt_update", C.c_double),
        ("tau0", C.c_double), ("dt_rad", C.c_double), ("eta", C.c_double),
        ("divB_switch", C.c_int), ("divB_itmax", C.c_int), ("divB_err", C.c_double),
        ("xbnd", C.c_int), ("bnd_top", C.c_int),
        ("bnd_bcrit", C.c_double), ("bnd_eps_top", C.c_double), ("p_bc", C.c_double), ("s_bc", C.c_double),
        ("spitzer", C.c_double),
    ]


EXPORTS = [
    "gpumhd_default_params", "gpumhd_create", "gpumhd_destroy", "gpumhd_set_params", "gpumhd_get_params",
    "gpumhd_last_error", "gpumhd_eos_init", "gpumhd_upload", "gpumhd_download", "gpumhd_upload_async",
    "gpumhd_download_async", "gpumhd_save_cons",
    "gpumhd_cons_to_prim", "gpumhd_adjust_valf_max", "gpumhd_get_limits", "gpumhd_mhd_residual",
    "gpumhd_sync_timestep", "gpumhd_source_integrate_tcheck", "gpumhd_tvdlimit", "gpumhd_tcheck",
    "gpumhd_exchange", "gpumhd_run_steps", "gpumhd_enqueue_steps", "gpumhd_synchronize", "gpumhd_step_info",
    "gpumhd_stream", "gpumhd_launch_count", "gpumhd_profile_steps", "gpumhd_cfl_dt_noalloc",
    "gpumhd_adjoint", "gpumhd_tile_from", "gpumhd_set_tuning", "gpumhd_get_tuning", "gpumhd_autotune", "gpumhd_ensemble_create",
    "gpumhd_ensemble_destroy", "gpumhd_ensemble_enqueue_steps", "gpumhd_ensemble_synchronize",
    "gpumhd_ensemble_last_error", "gpumhd_ensemble_stream", "gpumhd_ensemble_launch_count",
    "gpumhd_clean_divB", "gpumhd_divb_info", "gpumhd_boundary_info", "gpumhd_test_tma_wait",
    "gpumhd_set_divb_iters", "gpumhd_set_need_diagnostics", "gpumhd_upload_f32", "gpumhd_download_f32",
    "gpumhd_upload_async_f32", "gpumhd_download_async_f32", "gpumhd_ensemble_set_schedule",
    "gpumhd_ensemble_autotune",
]

_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libgpumhd.so (building it first if needed) and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise OSError(f"gpumhd library not built: {_build.LIB}")
        _build.build()
    L = C.CDLL(_build.LIB)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    fp = C.POINTER(C.c_float)
    P = C.POINTER(Params)
    sig = {
        "gpumhd_default_params": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_double]),
        "gpumhd_create": (C.c_int, [P, C.c_int, C.POINTER(vp)]),
        "gpumhd_destroy": (C.c_int, [vp]),
        "gpumhd_set_params": (C.c_int, [vp, P]),
        "gpumhd_get_params": (C.c_int, [vp, P]),
        "gpumhd_last_error": (C.c_char_p, [vp]),
        "gpumhd_eos_init": (C.c_int, [vp, C.c_char_p]),
        "gpumhd_upload": (C.c_int, [vp, C.c_int, dp]),
        "gpumhd_upload_async": (C.c_int, [vp, C.c_int, dp]),
        "gpumhd_download_async": (C.c_int, [vp, C.c_int, dp]),
        "gpumhd_download": (C.c_int, [vp, C.c_int, dp]),
        "gpumhd_upload_f32": (C.c_int, [vp, C.c_int, fp]),
        "gpumhd_upload_async_f32": (C.c_int, [vp, C.c_int, fp]),
        "gpumhd_download_async_f32": (C.c_int, [vp, C.c_int, fp]),
        "gpumhd_download_f32": (C.c_int, [vp, C.c_int, fp]),
        "gpumhd_save_cons": (C.c_int, [vp]),
        "gpumhd_cons_to_prim": (C.c_int, [vp]),
        "gpumhd_adjust_valf_max": (C.c_int, [vp]),
        "gpumhd_get_limits": (C.c_int, [vp, dp, dp, dp]),
        "gpumhd_mhd_residual": (C.c_int, [vp, dp]),
        "gpumhd_sync_timestep": (C.c_int, [vp, C.c_double, C.c_double, dp]),
        "gpumhd_source_integrate_tcheck": (C.c_int, [vp, C.c_int]),
        "gpumhd_tvdlimit": (C.c_int, [vp, C.c_double]),
        "gpumhd_tcheck": (C.c_int, [vp]),
        "gpumhd_exchange": (C.c_int, [vp, C.c_int]),
        "gpumhd_run_steps": (C.c_int, [vp, C.c_int, dp, C.c_int]),
        "gpumhd_enqueue_steps": (C.c_int, [vp, C.c_int]),
        "gpumhd_synchronize": (C.c_int, [vp]),
        "gpumhd_step_info": (C.c_int, [vp, dp, dp, dp, C.POINTER(C.c_int)]),
        "gpumhd_profile_steps": (C.c_int, [vp, C.c_int, dp]),
        "gpumhd_cfl_dt_noalloc": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, dp, C.c_double, vp, vp]),
        "gpumhd_stream": (vp, [vp]),
        "gpumhd_launch_count": (C.c_longlong, [vp]),
        "gpumhd_tile_from": (C.c_int, [vp, vp]),
        "gpumhd_adjoint": (C.c_int, [vp, C.c_int, C.c_int, dp, dp]),
        "gpumhd_set_tuning": (C.c_int, [vp, C.c_int, C.c_int]),
        "gpumhd_get_tuning": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "gpumhd_autotune": (C.c_int, [vp, C.c_int, dp]),
        "gpumhd_ensemble_create": (C.c_int, [C.POINTER(vp), C.c_int, C.POINTER(vp)]),
        "gpumhd_ensemble_destroy": (C.c_int, [vp]),
        "gpumhd_ensemble_enqueue_steps": (C.c_int, [vp, C.c_int]),
        "gpumhd_ensemble_synchronize": (C.c_int, [vp]),
        "gpumhd_ensemble_last_error": (C.c_char_p, [vp]),
        "gpumhd_ensemble_stream": (vp, [vp]),
        "gpumhd_ensemble_launch_count": (C.c_longlong, [vp]),
        "gpumhd_ensemble_set_schedule": (C.c_int, [vp, C.c_int, C.c_int]),
        "gpumhd_ensemble_autotune": (C.c_int, [vp, C.c_int, dp]),
        "gpumhd_clean_divB": (C.c_int, [vp]),
        "gpumhd_divb_info": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), dp, dp]),
        "gpumhd_boundary_info": (C.c_int, [vp, dp, dp]),
        "gpumhd_test_tma_wait": (C.c_int, [vp, C.c_longlong, C.c_int]),
        "gpumhd_set_divb_iters": (C.c_int, [vp, C.c_int]),
        "gpumhd_set_need_diagnostics": (C.c_int, [vp, C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def default_params(nx, ny, nz, dx=3.2e6, precision=64, **kw):
    p = Params()
    load().gpumhd_default_params(C.byref(p), nx, ny, nz, dx)
    p.precision = precision
    for k, v in kw.items():
        if k in ("dy", "dz"):
            p.dx[1 if k == "dy" else 2] = v
        elif isinstance(v, (list, tuple, np.ndarray)):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = float(x)
        else:
            setattr(p, k, v)
    return p


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class MuramGPU:
    """One device-resident MURaM grid (a gpumhd context)."""

    def __init__(self, params, device=0, eos_path=None):
        L = load()
        self._L = L
        self.params = params
        h = C.c_void_p()
        rc = L.gpumhd_create(C.byref(params), device, C.byref(h))
        if rc != OK:
            raise GpumhdError(rc, L.gpumhd_last_error(None).decode())
        self._h = h
        self.shape = (params.nz + 4, params.ny + 4, params.nx + 4)
        if eos_path is not None:
            self.eos_init(eos_path)

    def _chk(self, rc):
        if rc != OK:
            raise GpumhdError(rc, self._L.gpumhd_last_error(self._h).decode())
        return rc

    def close(self):
        if getattr(self, "_h", None):
            self._L.gpumhd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- data movement (ACCH::UpdateGPU / UpdateCPU)
    def upload(self, which, aos):
        """aos in cState layout: float64, or float32 as a SINGLE_PRECISION
        MURaM build holds it (any other dtype is converted to float64)."""
        if np.asarray(aos).dtype == np.float32:
            a = np.ascontiguousarray(aos)
            self._chk(self._L.gpumhd_upload_f32(self._h, which, a.ctypes.data_as(C.POINTER(C.c_float))))
            return
        a = np.ascontiguousarray(aos, dtype=np.float64)
        self._chk(self._L.gpumhd_upload(self._h, which, _dptr(a)))

    def download(self, which, dtype=np.float64):
        nf = 8 if which <= FIELD_RES else 1
        out = np.empty(int(np.prod(self.shape)) * nf, dtype=dtype)
        if out.dtype == np.float32:
            self._chk(self._L.gpumhd_download_f32(self._h, which, out.ctypes.data_as(C.POINTER(C.c_float))))
        elif out.dtype == np.float64:
            self._chk(self._L.gpumhd_download(self._h, which, _dptr(out)))
        else:
            raise ValueError(f"download: host layout float64 or float32, not {out.dtype}")
        return out

    def upload_state(self, U, which=FIELD_U):
        """U: (8, sz, sy, sx) float64 structure of arrays."""
        self.upload(which, np.moveaxis(np.asarray(U, dtype=np.float64), 0, -1))

    def download_state(self, which=FIELD_U):
        a = self.download(which)
        return np.ascontiguousarray(np.moveaxis(a.reshape(self.shape + (8,)), -1, 0))

    def download_field(self, which):
        return self.download(which).reshape(self.shape)

    def upload_field(self, which, f):
        self.upload(which, np.asarray(f, dtype=np.float64).reshape(-1))

    # -- the reference routines
    def eos_init(self, path):
        self._chk(self._L.gpumhd_eos_init(self._h, os.fsencode(path)))

    def set_need_diagnostics(self, on):
        """RunData::need_diagnostics: on zeroes the ten diagnostic arrays, which
        the per-routine calls that follow fill (an output step)."""
        self._chk(self._L.gpumhd_set_need_diagnostics(self._h, 1 if on else 0))

    def download_diagnostics(self):
        """tvar1..tvar8, Qres, Qvis as one (10, sz, sy, sx) array."""
        return np.stack([self.download_field(FIELD_DIAG + q) for q in range(10)])

    def SaveCons(self):
        self._chk(self._L.gpumhd_save_cons(self._h))

    def ConsToPrim(self):
        self._chk(self._L.gpumhd_cons_to_prim(self._h))

    def Adjust_Valf_Max(self):
        self._chk(self._L.gpumhd_adjust_valf_max(self._h))

    def limits(self):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        self._chk(self._L.gpumhd_get_limits(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def MHD_Residual(self):
        dt = C.c_double()
        self._chk(self._L.gpumhd_mhd_residual(self._h, C.byref(dt)))
        return dt.value

    def Sync_timestep(self, dt_rad, dt_mhd):
        cfl = C.c_double()
        self._chk(self._L.gpumhd_sync_timestep(self._h, dt_rad, dt_mhd, C.byref(cfl)))
        return cfl.value

    def Source_Integrate_Tcheck(self, stage):
        self._chk(self._L.gpumhd_source_integrate_tcheck(self._h, stage))

    def TVDlimit(self, dt_tvd):
        self._chk(self._L.gpumhd_tvdlimit(self._h, dt_tvd))

    def TCheck(self):
        self._chk(self._L.gpumhd_tcheck(self._h))

    def exchange_grid(self, with_bc=True):
        self._chk(self._L.gpumhd_exchange(self._h, 1 if with_bc else 0))

    def boundary_info(self):
        """(p_bc, s_bc) of the open bottom (negative until the first boundary call sets them)."""
        a, b = C.c_double(), C.c_double()
        self._chk(self._L.gpumhd_boundary_info(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def Clean_divB(self):
        self._chk(self._L.gpumhd_clean_divB(self._h))

    def set_divb_iters(self, next_iters):
        """Set Clean_divB's adaptive iteration count for the next call."""
        self._chk(self._L.gpumhd_set_divb_iters(self._h, int(next_iters)))

    def divb_info(self):
        """(iterations of the last cleaning, iterations of the next, max|divB|
        before and after the last cleaning in G)."""
        a, b = C.c_int(), C.c_int()
        e0, e1 = C.c_double(), C.c_double()
        self._chk(self._L.gpumhd_divb_info(self._h, C.byref(a), C.byref(b), C.byref(e0), C.byref(e1)))
        return a.value, b.value, e0.value, e1.value

    def step_reference_order(self, dt_rad=None, diagnostics=False):
        """One step through the per-routine entry points in ComputeSolution's
        order (src/solver.C:109-365); returns (dt, cfl).  diagnostics: an
        output step, whose diagnostics (need_diagnostics from stage 4 through
        TCheck) are left in the diagnostic arrays."""
        p = self.params
        dt_rad = p.dt_rad if dt_rad is None else dt_rad
        cfl = 0.0
        self.SaveCons()
        for stage in range(1, 5):
            self.ConsToPrim()
            if stage == 1:
                self.Adjust_Valf_Max()
            if stage == 4 and diagnostics:
                self.set_need_diagnostics(True)
            dt_mhd = self.MHD_Residual()
            if stage == 1:
                cfl = self.Sync_timestep(dt_rad, dt_mhd)
            self.Source_Integrate_Tcheck(stage)
            self.exchange_grid(True)
        dt = self.step_info()[0]
        if cfl <= p.CFL_tvd:
            self.TVDlimit(dt)
        else:
            self.TVDlimit(0.5 * dt)
            self.exchange_grid(False)
            self.TVDlimit(0.5 * dt)
        if p.divB_switch > 0:
            self.Clean_divB()
        self.TCheck()
        if diagnostics:
            self.set_need_diagnostics(False)
        self.exchange_grid(True)
        return dt, cfl

    # -- result / restart files (src/io_xysl.C OutputSolution, RestoreSolution)
    def OutputSolution(self, path, it, resfile="result", backup=True):
        """Download U and write result_prim_0..7, Header and backup.dat."""
        from . import muram_io
        dt, _, t, _ = self.step_info()
        inv_va2max = self.limits()[0]
        p = self.params
        muram_io.write_result(self.download_state(), path, it, tuple(p.dx), time=t, dt=dt,
                              inv_va2max=inv_va2max, resfile=resfile, backup=backup)

    def RestoreSolution(self, path, it, resfile="result"):
        """Read one output, convert it to conserved variables, upload it as U
        and U0, fill the ghosts and set the run time (backup.dat's when the
        directory has one, as RestoreSolution reads it, else the Header's);
        returns that time."""
        from . import muram_io
        p = self.params
        U = muram_io.read_result(path, it, resfile, shape_xyz=(p.nx, p.ny, p.nz))
        if os.path.exists(os.path.join(path, "backup.dat")):
            t = muram_io.read_backup(path)["time"]
        else:
            t = muram_io.read_header(path, it)["time"]
        p.time = t
        self._chk(self._L.gpumhd_set_params(self._h, C.byref(p)))
        self.upload_state(U)
        self.upload_state(U, FIELD_U0)
        self.exchange_grid(True)
        return t

    # -- fused path
    def run_steps(self, nsteps, capture=True):
        dts = np.zeros(max(nsteps, 1))
        self._chk(self._L.gpumhd_run_steps(self._h, nsteps, _dptr(dts), 1 if capture else 0))
        return dts[:nsteps]

    def enqueue_steps(self, nsteps):
        self._chk(self._L.gpumhd_enqueue_steps(self._h, nsteps))

    def synchronize(self):
        self._chk(self._L.gpumhd_synchronize(self._h))

    def step_info(self):
        dt, cfl, t = C.c_double(), C.c_double(), C.c_double()
        two = C.c_int()
        self._chk(self._L.gpumhd_step_info(self._h, C.byref(dt), C.byref(cfl), C.byref(t), C.byref(two)))
        return dt.value, cfl.value, t.value, two.value

    PHASES = ["step_control", "stage1", "stage2", "stage3", "stage4", "tvd_x", "tvd_y", "tvd_z",
              "tvd2_x", "tvd2_y", "tvd2_z", "divb_clean", "finish"]

    def profile_steps(self, nsteps=2):
        """Mean duration (ms) of each launch of a fused step, timed with CUDA events
        (divb_clean: all cleaning passes; finish: the end-of-step pass)."""
        ms = np.zeros(13)
        self._chk(self._L.gpumhd_profile_steps(self._h, nsteps, _dptr(ms)))
        return dict(zip(self.PHASES, ms.tolist()))

    def _xfer(self, name, which, ptr, host_dtype):
        if np.dtype(host_dtype) == np.float32:
            fn, t = getattr(self._L, name + "_f32"), C.c_float
        elif np.dtype(host_dtype) == np.float64:
            fn, t = getattr(self._L, name), C.c_double
        else:
            raise ValueError(f"host layout float64 or float32, not {np.dtype(host_dtype)}")
        self._chk(fn(self._h, which, C.cast(ptr, C.POINTER(t))))

    def upload_ptr(self, which, ptr, host_dtype=np.float64):
        """Upload from a raw host pointer (e.g. pinned memory) in cState layout
        of host_dtype (float64, or float32 as in a SINGLE_PRECISION build)."""
        self._xfer("gpumhd_upload", which, ptr, host_dtype)

    def download_ptr(self, which, ptr, host_dtype=np.float64):
        self._xfer("gpumhd_download", which, ptr, host_dtype)

    def upload_ptr_async(self, which, ptr, host_dtype=np.float64):
        """Upload from a host pointer without waiting: the copy overlaps the
        steps enqueued before it; the buffer must stay valid and unchanged
        until synchronize()."""
        self._xfer("gpumhd_upload_async", which, ptr, host_dtype)

    def download_ptr_async(self, which, ptr, host_dtype=np.float64):
        """Download to a host pointer without waiting; the data are there after synchronize()."""
        self._xfer("gpumhd_download_async", which, ptr, host_dtype)

    def adjoint(self, nsteps, dJ_dUT, checkpoint_every=5):
        """dJ/dU_0 for J(U_T) over nsteps fixed-dt FP64 steps from the current
        state; dJ_dUT and the result are (8, sz, sy, sx) arrays (ghosts ignored / zero)."""
        lam = np.ascontiguousarray(np.moveaxis(np.asarray(dJ_dUT, dtype=np.float64), 0, -1))
        out = np.empty_like(lam)
        self._chk(self._L.gpumhd_adjoint(self._h, nsteps, checkpoint_every, _dptr(lam), _dptr(out)))
        return np.ascontiguousarray(np.moveaxis(out, -1, 0))

    def tile_from(self, src):
        """This box's state becomes the periodic tiling of src's (set-up of large boxes)."""
        self._chk(self._L.gpumhd_tile_from(self._h, src._h))

    # -- launch shapes
    def test_tma_wait(self, wait_cycles=0, withhold_last=False):
        """Test hook of the TMA stage kernel's bounded waits (see gpumhd.h)."""
        self._chk(self._L.gpumhd_test_tma_wait(self._h, int(wait_cycles), 1 if withhold_last else 0))

    def set_tuning(self, stage_zchunk=0, tvd_chunk=0):
        self._chk(self._L.gpumhd_set_tuning(self._h, stage_zchunk, tvd_chunk))

    def tuning(self):
        k, z, t = C.c_int(), C.c_int(), C.c_int()
        self._chk(self._L.gpumhd_get_tuning(self._h, C.byref(k), C.byref(z), C.byref(t)))
        return dict(stage_kernel=k.value, stage_zchunk=z.value, tvd_chunk=t.value)

    def autotune(self, trial_steps=3):
        """Pick the fastest launch shapes for this box (state left unchanged);
        returns the best time per step in ms."""
        ms = C.c_double()
        self._chk(self._L.gpumhd_autotune(self._h, trial_steps, C.byref(ms)))
        return ms.value

    @property
    def stream(self):
        return self._L.gpumhd_stream(self._h)

    @property
    def launch_count(self):
        return self._L.gpumhd_launch_count(self._h)


class MuramEnsemble:
    """Several MuramGPU boxes advanced together by one graph launch per call."""

    def __init__(self, boxes):
        L = load()
        self._L = L
        self.boxes = list(boxes)
        arr = (C.c_void_p * len(self.boxes))(*[b._h.value for b in self.boxes])
        h = C.c_void_p()
        rc = L.gpumhd_ensemble_create(arr, len(self.boxes), C.byref(h))
        if rc != OK:
            raise GpumhdError(rc, L.gpumhd_ensemble_last_error(None).decode())
        self._h = h

    def _chk(self, rc):
        if rc != OK:
            raise GpumhdError(rc, self._L.gpumhd_ensemble_last_error(self._h).decode())

    def enqueue_steps(self, nsteps):
        self._chk(self._L.gpumhd_ensemble_enqueue_steps(self._h, nsteps))

    def synchronize(self):
        self._chk(self._L.gpumhd_ensemble_synchronize(self._h))

    def run_steps(self, nsteps):
        self.enqueue_steps(nsteps)
        self.synchronize()

    def set_schedule(self, steps_per_iteration=1, largest_first=False):
        """Steps of each box per loop iteration, and the branch order."""
        self._chk(self._L.gpumhd_ensemble_set_schedule(self._h, steps_per_iteration, 1 if largest_first else 0))

    def autotune(self, trial_steps=4):
        """Launch shapes of the boxes for this ensemble, timed from their
        current states (restored afterwards); returns ms per ensemble step."""
        ms = C.c_double()
        self._chk(self._L.gpumhd_ensemble_autotune(self._h, trial_steps, C.byref(ms)))
        return ms.value

    @property
    def stream(self):
        return self._L.gpumhd_ensemble_stream(self._h)

    @property
    def launch_count(self):
        return self._L.gpumhd_ensemble_launch_count(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._L.gpumhd_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
