"""Generate the golden fixtures of the MHD step from the reference itself.

Runs the reference MURaM hot-path sources (compiled unchanged by
``make -C oracle ref``) through ``oracle/refrun.py`` on small seeded boxes and
stores, per case, the initial state and the PCAST-style snapshots around each
routine of one traced step, the state after several steps, and the per-step
dt.  The EOS table is the committed ``eos_small.dat``.

The spitzer case adds the hyperbolic heat conduction (heat flux from zero,
hot top) and keeps the final heat flux.
The open_bottom case uses the reference's own physical x boundaries (open
bottom, top open to outflows) and keeps the p_bc and s_bc they set.
The va_adjust case runs the adaptive limits of Adjust_Valf_Max and keeps its
per-step log line (maxima, va_max, the limits and the near-limit counts).
The diagnostics cases switch on the reference's diagnostics for one step
(tvar1..8, Qres, Qvis after that step's TCheck) and keep them with the state.
The divb_cleaning case also runs the reference's Clean_divB after each TVD
pass and keeps the cleaning potential phi, the last divergence and the
iteration count of every step (parsed from the reference's own log line).

Usage (in a checkout with the reference sources available):
    python tests/golden/make_golden.py [case ...]     (default: every case)
"""
from __future__ import annotations

import hashlib
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from muram_main_gb300 import initial  # noqa: E402
from oracle import refrun  # noqa: E402

EOS = os.path.join(HERE, "eos_small.dat")


def cases():
    eos = initial.EosTable(EOS)
    yield "periodic", dict(nx=12, ny=8, nz=6, dx=3.2e6, periodic_x=1), \
        initial.periodic_box(eos, 12, 8, 6, seed=11), dict(steps=3, trace_step=1)
    yield "closed_gravity", dict(nx=16, ny=8, nz=6, dx=1.6e6, periodic_x=0, grav=2.74e4), \
        initial.stratified_box(eos, 16, 8, 6, dx=1.6e6, seed=12), dict(steps=3, trace_step=2)
    yield "two_half_tvd", dict(nx=8, ny=8, nz=6, dx=3.2e6, periodic_x=1, CFL=1.2, CFL_tvd=1.0), \
        initial.periodic_box(eos, 8, 8, 6, seed=13, v_rms=3.0e5, b_rms_gauss=400.0), dict(steps=3, trace_step=1)
    yield "divb_cleaning", dict(nx=10, ny=8, nz=6, dx=1.6e6, dy=1.2e6, dz=1.4e6, periodic_x=0, grav=2.74e4,
                                divB_switch=1, divB_itmax=4, divB_err=0.15, verbose=1), \
        initial.stratified_box(eos, 10, 8, 6, dx=1.6e6, seed=14), dict(steps=5, trace_step=2)
    yield "spitzer", dict(nx=12, ny=8, nz=6, dx=1.6e6, periodic_x=0, grav=2.74e4, xbnd=1, bnd_top=1,
                          bnd_eps_top=3e12, spitzer=1.0), \
        initial.stratified_box(eos, 12, 8, 6, dx=1.6e6, seed=16), dict(steps=6, trace_step=3)
    yield "open_bottom", dict(nx=12, ny=8, nz=6, dx=1.6e6, periodic_x=0, grav=2.74e4, xbnd=1, bnd_top=1), \
        initial.stratified_box(eos, 12, 8, 6, dx=1.6e6, seed=15), dict(steps=4, trace_step=2)
    # the adaptive Alfven-speed, velocity and energy limits of the reference's
    # 3-D test run (va_adjust 1, max_fill 100: TEST/Test_3D/parameters.dat:52-53)
    # with va_max low enough that v_lim adapts instead of sitting at va_max/3
    yield "va_adjust", dict(nx=16, ny=12, nz=8, dx=3.2e6, periodic_x=1, va_max=3.0e5, va_adjust=1.0,
                            max_fill=100.0, verbose=1), \
        initial.periodic_box(eos, 16, 12, 8, seed=17, v_rms=2.0e5, b_rms_gauss=800.0), dict(steps=8, trace_step=3)
    # the diagnostics of one output step (Run.need_diagnostics at stage 4 through
    # TVDlimit and TCheck, src/solver.C:264-289): closed x with gravity, Boris
    # corrections (va_max 3e5) and an energy ceiling that TCheck applies
    yield "diagnostics", dict(nx=12, ny=8, nz=6, dx=1.6e6, periodic_x=0, grav=2.74e4, va_max=3.0e5,
                              tchk_eps_max=1.686e12, diag_step=3), \
        initial.stratified_box(eos, 12, 8, 6, dx=1.6e6, seed=21, v_rms=1.0e5), dict(steps=4, trace_step=0)
    yield "diagnostics_spitzer", dict(nx=12, ny=8, nz=6, dx=1.6e6, periodic_x=0, grav=2.74e4, xbnd=1, bnd_top=1,
                                      bnd_eps_top=3e12, spitzer=1.0, diag_step=4), \
        initial.stratified_box(eos, 12, 8, 6, dx=1.6e6, seed=16), dict(steps=5, trace_step=0)
    yield "diagnostics_two_half", dict(nx=8, ny=8, nz=6, dx=3.2e6, periodic_x=1, CFL=1.2, CFL_tvd=1.0,
                                       diag_step=2), \
        initial.periodic_box(eos, 8, 8, 6, seed=23, v_rms=3.0e5, b_rms_gauss=400.0), dict(steps=3, trace_step=0)


KEEP = ["init_U", "s1_c2p_U", "s1_c2p_aux", "s1_res_R", "s1_res_dt", "s1_si_U", "s1_bc_U", "s2_c2p_U",
        "s4_bc_U", "s4_c2p_aux", "tvd_U", "divb_U", "tck_U", "end_U", "final_U", "dts", "limits",
        "final_phi", "final_divB"]
KEEP_BND = ["init_U", "s1_si_U", "s1_bc_U", "s4_bc_U", "s4_c2p_aux", "tvd_U", "tck_U", "end_U", "final_U", "dts",
            "limits"]
KEEP_DIVB = ["init_U", "tvd_U", "divb_phi_in", "divb_U", "tck_U", "final_U", "dts", "limits", "final_phi",
             "final_divB"]


def main(only=()):
    if not refrun.available():
        refrun.build()
    mpath = os.path.join(HERE, "MANIFEST.txt")
    manifest = {}
    if os.path.exists(mpath):
        for line in open(mpath).read().splitlines()[2:]:
            manifest[line.split(".npz")[0]] = line
    for name, hp, U, run in cases():
        if only and name not in only:
            continue
        hp = dict(hp)
        hp["eos"] = EOS
        out = refrun.run(U, hp, **run)
        keep = KEEP_DIVB if hp.get("divB_switch", 0) else (KEEP_BND if hp.get("xbnd", 0) else KEEP)
        if hp.get("spitzer", 0):
            keep = ["init_U", "final_U", "final_sflx", "dts", "limits"]
        if hp.get("diag_step", 0):
            keep = keep + ["diag", "diag_U"]
        arrays = {k: out[k] for k in keep if k in out}
        arrays["input_U"] = U
        arrays["trace_step"] = np.array(run["trace_step"])
        arrays["steps"] = np.array(run["steps"])
        if hp.get("xbnd", 0):
            summ = dict(x.split("=") for x in out["summary"].split())
            arrays["p_bc"] = np.array(float(summ["p_bc"]))
            arrays["s_bc"] = np.array(float(summ["s_bc"]))
        if hp.get("va_adjust", 0):
            # per step: max|v|, max c_s, va_max, v_lim, cells near v_lim, e_lim,
            # cells near e_lim (the reference's own log line)
            num = r"([-+0-9.eE]+)"
            pat = (r"Adjust_va_max \[\d+\]\s+" + num + r"\s+" + num + r"\s+" + num + r"\s+\|\s+" + num +
                   r" \(" + num + r"\)\s+" + num + r" \(" + num + r"\)")
            arrays["va_log"] = np.array([[float(x) for x in m] for m in re.findall(pat, out["stdout"])])
        if hp.get("divB_switch", 0):
            arrays["divb_iters"] = np.array([int(m) for m in re.findall(r"divB_max \[(\d+)\]", out["stdout"])])
        meta = {k: v for k, v in hp.items() if k != "eos"}
        for k, v in meta.items():
            arrays["param_" + k] = np.array(v)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **arrays)
        h = hashlib.sha256(open(path, "rb").read()).hexdigest()[:16]
        manifest[name] = f"{name}.npz {h} {out['summary'].strip().replace(chr(10), ' ')}"
        print(manifest[name])
    with open(mpath, "w") as fh:
        fh.write("# golden fixtures from the reference harness (make_golden.py)\n")
        fh.write(f"eos_small.dat {hashlib.sha256(open(EOS, 'rb').read()).hexdigest()}\n")
        fh.write("\n".join(manifest.values()) + "\n")


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
