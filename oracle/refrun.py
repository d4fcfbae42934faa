"""Run the reference MURaM hot path (compiled from the reference sources by
``make -C oracle ref``) on a state and collect its outputs.

Test infrastructure: used by tests and golden-fixture generation only.
The binary exists only where the reference sources were available to build it.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(HERE, "_ref", "muram_ref_harness")
DROPIN_BIN = os.path.join(HERE, "_ref", "muram_gpu_dropin")
# the reference sources: $MURAM_REF, else a checkout named "reference" beside
# this repository
REF_ROOT = os.environ.get("MURAM_REF") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))


def available():
    return os.path.exists(REF_BIN)


def build(ref_root=REF_ROOT):
    """Compile the reference harness if the reference sources exist."""
    if not os.path.isdir(ref_root):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}", "-j8"], check=True)
    return available()


def build_dropin(ref_root=REF_ROOT):
    """Link the reference harness against the MURaM-side shim and libgpumhd.so
    instead of the reference's hot-path objects (a link-level drop-in check)."""
    if not os.path.isdir(ref_root):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "dropin", f"REF={ref_root}", "-j8"], check=True)
    return os.path.exists(DROPIN_BIN)


def run(U, params, steps=1, trace_step=0, keep=None):
    """Run ``steps`` MURaM steps on the conserved state U (8, sz, sy, sx).

    ``params`` is a dict of harness keys (nx, ny, nz, dx, dy, dz, eos, CFL, ...).
    Returns a dict of numpy arrays: final_U, dts (per step: dt, cfl, dt_mhd),
    limits (per step: inv_va2max, v_lim, e_lim), with divB cleaning on
    final_phi and final_divB, the harness's stdout and, for the traced step,
    the PCAST-style snapshots keyed by name.
    """
    sz, sy, sx = U.shape[1:]
    p = dict(params)
    p["steps"] = steps
    p["trace_step"] = trace_step
    out = {}
    with tempfile.TemporaryDirectory(dir=keep) as td:
        pf = os.path.join(td, "params.txt")
        with open(pf, "w") as fh:
            for k, v in p.items():
                if isinstance(v, (list, tuple)):
                    v = " ".join(repr(float(x)) for x in v)
                fh.write(f"{k}={v}\n")
        sf = os.path.join(td, "state.bin")
        np.ascontiguousarray(np.moveaxis(U, 0, -1)).astype("<f8").tofile(sf)
        od = os.path.join(td, "out")
        os.makedirs(od)
        res = subprocess.run([REF_BIN, pf, sf, od], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"reference harness failed ({res.returncode}): {res.stderr[-2000:]}")
        out["stdout"] = res.stdout
        for fn in os.listdir(od):
            path = os.path.join(od, fn)
            if fn.endswith(".txt"):
                out[fn[:-4]] = open(path).read()
                continue
            name = fn[:-4]
            a = np.fromfile(path, dtype="<f8")
            if name.endswith("_U") or name.endswith("_R"):
                a = np.ascontiguousarray(np.moveaxis(a.reshape(sz, sy, sx, 8), -1, 0))
            elif name.endswith("_aux"):
                a = a.reshape(5, sz, sy, sx)
            elif name in ("final_phi", "final_divB", "divb_phi_in", "final_sflx"):
                a = a.reshape(sz, sy, sx)
            elif name == "diag":  # tvar1..8, Qres, Qvis of the diagnostics step
                a = a.reshape(10, sz, sy, sx)
            out[name] = a
    return out
