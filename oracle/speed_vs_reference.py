"""Single-core speed of the oracle (the C restatement of the reference path)
against the reference's own sources compiled unchanged (oracle/_ref), on the
CPU sample the benchmark's reference arm uses: a 128 (vertical) x 32 x 32
column of the stratified workload (16 km, gravity 2.74e4, closed x) on the
3000 x 3000 EOS table, FP64.

Test infrastructure: runs only where the reference harness was built (it
needs the reference sources).  The reference's time per step is taken as the
difference between an (1 + n)-step and a 1-step run of its harness, so that
process start-up and the EOS table read cancel.

    python oracle/speed_vs_reference.py [steps]
"""
from __future__ import annotations

import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this folder would shadow the oracle package with oracle.py
sys.path[:] = [ROOT] + [p for p in sys.path if os.path.abspath(p or ".") != HERE]


def main(steps=8):
    import bench
    from muram_main_gb300 import eos_table
    from oracle import oracle as O
    from oracle import refrun
    if not refrun.available() and not refrun.build():
        print("reference harness not available (no reference sources)")
        return 1
    eos_table.ensure_table(bench.EOS_BENCH, "bench")
    s = bench.SAMPLE
    U = bench.make_state(s["nx"], s["ny"], s["nz"], seed=1000)
    hp = dict(nx=s["nx"], ny=s["ny"], nz=s["nz"], dx=bench.WORKLOAD["dx"], periodic_x=0,
              grav=bench.WORKLOAD["grav"], eos=bench.EOS_BENCH)
    t = {}
    for n in (1, 1 + steps):
        t0 = time.perf_counter()
        refrun.run(U, hp, steps=n)
        t[n] = time.perf_counter() - t0
    ref_step = (t[1 + steps] - t[1]) / steps
    st = O.State(O.params_from_harness(hp), U)
    eos = O.Eos(bench.EOS_BENCH)
    st.step(eos, 1)
    t0 = time.perf_counter()
    st.step(eos, steps)
    port_step = (time.perf_counter() - t0) / steps
    cells = s["nx"] * s["ny"] * s["nz"]
    print(f"sample {s['nx']}x{s['ny']}x{s['nz']}, {steps} steps, one core each")
    print(f"reference (oracle/_ref): {ref_step * 1e3:.1f} ms/step = {cells / ref_step:.3e} cell-updates/s")
    print(f"oracle port:             {port_step * 1e3:.1f} ms/step = {cells / port_step:.3e} cell-updates/s")
    print(f"port / reference speed:  {ref_step / port_step:.3f}")
    return 0


if __name__ == "__main__":
    sys.exit(main(int(sys.argv[1]) if len(sys.argv) > 1 else 8))
