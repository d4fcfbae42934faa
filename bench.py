#!/usr/bin/env python
"""Benchmark of the MURaM MHD time step on GB300: cell-updates/s.

Default workload (N=1): the stratified convection-style box, 128 (vertical,
MURaM dimension 0) x 384 x 384 cells at 16 km, closed top/bottom, periodic
horizontally, gravity 2.74e4 cm/s^2, seeded random velocity and field, in FP32
storage and arithmetic; the FP64 mode of the same box is timed too and reported
under "fp64".  One step = SaveCons, 4 RK stages (residual, sources, update,
Tcheck), Sync_timestep, TVD and TCheck, ghost fill -- the whole time step.

--impl reference times the reference algorithm on the host cores (the oracle's
C restatement, or the reference harness where it was built) on bounded samples
of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MHD cell-updates/s per RK4 step"
UNIT = "cell-updates/s"
WORKLOAD = dict(nx=128, ny=384, nz=384, dx=1.6e6, grav=2.74e4, periodic_x=0)
DATA_DIR = os.path.join(ROOT, "muram_main_gb300", "_data")
EOS_BENCH = os.path.join(DATA_DIR, "eos_bench.dat")
# CPU sample: the full vertical extent with a 32 x 32 horizontal patch
SAMPLE = dict(nx=128, ny=32, nz=32)


def world():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def replica_max(ms):
    """The timed region's length as the whole job sees it: the maximum over
    the ranks (independent replicas, one per GPU; the only exchange is this
    reduction, over gloo)."""
    ws, _, _ = world()
    if ws == 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(ws, cells, steps, ms):
    """Whole-job cell-updates/s: every rank advances its own box of `cells`."""
    return ws * cells * steps / (ms / 1e3)


def make_state(nx, ny, nz, seed):
    from muram_main_gb300 import eos_table, initial
    eos_table.ensure_table(EOS_BENCH, "bench")
    tab = initial.EosTable(EOS_BENCH)
    return initial.stratified_box(tab, nx, ny, nz, dx=WORKLOAD["dx"], grav=WORKLOAD["grav"], seed=seed)


# ----------------------------------------------------------------- CPU side
def _cpu_worker(args):
    seed, steps, warmup = args
    import numpy as np  # noqa: F401
    from oracle import oracle as O
    U = make_state(SAMPLE["nx"], SAMPLE["ny"], SAMPLE["nz"], seed)
    p = O.make_params(SAMPLE["nx"], SAMPLE["ny"], SAMPLE["nz"], WORKLOAD["dx"], periodic_x=False,
                      grav=WORKLOAD["grav"])
    st = O.State(p, U)
    eos = O.Eos(EOS_BENCH)
    st.step(eos, warmup)
    t0 = time.perf_counter()
    st.step(eos, steps)
    dt = time.perf_counter() - t0
    return SAMPLE["nx"] * SAMPLE["ny"] * SAMPLE["nz"] * steps, dt


def cpu_baseline(cores, steps_per_core, warmup=1):
    """Oracle (C restatement of the reference path) on `cores` spawned processes,
    each advancing its own 128x32x32 column of the workload; aggregate rate."""
    from oracle import oracle as O
    O.build()
    from muram_main_gb300 import eos_table
    eos_table.ensure_table(EOS_BENCH, "bench")
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(1000 + i, steps_per_core, warmup) for i in range(cores)])
    cells = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    return cells / wall, wall


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self._proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self._proc.stdout:
            if self._stop.is_set():
                break
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def stop(self):
        self._stop.set()
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# -------------------------------------------------------------- GPU timing
def time_device(g, steps, warmup):
    """Device-resident throughput: CUDA events on the library's stream."""
    import torch
    stream = torch.cuda.ExternalStream(g.stream)
    g.enqueue_steps(warmup)
    g.synchronize()
    n0 = g.launch_count
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    g.enqueue_steps(steps)
    e1.record(stream)
    e1.synchronize()
    g.synchronize()
    return e0.elapsed_time(e1), g.launch_count - n0


def time_e2e(g, steps, U, host_dtype="float64", reps=5):
    """End to end through the C ABI: per step the host state (pinned, cState
    layout: float64 as MURaM's default build holds it, or float32 as its
    SINGLE_PRECISION build does) goes to the device, one fused step runs, and
    the result comes back to the host.  The transfers are the asynchronous
    ones, so one step's upload and the previous step's download overlap the
    steps around them; every byte of every step crosses the link inside the
    timed region.  Returns (median ms of reps runs of `steps` steps, h2d bytes
    per step, d2h bytes per step, result check, every run's ms)."""
    import numpy as np
    import torch
    from muram_main_gb300 import gpumhd
    aos = np.ascontiguousarray(np.moveaxis(U, 0, -1), dtype=host_dtype)
    h_in = torch.from_numpy(aos.reshape(-1)).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    h_ref = torch.empty_like(h_in).pin_memory()
    nbytes = h_in.numel() * h_in.element_size()
    # the expected result of one step from h_in, through the synchronous calls
    g.upload_ptr(gpumhd.FIELD_U, h_in.data_ptr(), host_dtype)
    g.run_steps(1)
    g.download_ptr(gpumhd.FIELD_U, h_ref.data_ptr(), host_dtype)
    g.upload_ptr_async(gpumhd.FIELD_U, h_in.data_ptr(), host_dtype)
    g.enqueue_steps(1)
    g.download_ptr_async(gpumhd.FIELD_U, h_out.data_ptr(), host_dtype)
    g.synchronize()
    torch.cuda.synchronize()
    # untimed passes first: right after the device-resident runs the pipeline
    # has been seen to run ~20 % slower for a second or two
    for _ in range(2):
        for _ in range(steps):
            g.upload_ptr_async(gpumhd.FIELD_U, h_in.data_ptr(), host_dtype)
            g.enqueue_steps(1)
            g.download_ptr_async(gpumhd.FIELD_U, h_out.data_ptr(), host_dtype)
        g.synchronize()
    runs = []
    for _ in range(reps):  # the host link's rate varies from run to run: the median of reps runs
        t0 = time.perf_counter()
        for _ in range(steps):
            g.upload_ptr_async(gpumhd.FIELD_U, h_in.data_ptr(), host_dtype)
            g.enqueue_steps(1)
            g.download_ptr_async(gpumhd.FIELD_U, h_out.data_ptr(), host_dtype)
        g.synchronize()
        runs.append((time.perf_counter() - t0) * 1e3)
    same = bool(torch.equal(h_out, h_ref))
    return sorted(runs)[len(runs) // 2], nbytes, nbytes, same, runs


def time_link(nbytes, reps=4):
    """The host link alone for one step's bytes: pinned host -> device,
    device -> pinned host, and both at once on two streams (GB/s per direction,
    best of reps, host clock around synchronised copies)."""
    import torch
    n = nbytes // 4
    h_a = torch.empty(n, dtype=torch.float32).pin_memory()
    h_b = torch.empty(n, dtype=torch.float32).pin_memory()
    d_a = torch.empty(n, dtype=torch.float32, device="cuda")
    d_b = torch.empty(n, dtype=torch.float32, device="cuda")
    s_a, s_b = torch.cuda.Stream(), torch.cuda.Stream()

    def best(fn):
        fn()
        torch.cuda.synchronize()
        t = None
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            t = dt if t is None else min(t, dt)
        return round(nbytes / t / 1e9, 1)

    def both():
        with torch.cuda.stream(s_a):
            d_a.copy_(h_a, non_blocking=True)
        with torch.cuda.stream(s_b):
            h_b.copy_(d_b, non_blocking=True)

    out = {"h2d_gbs": best(lambda: d_a.copy_(h_a, non_blocking=True)),
           "d2h_gbs": best(lambda: h_b.copy_(d_b, non_blocking=True)),
           "both_directions_gbs_each": best(both)}
    del h_a, h_b, d_a, d_b
    torch.cuda.empty_cache()
    return out


def words_per_cell(phase):
    """Algorithmic words moved per interior cell by one launch of each kernel
    (state words: 8 conserved variables + pressure)."""
    if phase == "stage1":
        return 8 + 1 + 8 + 1          # read U, p; write U', p'
    if phase in ("stage2", "stage3"):
        return 8 + 1 + 8 + 8 + 1      # read U, p, U0; write U', p'
    if phase == "stage4":
        return 8 + 1 + 8 + 8          # read U, p, U0; write U'
    if phase in ("tvd_x", "tvd_y"):
        return 8 + 1 + 8              # read U, stale p; write U
    if phase == "tvd_z":
        return 8 + 1 + 8              # the interior only; the end-of-step pass follows
    if phase == "finish":
        return 8 + 1                  # read U (TCheck stores only what it changes); write p
    return 0


# Algorithmic words per interior cell and step, the compulsory traffic of a
# fused design (ghost reads as cache hits): each of the 4 RK stages reads and
# writes the 8-word state, stages 2-4 also read U0, stage 4 stores the pressure
# the TVD sweeps use, and 3 TVD sweeps read 8 + 1 and write 8.  The roofline
# uses these counts; the kernels here also hand the pressure from stage to
# stage (words_per_cell above), which the counts leave out.
ALGO_STAGE_WORDS = 4 * 16 + 3 * 8 + 1      # 89 per 4 stage launches
ALGO_TVD_WORDS = 3 * 17                    # 51 per 3 sweeps
ALGO_STEP_WORDS = ALGO_STAGE_WORDS + ALGO_TVD_WORDS  # 140
# Floating-point operations per cell-update (4 stages, 3 TVD sweeps), counted
# from the reference's source to +-30 %: the FP64 mode's arithmetic roofline
FLOPS_PER_CELL_UPDATE = 3700.0
FLOPS_STAGE_PER_CELL = 2600.0 / 4          # per stage launch


def fp64_peak_tflops():
    """The GPU's FP64 rate as cuBLAS reaches it: a DGEMM of 8192^3 through
    torch.matmul (best of 5 after a warm-up, CUDA events)."""
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = None
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / (best / 1e3) / 1e12


def load_traffic():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh)
    return {}


def run_ours(args):
    import numpy as np  # noqa: F401
    import torch
    from muram_main_gb300 import build, eos_table, gpumhd
    ws, rank, lrank = world()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(lrank)
    build.build()
    eos_table.ensure_table(EOS_BENCH, "bench")
    wl = dict(WORKLOAD)
    if args.ny:  # a smaller horizontal extent, for profiler captures (the headline is the default)
        wl["ny"] = wl["nz"] = args.ny
    n_cells = wl["nx"] * wl["ny"] * wl["nz"]
    U = make_state(wl["nx"], wl["ny"], wl["nz"], seed=7 + rank)
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        with open(pk) as fh:
            peaks = json.load(fh)
    peak_gbs = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    # --divb: Clean_divB after every TVD pass at the reference's test settings
    # (divB_switch 1, divB_itmax 5, divB_err 0.2: TEST/Test_3D/parameters.dat)
    divb_kw = dict(divB_switch=1, divB_itmax=5, divB_err=0.2) if args.divb else {}
    # --xbnd: MURaM's physical x boundaries instead of the mirror rule, at the
    # reference's standard run settings (RUNDIR/parameters.dat: bnd_top 0,
    # bnd_pot 0, bnd_bcrit 2.5e30)
    if args.xbnd:
        divb_kw.update(xbnd=1, bnd_top=0, bnd_bcrit=2.5e30)
    # --spitzer K: hyperbolic Spitzer conduction with coefficient K (the reference's test run: 1e-6)
    if args.spitzer > 0:
        divb_kw.update(spitzer=args.spitzer)

    def context(prec, compensated=0):
        p = gpumhd.default_params(wl["nx"], wl["ny"], wl["nz"], wl["dx"], precision=prec,
                                  periodic_x=wl["periodic_x"], grav=wl["grav"], compensated=compensated,
                                  **divb_kw)
        g = gpumhd.MuramGPU(p, device=lrank, eos_path=EOS_BENCH)
        g.upload_state(U)
        return g

    # FP32 headline
    g = context(32)
    g.run_steps(1)  # builds the graph
    clocks = ClockSampler(lrank)
    clocks.start()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms, launches = time_device(g, args.steps, args.warmup)
    clocks.stop()
    ms = replica_max(ms)
    value = job_rate(ws, n_cells, args.steps, ms)
    dt, cfl, sim_t, two_half = g.step_info()
    divb = None
    if args.divb:
        last, nxt, e0, e1 = g.divb_info()
    phases = g.profile_steps(2)
    if args.divb:
        # words per cell: divergence passes 6 (the last 4), gradient passes 10
        words = 6 + 16 * last - 2
        divb = {"iterations_last_step": last, "max_divB_before_after_G": [e0, e1],
                "ms_per_step": round(phases["divb_clean"], 4),
                "algorithmic_bytes_per_step": words * 4 * n_cells,
                "hbm_gbs": round(words * 4 * n_cells / (phases["divb_clean"] / 1e3) / 1e9, 1),
                "settings": {k: v for k, v in divb_kw.items() if k.startswith("divB")}}
    # dominant kernel family: the RK stage kernel or the TVD sweep kernel
    fam = {"stage": ["stage1", "stage2", "stage3", "stage4"], "tvd": ["tvd_x", "tvd_y", "tvd_z"]}
    tot = {k: sum(phases[p] for p in v) for k, v in fam.items()}
    dom = max(tot, key=tot.get)
    launches_dom = fam[dom]
    mean_ms = tot[dom] / len(launches_dom)
    algo_words = ALGO_STAGE_WORDS if dom == "stage" else ALGO_TVD_WORDS
    bytes_per_launch = algo_words / len(launches_dom) * 4 * n_cells
    design_bytes_per_launch = sum(words_per_cell(p) for p in launches_dom) / len(launches_dom) * 4 * n_cells
    achieved = bytes_per_launch / (mean_ms / 1e3) / 1e9
    traffic = load_traffic().get(f"{dom}_f32_bytes_per_cell")
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak_gbs, "unit": "GB/s",
                "frac": round(achieved / peak_gbs, 4),
                "traffic": (traffic * n_cells if traffic else None),
                "kernel": f"k_stage (FP32, RK stages 1-4)" if dom == "stage" else "k_tvd_sweep (FP32, x/y/z)",
                "algorithmic_bytes_per_launch": bytes_per_launch, "mean_launch_ms": round(mean_ms, 4),
                "algorithmic_words_per_cell": f"{algo_words} per {len(launches_dom)} launches",
                "design_bytes_per_launch": design_bytes_per_launch,
                "peak_source": f"{peak_src} hbm_gbs"}
    if dom == "stage":
        roofline["limiter"] = ("instruction issue and dependency latency, not HBM (ncu: ~58 % issue active, "
                               "24-39 % DRAM throughput)")
    # whole-step bytes against HBM
    step_bytes = ALGO_STEP_WORDS * 4 * n_cells
    step_ms = ms / args.steps
    # end to end through the C ABI with host buffers
    e2e = None
    e2e_f32_host = None
    if not args.no_e2e:
        e2e_steps = max(4, min(args.steps, 50))
        e2e_ms, h2d, d2h, same, e2e_runs = time_e2e(g, e2e_steps, U)
        e2e_ms = replica_max(e2e_ms)
        e2e = {"value": job_rate(ws, n_cells, e2e_steps, e2e_ms), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e2e_steps,
               "ms_per_step": round(e2e_ms / e2e_steps, 3),
               "ms_per_step_runs": [round(x / e2e_steps, 3) for x in e2e_runs],
               "host_layout": "cState float64 (MURaM's default build)",
               "link_alone": time_link(h2d),
               "transfers": "asynchronous upload / download on copy streams, overlapping the neighbouring steps",
               "result_equals_synchronous_path": same}
        # the same with the float32 host layout of a SINGLE_PRECISION build
        f_ms, f_h2d, f_d2h, f_same, f_runs = time_e2e(g, e2e_steps, U, "float32")
        f_ms = replica_max(f_ms)
        e2e_f32_host = {"value": job_rate(ws, n_cells, e2e_steps, f_ms), "unit": UNIT,
                        "h2d_bytes_per_step": f_h2d, "d2h_bytes_per_step": f_d2h, "steps": e2e_steps,
                        "ms_per_step": round(f_ms / e2e_steps, 3),
                        "ms_per_step_runs": [round(x / e2e_steps, 3) for x in f_runs],
                        "host_layout": "cState float32 (MURaM built with SINGLE_PRECISION)",
                        "link_alone": time_link(f_h2d),
                        "result_equals_synchronous_path": f_same}
    # the per-routine entry points in ComputeSolution's order (how MURaM itself
    # calls the library through the drop-in shim), device-resident
    per_routine = None
    if not args.no_e2e:
        g.upload_state(U)
        g.exchange_grid(True)
        g.step_reference_order()
        g.synchronize()
        t0 = time.perf_counter()
        pr_steps = 3
        for _ in range(pr_steps):
            g.step_reference_order()
        g.synchronize()
        pr_ms = replica_max((time.perf_counter() - t0) * 1e3 / pr_steps)
        per_routine = {"value": job_rate(ws, n_cells, 1, pr_ms), "unit": UNIT, "ms_per_step": round(pr_ms, 3),
                       "steps": pr_steps, "calls": "SaveCons, 4 x (ConsToPrim, MHD_Residual, Source_Integrate_Tcheck, "
                       "exchange), TVDlimit, TCheck, exchange; host-timed, one host round trip per MHD_Residual"}
    g.close()
    del g
    # the compensated FP32 mode (rounding remainders carried through the RK
    # sums and the TVD sweeps) on the same box, timed the same way
    gc = context(32, compensated=1)
    gc.run_steps(1)
    gc.upload_state(U)
    ms_c, _ = time_device(gc, args.steps, args.warmup)
    ms_c = replica_max(ms_c)
    gc.close()
    del gc
    compensated = {"value": job_rate(ws, n_cells, args.steps, ms_c), "unit": UNIT,
                   "ms_per_step": round(ms_c / args.steps, 4), "steps": args.steps,
                   "cost_over_plain": round(ms_c / ms, 4)}
    # FP64 mode of the same box: throughput over --err-steps steps from the
    # initial state, and the per-field error of the FP32 runs (plain and
    # compensated) against it after the same steps.  The FP64 GPU mode matches
    # the reference CPU build to 1e-12 (tests), so it stands for the oracle here.
    fp64 = None
    fp32_err = None
    if not args.no_fp64:
        import numpy as np
        nerr = args.err_steps
        checkpoints = sorted({nerr, 2 * nerr})  # the 100-step bar and the configuration's 200-step run
        g64 = context(64)
        g64.run_steps(1)
        g64.upload_state(U)
        ms64, _ = time_device(g64, nerr, 0)
        ms64 = replica_max(ms64)
        value64 = job_rate(ws, n_cells, nerr, ms64)
        refs = {nerr: g64.download_state()[:, 2:-2, 2:-2, 2:-2]}
        for cp in checkpoints[1:]:
            g64.run_steps(cp - nerr)
            refs[cp] = g64.download_state()[:, 2:-2, 2:-2, 2:-2]
        ph64 = g64.profile_steps(2)
        g64.close()
        del g64
        stage64_ms = sum(ph64[f"stage{q}"] for q in range(1, 5)) / 4
        peak64 = fp64_peak_tflops()
        ach64 = FLOPS_STAGE_PER_CELL * n_cells / (stage64_ms / 1e3) / 1e12
        fp64 = {"value": value64, "unit": UNIT, "ms_per_step": ms64 / nerr, "steps": nerr,
                "fp32_over_fp64": value / value64,
                "roofline": {"bound": "fp64", "kernel": "k_stage_tm (FP64, RK stages 1-4)",
                             "achieved": round(ach64, 4), "peak": round(peak64, 4), "unit": "TFLOP/s",
                             "frac": round(ach64 / peak64, 4), "mean_launch_ms": round(stage64_ms, 4),
                             # the FP64 mode is compiled without FMA contraction (parity with the
                             # reference's no-FMA build): one flop per FP64 instruction, half the
                             # DGEMM's flops per instruction
                             "peak_without_fma": round(peak64 / 2, 4),
                             "frac_without_fma": round(ach64 / (peak64 / 2), 4),
                             "flops_per_cell_per_launch": FLOPS_STAGE_PER_CELL,
                             "peak_source": "measured: cuBLAS DGEMM 8192^3 via torch.matmul",
                             "hbm_frac": round(ALGO_STAGE_WORDS / 4 * 8 * n_cells / (stage64_ms / 1e3) / 1e9
                                               / peak_gbs, 4)},
                "phases_ms": {k: round(v, 3) for k, v in ph64.items()}}
        fp32_err = {"steps": checkpoints, "against": "FP64 GPU mode (= reference CPU build to 1e-12)",
                    "fields": ["rho", "Mx", "My", "Mz", "e", "Bx", "By", "Bz"]}
        for comp in (0, 1):
            p32 = gpumhd.default_params(wl["nx"], wl["ny"], wl["nz"], wl["dx"], precision=32,
                                        periodic_x=wl["periodic_x"], grav=wl["grav"], compensated=comp, **divb_kw)
            g32 = gpumhd.MuramGPU(p32, device=lrank, eos_path=EOS_BENCH)
            g32.upload_state(U)
            key = "compensated" if comp else "plain"
            fp32_err[key] = {}
            done = 0
            for cp in checkpoints:
                g32.run_steps(cp - done)
                done = cp
                got = g32.download_state()[:, 2:-2, 2:-2, 2:-2]
                ref = refs[cp]
                d = got - ref
                l2 = [float(np.sqrt(np.sum(d[f] ** 2) / np.sum(ref[f] ** 2))) for f in range(8)]
                linf = [float(np.max(np.abs(d[f])) / np.max(np.abs(ref[f]))) for f in range(8)]
                fp32_err[key][str(cp)] = {"rel_l2": [float(f"{x:.3e}") for x in l2],
                                          "rel_linf": [float(f"{x:.3e}") for x in linf],
                                          "max_rel_l2": float(f"{max(l2):.3e}")}
            g32.close()
        del refs
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded stratified box, generated EOS table 3000x3000)",
        "config": {"workload": f"stratified 128(vertical) x {wl['ny']} x {wl['nz']} at 16 km, closed top/bottom, "
                               "gravity 2.74e4"
                               + (", divB cleaning after every TVD pass" if args.divb else "")
                               + (", open bottom / closed top (MURaM's physical x boundaries)" if args.xbnd else "")
                               + (f", Spitzer conduction (coefficient {args.spitzer:g})" if args.spitzer > 0 else ""),
                   "cells": n_cells, "precision": "fp32 storage+arithmetic",
                   "l2": "inputs larger than L2 (state 0.64 GB per buffer)",
                   "tvd_branch": "two half steps" if two_half else "single", "dt_s": dt, "cfl": cfl,
                   "graph": "one CUDA graph per step", "replicas": ws},
        "roofline": roofline,
        "step_hbm_gbs": round(step_bytes / (step_ms / 1e3) / 1e9, 1),
        "phases_ms": {k: round(v, 4) for k, v in phases.items()},
        "e2e": e2e,
        "e2e_f32_host": e2e_f32_host,
        "per_routine": per_routine,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "fp32_compensated": compensated,
        "fp64": fp64,
        "fp32_error": fp32_err,
    }
    if divb:
        line["divb"] = divb
    if rank == 0 and ws == 1 and not args.no_cpu:
        cores = min(os.cpu_count() or 1, 16)
        rate, wall = cpu_baseline(cores, 8)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{cores} processes x 8 steps of a {SAMPLE['nx']}x{SAMPLE['ny']}x"
                                          f"{SAMPLE['nz']} column of the workload (FP64), {wall:.1f} s wall"}
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_ensemble(args):
    """Batched ensemble: 64 independent periodic FP32 boxes, sides drawn from
    {32, 48, 64, 96, 128} per axis, each with its own seed, velocity rms
    log-uniform in [0.2, 2] km/s and field rms log-uniform in [10, 500] G.
    Each box is autotuned, then all advance together in one graph launch
    (while-loop body = one step of every box).  Reported against the same
    boxes advanced one box per launch (each box's own per-step graph, box
    after box)."""
    import numpy as np
    import torch
    from muram_main_gb300 import eos_table, gpumhd, initial
    eos_table.ensure_table(EOS_BENCH, "bench")
    tab = initial.EosTable(EOS_BENCH)
    rng = np.random.default_rng(2024)
    sides = [32, 48, 64, 96, 128]
    nbox = args.boxes
    boxes, states, dims, cells = [], [], [], 0
    for b in range(nbox):
        nx, ny, nz = (int(x) for x in rng.choice(sides, 3))
        v_rms = float(np.exp(rng.uniform(np.log(0.2e5), np.log(2.0e5))))
        b_rms = float(np.exp(rng.uniform(np.log(10.0), np.log(500.0))))
        U = initial.periodic_box(tab, nx, ny, nz, dx=3.2e6, v_rms=v_rms, b_rms_gauss=b_rms, seed=1000 + b)
        p = gpumhd.default_params(nx, ny, nz, 3.2e6, precision=32)
        g = gpumhd.MuramGPU(p, eos_path=EOS_BENCH)
        g.upload_state(U)
        boxes.append(g)
        states.append(U)
        dims.append((nx, ny, nz))
        cells += nx * ny * nz
    steps = args.steps
    tune = [g.autotune(trial_steps=2) for g in boxes]
    kernels = [g.tuning() for g in boxes]

    def reset():
        for g, U in zip(boxes, states):
            g.upload_state(U)
        torch.cuda.synchronize()

    # one box per launch: each box's own per-step graph, box after box
    reset()
    for g in boxes:
        g.run_steps(1)
    reset()
    t0 = time.perf_counter()
    for g in boxes:
        g.enqueue_steps(steps)
        g.synchronize()
    t_single = time.perf_counter() - t0
    # the ensemble: one launch of the while-loop graph for all boxes and steps
    reset()
    ens = gpumhd.MuramEnsemble(boxes)
    stream = torch.cuda.ExternalStream(ens.stream)

    def timed(nsteps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        n0 = ens.launch_count
        e0.record(stream)
        ens.enqueue_steps(nsteps)
        e1.record(stream)
        ens.synchronize()
        return e0.elapsed_time(e1), ens.launch_count - n0

    # Launch shapes for the ensemble (gpumhd_ensemble_autotune): each box's
    # own autotuned shapes suit the box alone, which must fill the GPU by
    # itself; inside the ensemble longer stage z chunks and TVD chunks may
    # pay.  Timed from the current states, which the autotuner restores.
    reset()
    ens.run_steps(args.warmup)
    reset()
    tune_ms = ens.autotune(trial_steps=8)
    chosen = [g.tuning() for g in boxes]
    own = sum(1 for c, k in zip(chosen, kernels) if c["stage_zchunk"] == k["stage_zchunk"]
              and c["tvd_chunk"] == k["tvd_chunk"])
    whole = sum(1 for c, (nx, ny, nz) in zip(chosen, dims) if c["stage_zchunk"] == nz)
    reset()
    ens.run_steps(args.warmup)
    reset()
    ms, launches = timed(steps)
    value = cells * steps / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded periodic boxes, generated EOS table 3000x3000)",
        "config": {"workload": f"ensemble of {nbox} periodic FP32 boxes, sides in {sides}", "cells": cells,
                   "graph": "one launch: while-loop graph, body = one step of every box, branches largest "
                            "box first",
                   "autotuned": True},
        "ensemble_autotune": {"trial_ms_per_step": round(tune_ms, 3), "boxes_on_own_shapes": own,
                              "boxes_on_whole_z_chunks": whole,
                              "tvd_chunks": sorted({c["tvd_chunk"] for c in chosen})},
        "one_box_per_launch": {"value": cells * steps / t_single, "unit": UNIT,
                               "wall_s": round(t_single, 4)},
        "ensemble_over_one_box_per_launch": value / (cells * steps / t_single),
        "gpu_launches": launches,
        "tuning": {"stage_kernel_tma": sum(1 for k in kernels if k["stage_kernel"] == 0),
                   "best_ms_per_step_sum": round(sum(tune), 4)},
    }
    ens.close()
    for g in boxes:
        g.close()
    print(json.dumps(line))


def run_large(args):
    """Large single box: 256 (MURaM dimension 0) x 1024 x 1024 = 2.7e8 cells in
    FP32.  Its state is the periodic 4x4 tiling (in y and z) of a seeded
    256^3 periodic box from the 64^3 configuration's generators, built on the
    device, so that the host never holds the 17 GB float64 state."""
    import torch
    from muram_main_gb300 import eos_table, gpumhd, initial
    eos_table.ensure_table(EOS_BENCH, "bench")
    tab = initial.EosTable(EOS_BENCH)
    nx, ny, nz = 256, 1024, 1024
    seed_box = initial.periodic_box(tab, 256, 256, 256, dx=3.2e6, seed=99)

    def large_box(prec):
        gs = gpumhd.MuramGPU(gpumhd.default_params(256, 256, 256, 3.2e6, precision=prec), eos_path=EOS_BENCH)
        gs.upload_state(seed_box)
        gl = gpumhd.MuramGPU(gpumhd.default_params(nx, ny, nz, 3.2e6, precision=prec), eos_path=EOS_BENCH)
        gl.tile_from(gs)
        gs.close()
        return gl

    g = large_box(32)
    g.run_steps(1)
    ms, launches = time_device(g, args.steps, args.warmup)
    n_cells = nx * ny * nz
    phases = g.profile_steps(2)
    value = n_cells * args.steps / (ms / 1e3)
    step_bytes = ALGO_STEP_WORDS * 4 * n_cells
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded periodic box, generated EOS table 3000x3000)",
        "config": {"workload": "periodic 256(dim 0) x 1024 x 1024 FP32, 4x4 tiling of a seeded 256^3 box",
                   "cells": n_cells, "l2": "inputs larger than L2 (state 8.8 GB per buffer)"},
        "step_hbm_gbs": round(step_bytes / (ms / args.steps / 1e3) / 1e9, 1),
        "phases_ms": {k: round(v, 4) for k, v in phases.items()},
        "gpu_launches": launches,
    }
    g.close()
    if not args.no_fp64:
        # FP32 against the FP64 mode after the configuration's 50 steps from the
        # same tiled state (the FP64 mode matches the reference CPU build to 1e-12)
        import numpy as np
        nerr = 50
        res = {}
        for prec in (64, 32):
            gl = large_box(prec)
            t0 = time.perf_counter()
            gl.run_steps(nerr)
            res[prec] = (gl.download_state()[:, 2:-2, 2:-2, 2:-2], time.perf_counter() - t0)
            gl.close()
        ref, got = res[64][0], res[32][0]
        l2 = [float(f"{np.sqrt(np.sum((got[f] - ref[f]) ** 2) / np.sum(ref[f] ** 2)):.3e}") for f in range(8)]
        line["fp32_error"] = {"steps": nerr, "against": "FP64 GPU mode (= reference CPU build to 1e-12)",
                              "fields": ["rho", "Mx", "My", "Mz", "e", "Bx", "By", "Bz"], "rel_l2": l2,
                              "max_rel_l2": max(l2)}
        line["fp64"] = {"value": n_cells * nerr / res[64][1], "unit": UNIT, "steps": nerr,
                        "note": "host-timed run_steps incl. graph capture"}
        del res, ref, got
    del seed_box
    print(json.dumps(line))


def run_adjoint(args):
    """Adjoint sensitivity: a 128^3 periodic box (the 64^3 configuration's
    generators), J = sum over the top 8 layers of dimension 0 (vertical) of a
    seeded mask times B_x^2 after 20 fixed-dt steps.  dJ/dU_0 from the
    library's adjoint (FP64, checkpoints every 5 steps), checked against
    central differences of the FP64 forward along 32 seeded directions.  The
    check runs with an ideal-gas table, whose bilinear lookup is exact and
    smooth; with the Saha table the step is piecewise smooth (the bilinear
    table has a kink at every node) and central differences cross thousands of
    kinks on this machine, so that check is reported separately on 8 directions.
    The FP32 forward's J is reported beside the FP64 one."""
    import numpy as np
    from muram_main_gb300 import eos_table, gpumhd, initial
    eos_table.ensure_table(EOS_BENCH, "bench")
    eos_ideal = os.path.join(DATA_DIR, "eos_ideal.dat")
    eos_table.ensure_table(eos_ideal, "ideal")
    n, steps, every, eps = 128, 20, 5, 1e-8
    mask = np.random.default_rng(8).uniform(0.0, 1.0, (n, n, 8))

    def J(U):
        return float(np.sum(mask * U[5, 2:-2, 2:-2, -10:-2] ** 2))

    # TVD diffusion off: every TVD flux is multiplied by zero (tvd_coeff, the
    # boundary viscosity / resistivity profiles and the x hyperdiffusion all
    # 0), so the sweeps are the identity and the limiter's kinks drop out of
    # both the forward step and its adjoint
    no_tvd = dict(tvd_coeff=[0.0] * 4, tvd_visc_bnd=[0.0, 0.0], tvd_eta_bnd=[0.0, 0.0])

    def case(eos_path, ndir, tvd_off=False):
        tab = initial.EosTable(eos_path)
        U0 = initial.periodic_box(tab, n, n, n, seed=4)
        kw = dict(no_tvd) if tvd_off else {}

        def params(**more):
            p = gpumhd.default_params(n, n, n, 3.2e6, **kw, **more)
            if tvd_off:
                p.tvd[4] = 0.0  # tvd_vhyp
            return p

        g = gpumhd.MuramGPU(params(), eos_path=eos_path)
        g.upload_state(U0)
        dt = float(g.run_steps(1)[0]) * 0.6
        g.close()
        boxes = {prec: gpumhd.MuramGPU(params(precision=prec, autostep=0, dt=dt), eos_path=eos_path)
                 for prec in (64, 32)}
        g = boxes[64]

        def forward(box, U):
            box.upload_state(U)
            box.synchronize()
            t0 = time.perf_counter()
            box.run_steps(steps)
            t = time.perf_counter() - t0
            return box.download_state(), t

        UT, _ = forward(g, U0)
        _, t_fwd = forward(g, U0)
        UT32, _ = forward(boxes[32], U0)
        lam = np.zeros_like(UT)
        lam[5, 2:-2, 2:-2, -10:-2] = 2.0 * mask * UT[5, 2:-2, 2:-2, -10:-2]
        g.upload_state(U0)
        g.adjoint(1, lam, checkpoint_every=1)  # warm-up (allocation, first launches)
        g.upload_state(U0)
        g.synchronize()
        t0 = time.perf_counter()
        grad = g.adjoint(steps, lam, checkpoint_every=every)
        t_adj = time.perf_counter() - t0
        rng = np.random.default_rng(12)
        scale = np.sqrt(np.mean(U0[:, 2:-2, 2:-2, 2:-2] ** 2, axis=(1, 2, 3)))
        ads, fds = [], []
        for _ in range(ndir):
            v = np.zeros_like(U0)
            v[:, 2:-2, 2:-2, 2:-2] = rng.standard_normal((8, n, n, n)) * scale[:, None, None, None]
            v = initial.fill_ghosts(v, periodic_x=True)
            jp = J(forward(g, U0 + eps * v)[0])
            jm = J(forward(g, U0 - eps * v)[0])
            fds.append((jp - jm) / (2 * eps))
            ads.append(float(np.sum(grad * v)))
        ads, fds = np.array(ads), np.array(fds)
        rel = np.abs(ads - fds) / np.abs(fds)
        rel_rms = np.abs(ads - fds) / np.sqrt(np.mean(fds ** 2))
        for b in boxes.values():
            b.close()
        return {"dt_s": dt, "forward_s": round(t_fwd, 4), "adjoint_s": round(t_adj, 4),
                "fd_check": {"directions": ndir, "eps": eps, "rel_err_median": float(np.median(rel)),
                             "rel_err_max": float(np.max(rel)),
                             "err_over_rms_derivative_max": float(np.max(rel_rms))},
                "objective": {"fp64": J(UT), "fp32": J(UT32), "fp32_rel_diff": abs(J(UT32) - J(UT)) / abs(J(UT))}}

    smooth = case(eos_ideal, 32)
    smooth_no_tvd = case(eos_ideal, 32, tvd_off=True)
    saha = case(EOS_BENCH, 8)
    line = {
        "metric": "adjoint/forward time, with dJ/dU0 checked by central differences",
        "value": smooth["adjoint_s"] / smooth["forward_s"], "unit": "adjoint time / forward time",
        "n_gpus": 1, "steps": steps, "higher_is_better": False, "dtype": "f64",
        "data": "synthetic (seeded periodic box; ideal-gas and generated Saha EOS tables)",
        "config": {"workload": f"periodic {n}^3, objective: mask-weighted B_x^2 over the top 8 layers of "
                               "dimension 0, fixed dt", "checkpoint_every": every},
        "ideal_gas_table": smooth,
        "ideal_gas_table_tvd_off": smooth_no_tvd,
        "saha_table": saha,
    }
    print(json.dumps(line))


def run_reference(args):
    ws, rank, _ = world()
    if rank != 0:
        return
    cores = min(os.cpu_count() or 1, 16)
    steps = args.steps
    t0 = time.perf_counter()
    rate, wall = cpu_baseline(cores, steps, args.warmup)
    line = {
        "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": ws, "steps": steps, "warmup": args.warmup,
        "ms_per_step": SAMPLE["nx"] * SAMPLE["ny"] * SAMPLE["nz"] * cores / rate * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded stratified box, generated EOS table 3000x3000)",
        "config": {"workload": "stratified 128(vertical) x 384 x 384 at 16 km, closed top/bottom, gravity 2.74e4",
                   "sample": "128x32x32 columns, one per core"},
        "impl": "reference",
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} processes x {steps} steps (after {args.warmup} warm-up steps) of a "
                                   f"128x32x32 column of the workload (FP64), {wall:.1f} s wall"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": round(time.perf_counter() - t0, 2),
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 leg (and the FP32 error report)")
    ap.add_argument("--err-steps", type=int, default=100, help="steps of the FP64 leg and the FP32 error report")
    ap.add_argument("--workload", default="stratified", choices=["stratified", "ensemble", "large", "adjoint"],
                    help="stratified: the headline box; ensemble: 64 uneven boxes in one launch; "
                         "large: one 1024x1024x256 box; adjoint: gradient of a 20-step objective")
    ap.add_argument("--boxes", type=int, default=64, help="boxes of the ensemble workload")
    ap.add_argument("--ny", type=int, default=0,
                    help="horizontal size (y = z) of the stratified box instead of 384, for profiler captures")
    ap.add_argument("--spitzer", type=float, default=0.0,
                    help="stratified workload with hyperbolic Spitzer conduction of this coefficient")
    ap.add_argument("--xbnd", action="store_true",
                    help="stratified workload with MURaM's physical x boundaries (open bottom) instead of the mirror")
    ap.add_argument("--divb", action="store_true",
                    help="stratified workload with divB cleaning after every TVD pass (reference test settings)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ensemble":
        run_ensemble(args)
    elif args.workload == "large":
        run_large(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
