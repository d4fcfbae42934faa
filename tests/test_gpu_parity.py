"""GPU parity through the C ABI against the reference's golden fixtures and the oracle.

FP64 tolerance: relative L-infinity (max |gpu - ref| / max |ref| per field)
of 1e-12 -- the bar for the FP64 GPU mode.  The GPU's exp/log differ from the
host C library by at most a few ulp, so exact equality is not expected where
the EOS is involved; the observed errors are printed.
FP32 tolerance: relative L2 per field of 1e-5 after the run.
"""
import os

import numpy as np
import pytest

import helpers as H
from muram_main_gb300 import gpumhd, initial

TOL64 = 1e-12
TOL32_L2 = 1e-5

pytestmark = pytest.mark.gpu


# stage_kernel 0: TMA plane loads + tensor-memory z ring (where the box allows
# it); 1: the plain-load stage kernel.  Both must meet the same bars.
KERNELS = [0, 1]


def ctx_for(hp, precision=64, stage_kernel=0):
    p = H.gpu_params(hp, precision)
    p.stage_kernel = stage_kernel
    return gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL)


def check(name, got, ref, tol=TOL64):
    e = H.rel_linf(got, ref)
    print(f"{name}: rel Linf per field {np.array2string(e, precision=2)}")
    assert np.all(e <= tol), (name, e)


def test_cons_to_prim(gpu_lib):
    d, hp = H.load_case("periodic")
    g = ctx_for(hp)
    g.upload_state(d["init_U"])
    g.ConsToPrim()
    check("ConsToPrim U", g.download_state(), d["s1_c2p_U"])
    aux = np.stack([g.download_field(w) for w in range(gpumhd.FIELD_PRES, gpumhd.FIELD_AMB + 1)])
    check("ConsToPrim pres/temp/ne/rhoi/amb", aux, d["s1_c2p_aux"])


@pytest.mark.parametrize("kernel", KERNELS)
def test_mhd_residual_and_dt(gpu_lib, kernel):
    d, hp = H.load_case("periodic")
    g = ctx_for(hp, stage_kernel=kernel)
    g.upload_state(d["s1_c2p_U"])
    g.upload_field(gpumhd.FIELD_PRES, d["s1_c2p_aux"][0])
    g.upload_state(np.zeros_like(d["s1_c2p_U"]), gpumhd.FIELD_RES)
    g.Adjust_Valf_Max()
    assert list(g.limits()) == list(d["limits"][:3])
    dt = g.MHD_Residual()
    assert abs(dt / d["s1_res_dt"][0] - 1) <= TOL64
    check("MHD_Residual", g.download_state(gpumhd.FIELD_RES), d["s1_res_R"])


def test_source_integrate_and_exchange(gpu_lib):
    d, hp = H.load_case("periodic")
    g = ctx_for(hp)
    g.upload_state(d["s1_c2p_U"])
    g.upload_state(d["init_U"], gpumhd.FIELD_U0)
    g.upload_state(d["s1_res_R"], gpumhd.FIELD_RES)
    g.upload_field(gpumhd.FIELD_PRES, d["s1_c2p_aux"][0])
    g.Adjust_Valf_Max()
    cfl = g.Sync_timestep(g.params.dt_rad, float(d["s1_res_dt"][0]))
    assert g.step_info()[0] == d["dts"][0] and cfl == d["dts"][1]
    g.Source_Integrate_Tcheck(1)
    check("Source_Integrate_Tcheck", g.download_state(), d["s1_si_U"])
    assert not g.download_state(gpumhd.FIELD_RES).any()
    g.exchange_grid(True)
    check("exchange+BC", g.download_state(), d["s1_bc_U"])


@pytest.mark.parametrize("name", H.CASES)
def test_tvd_and_tcheck(gpu_lib, name):
    d, hp = H.load_case(name)
    g = ctx_for(hp)
    t = int(d["trace_step"])
    dt = float(d["dts"][3 * (t - 1)])
    cfl = float(d["dts"][3 * (t - 1) + 1])
    g.upload_state(d["s4_bc_U"])
    g.upload_field(gpumhd.FIELD_PRES, d["s4_c2p_aux"][0])
    g.upload_field(gpumhd.FIELD_PRES, d["s4_c2p_aux"][0])
    if cfl <= g.params.CFL_tvd:
        g.TVDlimit(dt)
    else:
        g.TVDlimit(0.5 * dt)
        g.exchange_grid(False)
        g.TVDlimit(0.5 * dt)
    check(f"TVDlimit[{name}]", g.download_state(), d["tvd_U"])
    g.TCheck()
    check(f"TCheck[{name}]", g.download_state(), d["tck_U"])
    g.exchange_grid(True)
    check(f"final exchange[{name}]", g.download_state(), d["end_U"])


@pytest.mark.parametrize("name", H.CASES)
def test_reference_order_steps(gpu_lib, name):
    d, hp = H.load_case(name)
    g = ctx_for(hp)
    g.upload_state(d["input_U"])
    g.exchange_grid(True)
    dts = [g.step_reference_order()[0] for _ in range(int(d["steps"]))]
    assert np.allclose(dts, d["dts"].reshape(-1, 3)[:, 0], rtol=TOL64, atol=0)
    check(f"per-routine steps[{name}]", g.download_state(), d["final_U"])


@pytest.mark.parametrize("name", H.CASES)
@pytest.mark.parametrize("capture", [0, 1])
@pytest.mark.parametrize("kernel", KERNELS)
def test_fused_steps(gpu_lib, name, capture, kernel):
    d, hp = H.load_case(name)
    g = ctx_for(hp, stage_kernel=kernel)
    g.upload_state(d["input_U"])
    dts = g.run_steps(int(d["steps"]), capture=bool(capture))
    assert np.allclose(dts, d["dts"].reshape(-1, 3)[:, 0], rtol=TOL64, atol=0)
    check(f"fused steps[{name}, graph={capture}, kernel={kernel}]", g.download_state(), d["final_U"])
    assert g.step_info()[3] == (1 if name == "two_half_tvd" else 0)


def _oracle_run(hp, U, steps):
    from oracle import oracle as O
    eos = O.Eos(H.EOS_SMALL)
    st = O.State(H.oracle_params(hp), U)
    dts = st.step(eos, steps)
    return st.U, dts


def test_fused_fp64_64cubed_bench_table_100_steps(gpu_lib):
    """The plain FP64 step at its stated size: a 64^3 fully periodic box at 32 km
    on the full 3000 x 3000 EOS table (uniform rho = 3e-7 g/cm^3 at 6000 K,
    1 km/s rms velocity and 100 G rms divergence-free field on wavenumbers
    1-8), 100 fused steps at CFL 0.8 with TVD diffusion: dt equal to 1e-12 at
    every step and relative L-infinity <= 1e-12 per field against the oracle."""
    from muram_main_gb300 import eos_table
    from oracle import oracle as O
    path = os.path.join(H.ROOT, "muram_main_gb300", "_data", "eos_bench.dat")
    eos_table.ensure_table(path, "bench")
    tab = initial.EosTable(path)
    U = initial.periodic_box(tab, 64, 64, 64, dx=3.2e6, seed=2024)
    st = O.State(O.make_params(64, 64, 64, 3.2e6), U)
    dts_ref = [x[0] for x in st.step(O.Eos(path), 100)]
    g = gpumhd.MuramGPU(gpumhd.default_params(64, 64, 64, 3.2e6), eos_path=path)
    g.upload_state(U)
    dts = g.run_steps(100)
    assert np.allclose(dts, dts_ref, rtol=TOL64, atol=0), np.max(np.abs(np.array(dts) / dts_ref - 1))
    assert g.step_info()[3] == 0  # the single-sweep TVD branch (cfl = 0.8 <= CFL_tvd)
    check("FP64 fused vs oracle, 64^3 at 32 km, 3000x3000 table, 100 steps", H.interior(g.download_state()),
          H.interior(st.U))


@pytest.mark.parametrize("kernel", KERNELS)
def test_fused_vs_oracle_anisotropic(gpu_lib, kernel):
    tab = initial.EosTable(H.EOS_SMALL)
    hp = dict(nx=40, ny=24, nz=20, dx=2.4e6, dy=3.2e6, dz=4.0e6)
    U = initial.periodic_box(tab, 40, 24, 20, dx=2.4e6, dy=3.2e6, dz=4.0e6, seed=77)
    ref, dts_ref = _oracle_run(hp, U, 12)
    p = gpumhd.default_params(40, 24, 20, 2.4e6, dy=3.2e6, dz=4.0e6, stage_kernel=kernel)
    g = gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL)
    g.upload_state(U)
    dts = g.run_steps(12)
    assert np.allclose(dts, [x[0] for x in dts_ref], rtol=TOL64, atol=0)
    check("fused vs oracle, 40x24x20, 12 steps", g.download_state(), ref)


def test_fused_fp64_100_steps(gpu_lib):
    """The FP64 bar: relative L-infinity <= 1e-12 after 100 steps (32^3 periodic box)."""
    tab = initial.EosTable(H.EOS_SMALL)
    hp = dict(nx=32, ny=32, nz=32)
    U = initial.periodic_box(tab, 32, 32, 32, seed=5)
    ref, _ = _oracle_run(hp, U, 100)
    g = gpumhd.MuramGPU(gpumhd.default_params(32, 32, 32, 3.2e6), eos_path=H.EOS_SMALL)
    g.upload_state(U)
    g.run_steps(100)
    check("FP64 fused vs oracle, 32^3, 100 steps", H.interior(g.download_state()), H.interior(ref))


@pytest.mark.parametrize("kernel", KERNELS)
def test_fused_fp32_error_vs_fp64_oracle(gpu_lib, kernel):
    """FP32 storage and arithmetic: relative L2 per field after 100 steps."""
    tab = initial.EosTable(H.EOS_SMALL)
    hp = dict(nx=32, ny=32, nz=32)
    U = initial.periodic_box(tab, 32, 32, 32, seed=5)
    ref, _ = _oracle_run(hp, U, 100)
    g = gpumhd.MuramGPU(gpumhd.default_params(32, 32, 32, 3.2e6, precision=32, stage_kernel=kernel),
                        eos_path=H.EOS_SMALL)
    g.upload_state(U)
    g.run_steps(100)
    e = H.rel_l2(H.interior(g.download_state()), H.interior(ref))
    print("FP32 vs FP64 oracle rel L2 per field:", np.array2string(e, precision=2))
    assert np.all(e <= TOL32_L2), e


def test_fp32_reference_order_steps_vs_fp64_oracle(gpu_lib):
    """FP32 through the per-routine entry points (MURaM's drop-in use: ConsToPrim,
    MHD_Residual, Source_Integrate_Tcheck, TVDlimit, ... in ComputeSolution's
    order): relative L2 per field after 40 steps, the FP32 bar."""
    tab = initial.EosTable(H.EOS_SMALL)
    U = initial.periodic_box(tab, 32, 32, 32, seed=5)
    ref, _ = _oracle_run(dict(nx=32, ny=32, nz=32), U, 40)
    g = gpumhd.MuramGPU(gpumhd.default_params(32, 32, 32, 3.2e6, precision=32), eos_path=H.EOS_SMALL)
    g.upload_state(U)
    g.exchange_grid(True)
    for _ in range(40):
        g.step_reference_order()
    e = H.rel_l2(H.interior(g.download_state()), H.interior(ref))
    print("FP32 per-routine vs FP64 oracle rel L2 per field:", np.array2string(e, precision=2))
    assert np.all(e <= TOL32_L2), e
    g.close()


@pytest.mark.parametrize("precision", [64, 32])
def test_cons_to_prim_outputs_are_those_of_the_call(gpu_lib, precision):
    """ConsToPrim's temperature, n_e, rho_i and amb are formed on first access
    from the density and internal energy the call saw: steps that change the
    state afterwards leave them as they were, a second ConsToPrim replaces
    them, and the values equal, bit for bit, those read right after the call."""
    d, hp = H.load_case("periodic")
    aux = range(gpumhd.FIELD_TEMP, gpumhd.FIELD_AMB + 1)
    ref = ctx_for(hp, precision=precision)
    ref.upload_state(d["init_U"])
    ref.ConsToPrim()
    at_once = np.stack([ref.download_field(w) for w in aux])
    ref.close()
    g = ctx_for(hp, precision=precision)
    g.upload_state(d["init_U"])
    g.exchange_grid(True)
    g.SaveCons()
    g.ConsToPrim()
    g.Adjust_Valf_Max()
    dt_mhd = g.MHD_Residual()
    g.Sync_timestep(g.params.dt_rad, dt_mhd)
    g.Source_Integrate_Tcheck(1)
    g.exchange_grid(True)
    later = np.stack([g.download_field(w) for w in aux])
    assert np.array_equal(later, at_once)
    # the next stage's ConsToPrim: its own outputs, as read at once from its state
    U1 = g.download_state()
    g.ConsToPrim()
    second = np.stack([g.download_field(w) for w in aux])
    h = ctx_for(hp, precision=precision)
    h.upload_state(U1)
    h.ConsToPrim()
    assert np.array_equal(second, np.stack([h.download_field(w) for w in aux]))
    assert not np.array_equal(second, at_once)
    g.close()
    h.close()


def test_fp32_cons_to_prim_outputs(gpu_lib):
    """ConsToPrim's five EOS outputs in FP32 (float table lookups) against the
    FP64 routine on the reference fixture's state: the FP32 bar, relative L2
    per field <= 1e-5 (measured 3.5e-8 for the pressure, 2.3e-6 for n_e,
    whose logarithm varies fastest across the table cells)."""
    d, hp = H.load_case("periodic")
    out = {}
    for prec in (64, 32):
        g = ctx_for(hp, precision=prec)
        g.upload_state(d["init_U"])
        g.ConsToPrim()
        out[prec] = np.stack([g.download_field(w) for w in range(gpumhd.FIELD_PRES, gpumhd.FIELD_AMB + 1)])
        g.close()
    e = H.rel_l2(out[32], out[64])
    print("FP32 ConsToPrim pres/temp/ne/rhoi/amb rel L2:", np.array2string(e, precision=2))
    assert np.all(e <= TOL32_L2), e


def test_fp32_stage_kernels_agree_on_stratified_box(gpu_lib):
    """Closed x with gravity, partial tiles in every direction (36 x 20 x 12):
    the TMA / tensor-memory and the plain-load stage kernels give the same
    FP32 state after 10 steps, to float rounding."""
    tab = initial.EosTable(H.EOS_SMALL)
    U = initial.stratified_box(tab, 36, 20, 12, seed=3)
    out = []
    for kernel in KERNELS:
        p = gpumhd.default_params(36, 20, 12, 1.6e6, precision=32, periodic_x=0, grav=2.74e4, stage_kernel=kernel)
        g = gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL)
        g.upload_state(U)
        g.run_steps(10)
        out.append(g.download_state())
        g.close()
    e = H.rel_linf(out[0], out[1])
    print("TMA vs plain-load stage kernel, FP32, rel Linf:", np.array2string(e, precision=2))
    assert np.all(e <= 1e-5), e


def test_fp32_shape_without_tma_rows(gpu_lib):
    """nx = 30: rows of 34 floats are not 16-byte multiples, so the context
    takes the plain-load kernel; it still meets the FP32 bar (20 steps)."""
    tab = initial.EosTable(H.EOS_SMALL)
    hp = dict(nx=30, ny=16, nz=12)
    U = initial.periodic_box(tab, 30, 16, 12, seed=8)
    ref, _ = _oracle_run(hp, U, 20)
    g = gpumhd.MuramGPU(gpumhd.default_params(30, 16, 12, 3.2e6, precision=32), eos_path=H.EOS_SMALL)
    g.upload_state(U)
    g.run_steps(20)
    e = H.rel_l2(H.interior(g.download_state()), H.interior(ref))
    assert np.all(e <= TOL32_L2), e


def test_fp32_compensated_rk_updates(gpu_lib):
    """FP32 with compensated (Kahan) RK updates: meets the FP32 bar after 100
    steps, and its state differs from the plain FP32 run (the remainders are
    carried)."""
    tab = initial.EosTable(H.EOS_SMALL)
    hp = dict(nx=32, ny=32, nz=32)
    U = initial.periodic_box(tab, 32, 32, 32, seed=5)
    ref, _ = _oracle_run(hp, U, 100)
    errs = {}
    states = {}
    for comp in (0, 1):
        g = gpumhd.MuramGPU(gpumhd.default_params(32, 32, 32, 3.2e6, precision=32, compensated=comp),
                            eos_path=H.EOS_SMALL)
        g.upload_state(U)
        g.run_steps(100)
        states[comp] = H.interior(g.download_state())
        errs[comp] = H.rel_l2(states[comp], H.interior(ref))
        g.close()
    print("FP32 rel L2 per field, plain:", np.array2string(errs[0], precision=2))
    print("FP32 rel L2 per field, compensated:", np.array2string(errs[1], precision=2))
    assert np.all(errs[1] <= TOL32_L2), errs[1]
    assert not np.array_equal(states[0], states[1])


def test_fp32_compensated_stratified_200_steps(gpu_lib):
    """The stratified configuration at its run length (128 vertical x 64 x 64
    at 16 km on the 3000 x 3000 table, closed x, gravity 2.74e4), 200 steps:
    compensated FP32 -- the rounding remainders carried through the RK stage
    sums and the TVD sweeps -- meets relative L2 <= 1e-5 per field against the
    FP64 mode (which matches the reference to 1e-12), and improves on plain
    FP32 in the vertical momentum, the field hydrostatic balance makes the
    most sensitive to rounding."""
    import bench
    from muram_main_gb300 import eos_table
    eos_table.ensure_table(bench.EOS_BENCH, "bench")
    U = bench.make_state(128, 64, 64, seed=7)
    res = {}
    for prec, comp in ((64, 0), (32, 0), (32, 1)):
        p = gpumhd.default_params(128, 64, 64, 1.6e6, precision=prec, periodic_x=0, grav=2.74e4, compensated=comp)
        g = gpumhd.MuramGPU(p, eos_path=bench.EOS_BENCH)
        g.upload_state(U)
        g.run_steps(200)
        res[(prec, comp)] = H.interior(g.download_state())
        g.close()
    ref = res[(64, 0)]
    e0 = H.rel_l2(res[(32, 0)], ref)
    e1 = H.rel_l2(res[(32, 1)], ref)
    print("stratified 200 steps, FP32 rel L2 -- plain:", np.array2string(e0, precision=2),
          "compensated:", np.array2string(e1, precision=2))
    assert np.all(e1 <= TOL32_L2), e1
    assert e1[1] < e0[1]


@pytest.mark.parametrize("name", ["two_half_tvd", "closed_gravity"])
def test_fp32_compensated_fixtures(gpu_lib, name):
    """Compensated FP32 on the reference's fixtures: two half TVD passes (the
    remainders carried through both), and the closed x with gravity (ghost
    images of the mirror rule)."""
    d, hp = H.load_case(name)
    p = H.gpu_params(hp, 32)
    p.compensated = 1
    g = gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL)
    g.upload_state(d["input_U"])
    dts = g.run_steps(int(d["steps"]))
    assert np.allclose(dts, d["dts"].reshape(-1, 3)[:, 0], rtol=1e-5, atol=0)
    e = H.rel_l2(H.interior(g.download_state()), H.interior(d["final_U"]))
    print(f"compensated FP32 [{name}] rel L2:", np.array2string(e, precision=2))
    assert np.all(e <= TOL32_L2), e


def _oracle_run_p(p, U, steps):
    from oracle import oracle as O
    eos = O.Eos(H.EOS_SMALL)
    st = O.State(p, U)
    dts = st.step(eos, steps)
    return st.U, dts


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("case", ["periodic", "closed"])
def test_resistivity_vs_oracle(gpu_lib, kernel, case):
    """MHD_Residual with resistivity: B diffusion, ohmic heating, and (closed
    case, large eta) the resistive time-step limit; fused and per-routine
    steps against the oracle (bit-pinned to the reference with eta > 0)."""
    from oracle import oracle as O
    tab = initial.EosTable(H.EOS_SMALL)
    if case == "periodic":
        nx, ny, nz, eta = 20, 16, 12, 3e10
        U = initial.periodic_box(tab, nx, ny, nz, seed=23)
        kw = dict(periodic_x=1, grav=0.0)
        dx = 3.2e6
    else:
        nx, ny, nz, eta = 16, 12, 10, 2e12
        U = initial.stratified_box(tab, nx, ny, nz, seed=29)
        kw = dict(periodic_x=0, grav=2.74e4)
        dx = 1.6e6
    ref, dts_ref = _oracle_run_p(O.make_params(nx, ny, nz, dx, periodic_x=bool(kw["periodic_x"]), grav=kw["grav"],
                                               eta=eta), U, 5)
    p = gpumhd.default_params(nx, ny, nz, dx, stage_kernel=kernel, eta=eta, **kw)
    g = gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL)
    g.upload_state(U)
    dts = g.run_steps(5)
    assert np.allclose(dts, [d[0] for d in dts_ref], rtol=TOL64, atol=0)
    check(f"resistivity fused [{case}, kernel={kernel}]", g.download_state(), ref)
    g.close()
    g = gpumhd.MuramGPU(gpumhd.default_params(nx, ny, nz, dx, stage_kernel=kernel, eta=eta, **kw),
                        eos_path=H.EOS_SMALL)
    g.upload_state(U)
    g.exchange_grid(True)
    for _ in range(5):
        g.step_reference_order()
    check(f"resistivity per-routine [{case}, kernel={kernel}]", g.download_state(), ref)
    g.close()


def test_resistivity_fp32(gpu_lib):
    from oracle import oracle as O
    tab = initial.EosTable(H.EOS_SMALL)
    U = initial.periodic_box(tab, 32, 32, 32, seed=5)
    ref, _ = _oracle_run_p(O.make_params(32, 32, 32, 3.2e6, eta=3e10), U, 50)
    g = gpumhd.MuramGPU(gpumhd.default_params(32, 32, 32, 3.2e6, precision=32, eta=3e10), eos_path=H.EOS_SMALL)
    g.upload_state(U)
    g.run_steps(50)
    e = H.rel_l2(H.interior(g.download_state()), H.interior(ref))
    print("FP32 with resistivity vs FP64 oracle, rel L2:", np.array2string(e, precision=2))
    assert np.all(e <= TOL32_L2), e
    g.close()
