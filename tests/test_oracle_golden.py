"""The C restatement (oracle) against the reference's own outputs.

The golden fixtures were produced by the reference MURaM sources compiled
unchanged (tests/golden/make_golden.py); every comparison here is bit-exact.
When the reference harness binary is present (it is built only where the
reference sources exist), extra seeded cases are compared live.
"""
import ctypes as C

import numpy as np
import pytest

import helpers as H
from muram_main_gb300 import initial
from oracle import oracle as O
from oracle import refrun


@pytest.fixture(scope="module")
def eos():
    return O.Eos(H.EOS_SMALL)


@pytest.mark.parametrize("name", H.CASES)
def test_full_steps_bitexact(name, eos):
    d, hp = H.load_case(name)
    st = O.State(H.oracle_params(hp), d["input_U"])
    assert np.array_equal(st.U, d["init_U"])
    dts = st.step(eos, int(d["steps"]))
    ref = d["dts"].reshape(-1, 3)
    assert [x[0] for x in dts] == list(ref[:, 0])
    assert [x[1] for x in dts] == list(ref[:, 1])
    assert np.array_equal(st.U, d["final_U"])


def test_routines_bitexact_periodic(eos):
    d, hp = H.load_case("periodic")
    p = H.oracle_params(hp)
    L = O.lib()
    U = d["init_U"].copy()
    aux = np.zeros((5,) + U.shape[1:])
    L.mo_cons_to_prim(C.byref(p), eos.ptr, U, aux[0], aux[1], aux[2], aux[3], aux[4])
    assert np.array_equal(U, d["s1_c2p_U"])
    assert np.array_equal(aux, d["s1_c2p_aux"])
    L.mo_adjust_valf_max(C.byref(p), U, aux[0], np.zeros(5))
    assert [p.inv_va2max, p.v_lim, p.e_lim] == list(d["limits"][:3])
    R = np.zeros_like(U)
    dt = L.mo_mhd_residual(C.byref(p), U, aux[0], R)
    assert dt == d["s1_res_dt"][0]
    assert np.array_equal(R, d["s1_res_R"])
    cfl = C.c_double()
    assert L.mo_sync_timestep(C.byref(p), p.dt_rad, dt, C.byref(cfl)) == 0
    assert p.dt == d["dts"][0]
    U0 = d["init_U"].copy()
    L.mo_source_integrate_tcheck(C.byref(p), U, U0, R, 1)
    assert np.array_equal(U, d["s1_si_U"])
    assert not R.any()
    L.mo_boundaries(C.byref(p), U)
    assert np.array_equal(U, d["s1_bc_U"])
    # TVD of the traced step on its stage-4 state with the stale pressure
    U = d["s4_bc_U"].copy()
    L.mo_tvdlimit(C.byref(p), U, np.ascontiguousarray(d["s4_c2p_aux"][0]), p.dt)
    assert np.array_equal(U, d["tvd_U"])
    L.mo_tcheck(C.byref(p), U)
    assert np.array_equal(U, d["tck_U"])
    L.mo_boundaries(C.byref(p), U)
    assert np.array_equal(U, d["end_U"])


def test_divb_cleaning_bitexact(eos):
    """Clean_divB after each TVD pass (closed x, gravity, unequal dx/dy/dz):
    the state, the cleaning potential phi carried between steps, the last
    divergence and the adaptive iteration count of every step match the
    reference bit for bit; and the cleaning alone on the traced step's
    post-TVD state and incoming phi reproduces the reference's output."""
    d, hp = H.load_case("divb_cleaning")
    p = H.oracle_params(hp)
    st = O.State(p, d["input_U"])
    dts = st.step(eos, int(d["steps"]))
    assert [x[0] for x in dts] == list(d["dts"].reshape(-1, 3)[:, 0])
    assert np.array_equal(st.U, d["final_U"])
    assert np.array_equal(st.phi, d["final_phi"])
    assert np.array_equal(st.divB, d["final_divB"])
    assert [x[0] for x in st.divb_log] == list(d["divb_iters"])
    assert len(set(d["divb_iters"])) > 1  # the iteration count adapts
    # one call on the traced step's post-TVD state
    t = int(d["trace_step"])
    p2 = H.oracle_params(hp)
    p2.divB_next_iter = int(d["divb_iters"][t - 1])
    U = d["tvd_U"].copy()
    phi = d["divb_phi_in"].copy()
    divB = np.zeros_like(phi)
    O.lib().mo_clean_divB(C.byref(p2), U, phi, divB)
    assert p2.divB_last_iters == d["divb_iters"][t - 1]
    assert p2.divB_next_iter == d["divb_iters"][t]
    assert np.array_equal(U, d["divb_U"])
    O.lib().mo_tcheck(C.byref(p2), U)
    assert np.array_equal(U, d["tck_U"])


def test_open_bottom_bitexact(eos):
    """MURaM's physical x boundaries (open bottom through the inverse EOS,
    top open to outflows) after every stage and step: the reference's state,
    dt and the p_bc / s_bc its first call sets, bit for bit; and the stage-1
    boundary call alone on the traced step."""
    d, hp = H.load_case("open_bottom")
    p = H.oracle_params(hp)
    st = O.State(p, d["input_U"], eos)
    assert np.array_equal(st.U, d["init_U"])
    assert p.p_bc == float(d["p_bc"]) and p.s_bc == float(d["s_bc"])
    dts = st.step(eos, int(d["steps"]))
    assert [x[0] for x in dts] == list(d["dts"].reshape(-1, 3)[:, 0])
    assert np.array_equal(st.U, d["final_U"])
    U = d["s1_si_U"].copy()
    O.lib().mo_boundaries_eos(C.byref(p), eos.ptr, U)
    assert np.array_equal(U, d["s1_bc_U"])


def test_spitzer_bitexact(eos):
    """Hyperbolic Spitzer conduction (heat flux along B with its hyperdiffusion
    and relaxation to the saturation-limited Spitzer flux; physical x
    boundaries with a hot top): state and heat flux match the reference bit
    for bit, and the conduction changes the energy well above rounding."""
    d, hp = H.load_case("spitzer")
    st = O.State(H.oracle_params(hp), d["input_U"], eos)
    dts = st.step(eos, int(d["steps"]))
    assert [x[0] for x in dts] == list(d["dts"].reshape(-1, 3)[:, 0])
    assert np.array_equal(st.U, d["final_U"])
    assert np.array_equal(st.sflx, d["final_sflx"])
    assert np.abs(st.sflx).max() > 0
    hp0 = dict(hp, spitzer=0.0)
    st0 = O.State(H.oracle_params(hp0), d["input_U"], eos)
    st0.step(eos, int(d["steps"]))
    assert np.max(np.abs(st0.U[4] - st.U[4])) > 1e-8 * np.max(np.abs(st.U[4]))


def test_eos_interpolation_exact_at_nodes(eos):
    """Known answer: at a table node the bilinear lookup returns exp of the node value."""
    t = initial.EosTable(H.EOS_SMALL)
    i, j = 37, 61
    ee = float(np.exp(t.xeps[i]) - t.eps_off)
    rho = float(np.exp(t.xlr[j]))
    lnT = float(t.tables[1][i, j]) * t.del_eps * t.del_lr
    assert abs(t.T_interp(ee, rho) / np.exp(lnT) - 1.0) < 1e-6


def test_uniform_state_is_stationary(eos):
    """Known answer: a uniform state at rest has zero residual and an unchanged TVD pass."""
    p = O.make_params(8, 8, 8, 3.2e6)
    U = np.zeros((8, 12, 12, 12))
    U[0] = 3e-7
    U[4] = 3e-7 * 6e11
    U[5] = 1.0
    L = O.lib()
    aux = np.zeros((5,) + U.shape[1:])
    W = U.copy()
    L.mo_cons_to_prim(C.byref(p), eos.ptr, W, aux[0], aux[1], aux[2], aux[3], aux[4])
    L.mo_adjust_valf_max(C.byref(p), W, aux[0], np.zeros(5))
    R = np.zeros_like(U)
    L.mo_mhd_residual(C.byref(p), W, aux[0], R)
    assert np.all(H.interior(R) == 0.0)
    V = U.copy()
    p.dt = 1.0
    L.mo_tvdlimit(C.byref(p), V, aux[0], 1.0)
    assert np.allclose(V, U, rtol=1e-15, atol=0)


@pytest.mark.skipif(not refrun.available(), reason="reference harness not built here")
@pytest.mark.parametrize("seed", [101, 202])
def test_live_reference_random_boxes(seed, eos):
    """Extra seeded boxes, anisotropic and non-cubic, run by the reference and the oracle."""
    tab = initial.EosTable(H.EOS_SMALL)
    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(v) for v in rng.integers(5, 11, size=3))
    U = initial.periodic_box(tab, nx, ny, nz, dx=2.4e6, dy=3.2e6, dz=4.0e6, seed=seed,
                             v_rms=float(rng.uniform(0.5e5, 3e5)), b_rms_gauss=float(rng.uniform(20, 600)))
    hp = dict(nx=nx, ny=ny, nz=nz, dx=2.4e6, dy=3.2e6, dz=4.0e6, eos=H.EOS_SMALL)
    ref = refrun.run(U, hp, steps=4)
    st = O.State(H.oracle_params(hp), U)
    st.step(eos, 4)
    assert np.array_equal(st.U, ref["final_U"])


@pytest.mark.skipif(not refrun.available(), reason="reference harness not built here")
@pytest.mark.parametrize("case", ["periodic", "closed", "open_cold_top"])
def test_live_reference_spitzer(case, eos):
    """The conduction on a periodic box, with the mirror rule, and with the
    physical boundaries and no hot top (its top layers' heat flux zeroed)."""
    tab = initial.EosTable(H.EOS_SMALL)
    if case == "periodic":
        U = initial.periodic_box(tab, 12, 8, 10, seed=3)
        hp = dict(nx=12, ny=8, nz=10, dx=3.2e6, dy=2.4e6, dz=2.0e6)
    else:
        U = initial.stratified_box(tab, 12, 8, 6, dx=1.6e6, seed=17)
        hp = dict(nx=12, ny=8, nz=6, dx=1.6e6, periodic_x=0, grav=2.74e4)
        if case == "open_cold_top":
            hp.update(xbnd=1, bnd_top=0)
    hp.update(eos=H.EOS_SMALL, spitzer=0.5)
    ref = refrun.run(U, hp, steps=5)
    st = O.State(H.oracle_params(hp), U, eos)
    st.step(eos, 5)
    assert np.array_equal(st.U, ref["final_U"])
    assert np.array_equal(st.sflx, ref["final_sflx"])


@pytest.mark.skipif(not refrun.available(), reason="reference harness not built here")
@pytest.mark.parametrize("top,eps_top,bcrit,seed", [(0, 0.0, 1e10, 17), (1, 0.0, 1e10, 18), (1, 3e12, 40.0, 19)])
def test_live_reference_open_bottom(top, eps_top, bcrit, seed, eos):
    """The physical x boundaries against the reference run live: closed and
    half-open top, a fixed top internal energy, and a B_crit low enough that
    the footpoint factor changes the bottom momenta."""
    tab = initial.EosTable(H.EOS_SMALL)
    U = initial.stratified_box(tab, 12, 8, 6, dx=1.6e6, seed=seed)
    hp = dict(nx=12, ny=8, nz=6, dx=1.6e6, periodic_x=0, grav=2.74e4, eos=H.EOS_SMALL, xbnd=1, bnd_top=top,
              bnd_eps_top=eps_top, bnd_bcrit=bcrit)
    ref = refrun.run(U, hp, steps=4)
    st = O.State(H.oracle_params(hp), U, eos)
    st.step(eos, 4)
    assert np.array_equal(st.U, ref["final_U"])


@pytest.mark.skipif(not refrun.available(), reason="reference harness not built here")
@pytest.mark.parametrize("periodic_x,itmax,err", [(1, 5, 0.2), (0, 1, 0.5), (1, 3, 0.01)])
def test_live_reference_divb_cleaning(periodic_x, itmax, err, eos):
    """Clean_divB on periodic and closed boxes, with iteration caps below and
    above the starting count of 3, against the reference run live."""
    import re
    tab = initial.EosTable(H.EOS_SMALL)
    if periodic_x:
        U = initial.periodic_box(tab, 12, 8, 10, seed=3)
        hp = dict(nx=12, ny=8, nz=10, dx=3.2e6, dy=2.4e6, dz=2.0e6)
    else:
        U = initial.stratified_box(tab, 10, 8, 6, seed=17)
        hp = dict(nx=10, ny=8, nz=6, dx=1.6e6, periodic_x=0, grav=2.74e4)
    hp.update(eos=H.EOS_SMALL, divB_switch=1, divB_itmax=itmax, divB_err=err, verbose=1)
    ref = refrun.run(U, hp, steps=5)
    st = O.State(H.oracle_params(hp), U)
    st.step(eos, 5)
    assert np.array_equal(st.U, ref["final_U"])
    assert np.array_equal(st.phi, ref["final_phi"])
    iters = [int(m) for m in re.findall(r"divB_max \[(\d+)\]", ref["stdout"])]
    assert [x[0] for x in st.divb_log] == iters


@pytest.mark.skipif(not refrun.available(), reason="reference harness not built here")
@pytest.mark.parametrize("eta", [3e10, 2e12])
def test_live_reference_resistivity(eta, eos):
    """MHD_Residual with resistivity (Physics.params[i_param_eta] > 0): ohmic
    heating from the running curl B, the B diffusion term, and the resistive
    time-step limit (the larger eta sets dt) -- reference and oracle agree bit
    for bit over several steps, closed x with gravity included."""
    tab = initial.EosTable(H.EOS_SMALL)
    U = initial.stratified_box(tab, 10, 8, 6, seed=17)
    hp = dict(nx=10, ny=8, nz=6, dx=1.6e6, periodic_x=0, grav=2.74e4, eta=eta, eos=H.EOS_SMALL)
    ref = refrun.run(U, hp, steps=3)
    st = O.State(H.oracle_params(hp), U)
    dts = st.step(eos, 3)
    assert np.array_equal(st.U, ref["final_U"])
    assert np.array_equal(np.array([d[0] for d in dts]), ref["dts"].reshape(-1, 3)[:, 0])
    if eta > 1e12:  # dt set by the resistive limit dt_diff_fac / eta
        dxmin = 1.6e6
        assert ref["dts"].reshape(-1, 3)[0, 0] <= 0.8 * (dxmin * dxmin / 6.0) / eta * 1.0000001


def test_va_adjust_bitexact(eos):
    """Adjust_Valf_Max with adaptive limits at the reference's 3-D test settings
    (va_adjust 1, max_fill 100): the first call sets v_lim and e_lim from the
    maxima, later calls scale them by 1.04, 1.01 or 0.99 from the near-limit
    counts and clamp them, va_max follows the maxima; the limits of every
    step, dt and the state match the reference bit for bit."""
    d, hp = H.load_case("va_adjust")
    st = O.State(H.oracle_params(hp), d["input_U"])
    dts = st.step(eos, int(d["steps"]))
    assert [x[0] for x in dts] == list(d["dts"].reshape(-1, 3)[:, 0])
    assert [list(x) for x in st.limits_log] == d["limits"].reshape(-1, 3).tolist()
    assert np.array_equal(st.U, d["final_U"])
    # the fixture exercises the adaptation: e_lim raised by 4 % and by 1 %, v_lim lowered by 1 %
    lim = d["limits"].reshape(-1, 3)
    ratios_e = set(np.round(lim[1:, 2] / lim[:-1, 2], 6))
    assert {1.04, 1.01} <= ratios_e
    assert np.allclose(lim[2:, 1] / lim[1:-1, 1], 0.99, rtol=1e-12)


@pytest.mark.skipif(not refrun.available(), reason="reference harness not built here")
@pytest.mark.parametrize("max_fill,va_max,v_rms,seed", [(2.0, 3.0e5, 3.0e5, 41), (30.0, 2.0e6, 1.0e5, 42),
                                                        (1000.0, 1.0e5, 2.0e5, 43)])
def test_live_reference_va_adjust(max_fill, va_max, v_rms, seed, eos):
    """The adaptive limits against the reference run live, with near-limit
    counts above 4 max_fill, between, and below max_fill / 2, and a va_max
    floor (va_max / 3, (va_max / 2)^2) that binds or not."""
    tab = initial.EosTable(H.EOS_SMALL)
    U = initial.periodic_box(tab, 12, 10, 8, seed=seed, v_rms=v_rms, b_rms_gauss=600.0)
    hp = dict(nx=12, ny=10, nz=8, dx=3.2e6, eos=H.EOS_SMALL, va_adjust=1.0, max_fill=max_fill, va_max=va_max)
    ref = refrun.run(U, hp, steps=6)
    st = O.State(H.oracle_params(hp), U)
    dts = st.step(eos, 6)
    assert np.array_equal(np.array([x[0] for x in dts]), ref["dts"].reshape(-1, 3)[:, 0])
    assert np.array_equal(np.array(st.limits_log).reshape(-1), ref["limits"])
    assert np.array_equal(st.U, ref["final_U"])


DIAG_NAMES = ["tvar1", "tvar2", "tvar3", "tvar4", "tvar5", "tvar6", "tvar7", "tvar8", "Qres", "Qvis"]


@pytest.mark.parametrize("name", ["diagnostics", "diagnostics_spitzer", "diagnostics_two_half"])
def test_diagnostics_bitexact(name, eos):
    """An output step's diagnostics (Run.need_diagnostics from stage 4 through
    TVDlimit and TCheck): the energy-flux divergence, its conduction share and
    the Lorentz work of MHD_Residual, Source_Integrate's radiation factor,
    gravity work, Boris energy and TCheck energy change, and TVDlimit's
    energy change, Boris part, resistive and viscous heating and floor
    change -- bit for bit against the reference, with the state."""
    d, hp = H.load_case(name)
    st = O.State(H.oracle_params(hp), d["input_U"], eos)
    ds = int(hp["diag_step"])
    st.step(eos, ds, diagnostics_at=ds)
    assert np.array_equal(H.interior(st.U), H.interior(d["diag_U"]))
    for q in range(10):
        assert np.array_equal(st.diag[q], d["diag"][q]), DIAG_NAMES[q]
    st.step(eos, int(d["steps"]) - ds)
    assert np.array_equal(st.U, d["final_U"])
    assert not st.p.need_diagnostics  # off again after the output step
