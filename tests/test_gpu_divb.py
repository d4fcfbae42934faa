"""divB cleaning (Clean_divB, src/clean_divB.C:35-369) on the GPU.

Against the reference's own fixture (closed x, gravity, unequal dx/dy/dz,
cleaning after every TVD pass) and against the oracle, whose restatement of
Clean_divB is bit-pinned to the reference.  Checked per step: the state, the
cleaning potential phi carried between steps, the last divergence, and the
adaptive iteration count.  FP64 bar: relative L-infinity 1e-12 per field (the
EOS's exp/log differ from the host's by a few ulp); FP32: relative L2 1e-5.
"""
import ctypes as C

import numpy as np
import pytest

import helpers as H
from muram_main_gb300 import gpumhd, initial

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
KERNELS = [0, 1]


def ctx_for(hp, precision=64, stage_kernel=0):
    p = H.gpu_params(hp, precision)
    p.stage_kernel = stage_kernel
    return gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL)


def check(name, got, ref, tol=TOL64):
    e = H.rel_linf(got, ref)
    print(f"{name}: rel Linf per field {np.array2string(e, precision=2)}")
    assert np.all(e <= tol), (name, e)


def check_scalar(name, got, ref, tol=TOL64):
    e = H.rel_linf(H.interior(got)[None], H.interior(ref)[None])[0]
    print(f"{name}: rel Linf {e:.2e}")
    assert e <= tol, (name, e)


@pytest.mark.parametrize("capture", [0, 1])
@pytest.mark.parametrize("kernel", KERNELS)
def test_fused_steps_vs_reference_fixture(gpu_lib, kernel, capture):
    d, hp = H.load_case("divb_cleaning")
    g = ctx_for(hp, stage_kernel=kernel)
    g.upload_state(d["input_U"])
    dts, iters = [], []
    for _ in range(int(d["steps"])):
        dts.append(g.run_steps(1, capture=bool(capture))[0])
        iters.append(g.divb_info()[0])
    assert iters == list(d["divb_iters"])
    assert np.allclose(dts, d["dts"].reshape(-1, 3)[:, 0], rtol=TOL64, atol=0)
    check(f"fused steps with cleaning [kernel={kernel}, graph={capture}]", g.download_state(), d["final_U"])
    check_scalar("phi", g.download_field(gpumhd.FIELD_PHI), d["final_phi"])
    check_scalar("divB", g.download_field(gpumhd.FIELD_DIVB), d["final_divB"])
    g.close()


def test_reference_order_steps_vs_reference_fixture(gpu_lib):
    d, hp = H.load_case("divb_cleaning")
    g = ctx_for(hp)
    g.upload_state(d["input_U"])
    g.exchange_grid(True)
    iters = []
    for _ in range(int(d["steps"])):
        g.step_reference_order()
        iters.append(g.divb_info()[0])
    assert iters == list(d["divb_iters"])
    check("per-routine steps with cleaning", g.download_state(), d["final_U"])
    check_scalar("phi", g.download_field(gpumhd.FIELD_PHI), d["final_phi"])
    g.close()


def test_clean_divB_call_vs_oracle(gpu_lib):
    """One Clean_divB call on the fixture's post-TVD state and incoming phi:
    state (ghosts included), phi, divB and the reported errors."""
    from oracle import oracle as O
    d, hp = H.load_case("divb_cleaning")
    g = ctx_for(hp)
    g.upload_state(d["tvd_U"])
    g.upload_field(gpumhd.FIELD_PHI, d["divb_phi_in"])
    g.Clean_divB()
    p = H.oracle_params(hp)
    assert p.divB_next_iter == 3 and g.divb_info()[0] == 3
    U = d["tvd_U"].copy()
    phi = d["divb_phi_in"].copy()
    divB = np.zeros_like(phi)
    O.lib().mo_clean_divB(C.byref(p), U, phi, divB)
    check("Clean_divB state", g.download_state(), U)
    check_scalar("Clean_divB phi", g.download_field(gpumhd.FIELD_PHI), phi)
    check_scalar("Clean_divB divB", g.download_field(gpumhd.FIELD_DIVB), divB)
    last, nxt, e0, e1 = g.divb_info()
    assert (last, nxt) == (p.divB_last_iters, p.divB_next_iter)
    assert abs(e0 - p.divB_err0) <= TOL64 * p.divB_err0 and abs(e1 - p.divB_err1) <= TOL64 * p.divB_err1
    g.close()


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("case", ["periodic", "two_half", "capped"])
def test_fused_vs_oracle(gpu_lib, kernel, case):
    """Periodic boxes (the wrapped neighbours of B and phi), a box that takes
    two half TVD passes, and an iteration cap below the starting count."""
    from oracle import oracle as O
    tab = initial.EosTable(H.EOS_SMALL)
    if case == "two_half":
        nx, ny, nz = 16, 12, 10
        U = initial.periodic_box(tab, nx, ny, nz, seed=43, v_rms=3.0e5, b_rms_gauss=400.0)
        hp = dict(nx=nx, ny=ny, nz=nz, dx=3.2e6, CFL=1.2, CFL_tvd=1.0)
    else:
        nx, ny, nz = 24, 16, 12
        U = initial.periodic_box(tab, nx, ny, nz, seed=41)
        hp = dict(nx=nx, ny=ny, nz=nz, dx=3.2e6, dy=2.4e6, dz=2.0e6)
    hp.update(divB_switch=1, divB_itmax=1 if case == "capped" else 5, divB_err=0.2)
    st = O.State(H.oracle_params(hp), U)
    eos = O.Eos(H.EOS_SMALL)
    g = ctx_for(hp, stage_kernel=kernel)
    g.upload_state(U)
    for s in range(6):
        st.step(eos, 1)
        g.run_steps(1)
        assert g.divb_info()[0] == st.divb_log[-1][0], s
    if case == "two_half":
        assert g.step_info()[3] == 1
    check(f"cleaning vs oracle [{case}, kernel={kernel}]", g.download_state(), st.U)
    check_scalar("phi", g.download_field(gpumhd.FIELD_PHI), st.phi)
    g.close()


def test_fp32_cleaning_vs_fp64_oracle(gpu_lib):
    """FP32 with cleaning against the FP64 oracle after 100 steps.

    Clean_divB's iteration count adapts from the ratio of max|divB| after and
    before the iterations against divB_err.  Where that ratio lands close to
    divB_err, the FP32 divergence (a small difference of float fluxes) can
    fall on the other side of it: FP32 then takes one iteration more or fewer
    on that step and departs from FP64 by far more than rounding (an earlier
    build measured 5e-5 relative L2 in B on this machine).  Both runs are checked:
    one on FP64's iteration sequence (set before each step through
    gpumhd_set_divb_iters) and the free-running one; the steps whose counts
    differ are printed."""
    from oracle import oracle as O
    tab = initial.EosTable(H.EOS_SMALL)
    U = initial.periodic_box(tab, 32, 32, 32, seed=5)
    hp = dict(nx=32, ny=32, nz=32, dx=3.2e6, divB_switch=1, divB_itmax=5, divB_err=0.2)
    st = O.State(H.oracle_params(hp), U)
    st.step(O.Eos(H.EOS_SMALL), 100)
    iters64 = [x[0] for x in st.divb_log]
    forced = ctx_for(hp, precision=32)
    free = ctx_for(hp, precision=32)
    forced.upload_state(U)
    free.upload_state(U)
    iters32 = []
    for s in range(100):
        forced.set_divb_iters(iters64[s])
        forced.run_steps(1)
        assert forced.divb_info()[0] == iters64[s]
        free.run_steps(1)
        iters32.append(free.divb_info()[0])
    e_free = H.rel_l2(H.interior(free.download_state()), H.interior(st.U))
    e = H.rel_l2(H.interior(forced.download_state()), H.interior(st.U))
    flips = [s for s in range(100) if iters32[s] != iters64[s]]
    print("FP32 with cleaning vs FP64 oracle after 100 steps, rel L2 -- on FP64's iteration counts:",
          np.array2string(e, precision=2), "free-running:", np.array2string(e_free, precision=2),
          "steps whose count differs:", flips[:10])
    assert np.all(e <= 1e-5), e
    assert np.all(e_free <= 1e-5), (e_free, flips)
    forced.close()
    free.close()


def test_cleaning_reduces_divergence_and_is_timed(gpu_lib):
    """The cleaning lowers max|divB| within each call, and the per-phase
    profile reports its time."""
    tab = initial.EosTable(H.EOS_SMALL)
    U = initial.periodic_box(tab, 32, 24, 16, seed=8)
    g = ctx_for(dict(nx=32, ny=24, nz=16, dx=3.2e6, divB_switch=1, divB_itmax=5, divB_err=0.2))
    g.upload_state(U)
    g.run_steps(3)
    last, nxt, e0, e1 = g.divb_info()
    assert 1 <= last <= 5 and 1 <= nxt <= 5 and e1 < e0
    ph = g.profile_steps(2)
    assert ph["divb_clean"] > 0
    g.close()


def test_ensemble_with_cleaning(gpu_lib):
    """Boxes with and without cleaning in one graph launch equal the boxes
    run one by one, launch counts included."""
    tab = initial.EosTable(H.EOS_SMALL)
    shapes = [(16, 12, 8, 1), (20, 16, 12, 0), (24, 12, 8, 1)]

    def box(nx, ny, nz, on, seed):
        g = ctx_for(dict(nx=nx, ny=ny, nz=nz, dx=3.2e6, divB_switch=on, divB_itmax=4, divB_err=0.2))
        g.upload_state(initial.periodic_box(tab, nx, ny, nz, seed=seed))
        return g

    alone = []
    for q, (nx, ny, nz, on) in enumerate(shapes):
        g = box(nx, ny, nz, on, 60 + q)
        g.run_steps(4)
        alone.append(g.download_state())
        g.close()
    boxes = [box(nx, ny, nz, on, 60 + q) for q, (nx, ny, nz, on) in enumerate(shapes)]
    ens = gpumhd.MuramEnsemble(boxes)
    ens.run_steps(4)
    per_step = 1 + sum(9 + (3 + 2 * 4 if on else 0) for *_, on in shapes)  # second TVD pass: conditional
    assert ens.launch_count == per_step * 4 + 1
    for ref, g in zip(alone, boxes):
        assert np.array_equal(g.download_state(), ref)
    ens.close()
    for g in boxes:
        g.close()
