"""Ensembles of boxes in one graph launch, and the launch-shape autotuner.

Both change only how work is launched, so the results must equal those of
the boxes run one by one (bit for bit: the per-cell arithmetic is the same).
"""
import numpy as np
import pytest

import helpers as H
from muram_main_gb300 import gpumhd, initial

pytestmark = pytest.mark.gpu


def _box(nx, ny, nz, precision, seed, closed=False):
    tab = initial.EosTable(H.EOS_SMALL)
    if closed:
        U = initial.stratified_box(tab, nx, ny, nz, seed=seed)
        p = gpumhd.default_params(nx, ny, nz, 1.6e6, precision=precision, periodic_x=0, grav=2.74e4)
    else:
        U = initial.periodic_box(tab, nx, ny, nz, seed=seed)
        p = gpumhd.default_params(nx, ny, nz, 3.2e6, precision=precision)
    g = gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL)
    g.upload_state(U)
    return g


SHAPES = [(16, 12, 8, 64, 1, False), (24, 20, 12, 64, 2, True), (32, 16, 20, 32, 3, False), (18, 14, 10, 32, 4, True)]


def test_ensemble_equals_boxes_run_one_by_one(gpu_lib):
    steps = 6
    alone = []
    for nx, ny, nz, prec, seed, closed in SHAPES:
        g = _box(nx, ny, nz, prec, seed, closed)
        g.run_steps(steps)
        alone.append((g.download_state(), g.step_info()))
        g.close()
    boxes = [_box(*s) for s in SHAPES]
    ens = gpumhd.MuramEnsemble(boxes)
    ens.run_steps(steps // 2)
    ens.run_steps(steps - steps // 2)  # a second launch continues the loop
    # 9 kernels per box and step always run; the second TVD half pass (3 more)
    # sits in a conditional node that these steps do not take
    assert ens.launch_count == (9 * len(boxes) + 1) * steps + 2
    for (ref, info), g in zip(alone, boxes):
        got = g.download_state()
        assert np.array_equal(got, ref), np.max(np.abs(got - ref))
        assert g.step_info()[2] == info[2]  # same simulated time
    ens.close()
    for g in boxes:
        g.close()


@pytest.mark.parametrize("unroll,largest_first", [(3, False), (4, True)])
def test_ensemble_schedule_keeps_results(gpu_lib, unroll, largest_first):
    """Several steps of each box per loop iteration, and the branches in order
    of decreasing size: the same steps of the same boxes, so the same bits;
    10 steps = whole iterations plus a remainder run one step at a time."""
    steps = 10
    alone = []
    for nx, ny, nz, prec, seed, closed in SHAPES:
        g = _box(nx, ny, nz, prec, seed, closed)
        g.run_steps(steps)
        alone.append(g.download_state())
        g.close()
    boxes = [_box(*s) for s in SHAPES]
    ens = gpumhd.MuramEnsemble(boxes)
    ens.set_schedule(unroll, largest_first)
    ens.run_steps(steps)
    nk, n1 = steps // unroll, steps % unroll
    assert ens.launch_count == 9 * len(boxes) * steps + nk + n1 + (nk > 0) + (n1 > 0)
    for ref, g in zip(alone, boxes):
        assert np.array_equal(g.download_state(), ref)
    ens.close()
    for g in boxes:
        g.close()


def test_box_calls_after_an_ensemble_launch(gpu_lib):
    """Per-box calls queued after an ensemble launch see its result."""
    g1 = _box(16, 12, 8, 64, 11)
    g2 = _box(16, 12, 8, 64, 11)
    ens = gpumhd.MuramEnsemble([g1])
    ens.enqueue_steps(3)
    g1.run_steps(2)           # ordered after the ensemble's steps
    g2.run_steps(5)
    assert np.array_equal(g1.download_state(), g2.download_state())
    ens.close()
    g1.close()
    g2.close()


@pytest.mark.parametrize("precision", [64, 32])
def test_autotune_keeps_state_and_results(gpu_lib, precision):
    a = _box(40, 24, 20, precision, 21, closed=True)
    b = _box(40, 24, 20, precision, 21, closed=True)
    U0 = a.download_state()
    ms = a.autotune(trial_steps=2)
    assert ms > 0
    t = a.tuning()
    assert t["stage_kernel"] in (0, 1) and t["stage_zchunk"] >= 0 and t["tvd_chunk"] in (16, 32, 64)
    assert np.array_equal(a.download_state(), U0)
    assert a.step_info()[2] == b.step_info()[2]
    a.run_steps(5)
    b.run_steps(5)
    if precision == 64:
        assert np.array_equal(a.download_state(), b.download_state())
    else:
        # FP32: the two stage kernels contract different products into FMAs
        assert np.all(H.rel_linf(a.download_state(), b.download_state()) <= 1e-5)
    a.close()
    b.close()


def test_explicit_tuning_gives_same_results(gpu_lib):
    ref = _box(24, 20, 36, 64, 5)
    ref.run_steps(4)
    for zc, td in [(36, 16), (5, 64), (9, 32)]:
        g = _box(24, 20, 36, 64, 5)
        g.set_tuning(zc, td)
        g.run_steps(4)
        assert np.array_equal(g.download_state(), ref.download_state()), (zc, td)
        g.close()
    ref.close()


@pytest.mark.parametrize("closed", [False, True])
def test_fp32_stage_layouts_agree(gpu_lib, closed):
    """FP32 stage kernel: on z chunks of 16 planes or more, stages 1 and 4 and
    the residual take the three-slot, double-buffered layout (one barrier per
    plane); on shorter chunks every stage takes the four-slot layout.  Same
    per-cell arithmetic, so the states agree to the FMA contractions of the
    two compiled instances; so do the per-routine residual and its dt."""
    runs = []
    for zc in (48, 8):
        g = _box(64, 32, 48, 32, 7, closed=closed)
        g.set_tuning(zc, 0)
        g.run_steps(6)
        U = g.download_state()
        g.ConsToPrim()
        g.Adjust_Valf_Max()
        dt = g.MHD_Residual()
        runs.append((U, dt, g.download_state(gpumhd.FIELD_RES)))
        g.close()
    (ua, dta, ra), (ub, dtb, rb) = runs
    assert np.all(H.rel_linf(ua, ub) <= 1e-6), H.rel_linf(ua, ub)
    assert abs(dta / dtb - 1) <= 1e-6
    assert np.all(H.rel_linf(ra, rb) <= 1e-5), H.rel_linf(ra, rb)


def test_tile_from_commutes_with_the_step(gpu_lib):
    """A periodic box tiled 2 x 3 x 2 and advanced equals the advanced small
    box tiled the same way (the periodic step treats every copy alike)."""
    small = _box(16, 12, 8, 64, 31)
    big = gpumhd.MuramGPU(gpumhd.default_params(32, 36, 16, 3.2e6), eos_path=H.EOS_SMALL)
    big.tile_from(small)
    U0 = small.download_state()[:, 2:-2, 2:-2, 2:-2]
    assert np.array_equal(big.download_state()[:, 2:-2, 2:-2, 2:-2], np.tile(U0, (1, 2, 3, 2)))
    small.run_steps(4)
    big.run_steps(4)
    U1 = small.download_state()[:, 2:-2, 2:-2, 2:-2]
    assert np.array_equal(big.download_state()[:, 2:-2, 2:-2, 2:-2], np.tile(U1, (1, 2, 3, 2)))
    small.close()
    big.close()


def _box_kw(nx, ny, nz, precision, seed, **kw):
    tab = initial.EosTable(H.EOS_SMALL)
    p = gpumhd.default_params(nx, ny, nz, 3.2e6, precision=precision, **kw)
    g = gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL)
    g.upload_state(initial.periodic_box(tab, nx, ny, nz, seed=seed))
    return g


CARRIED = {"divb": dict(divB_switch=1, divB_itmax=4, divB_err=0.2), "spitzer": dict(spitzer=0.5)}


@pytest.mark.parametrize("kind", sorted(CARRIED))
def test_autotune_restores_carried_fields(gpu_lib, kind):
    """The trial steps of the autotuner also advance what a step carries
    besides the state (the cleaning potential phi, the heat flux); both are
    given back, so a tuned box continues exactly as an untuned one (FP64:
    the shapes do not change the bits)."""
    a = _box_kw(32, 16, 24, 64, 71, **CARRIED[kind])
    b = _box_kw(32, 16, 24, 64, 71, **CARRIED[kind])
    a.run_steps(3)
    b.run_steps(3)
    a.autotune(trial_steps=2)
    a.run_steps(4)
    b.run_steps(4)
    assert np.array_equal(a.download_state(), b.download_state())
    field = gpumhd.FIELD_PHI if kind == "divb" else gpumhd.FIELD_SFLX
    assert np.array_equal(a.download_field(field), b.download_field(field))
    assert a.step_info()[2] == b.step_info()[2]
    a.close()
    b.close()


def test_ensemble_autotune_keeps_results(gpu_lib):
    """gpumhd_ensemble_autotune times launch shapes on the boxes' current
    states and restores them: FP64 boxes (plain, with cleaning, with
    conduction) continue bit for bit as when run alone; the FP32 box to the
    FMA contractions of the two stage-kernel layouts its new z chunk may
    select."""
    specs = [(16, 12, 8, 64, 81, {}), (24, 16, 12, 64, 82, CARRIED["divb"]), (20, 12, 16, 64, 83, CARRIED["spitzer"]),
             (32, 16, 24, 32, 84, {})]
    alone = []
    for nx, ny, nz, prec, seed, kw in specs:
        g = _box_kw(nx, ny, nz, prec, seed, **kw)
        g.run_steps(6)
        alone.append(g.download_state())
        g.close()
    boxes = [_box_kw(nx, ny, nz, prec, seed, **kw) for nx, ny, nz, prec, seed, kw in specs]
    ens = gpumhd.MuramEnsemble(boxes)
    ens.run_steps(2)
    ms = ens.autotune(trial_steps=2)
    assert ms > 0
    ens.run_steps(4)
    for (nx, ny, nz, prec, seed, kw), ref, g in zip(specs, alone, boxes):
        got = g.download_state()
        if prec == 64:
            assert np.array_equal(got, ref), (nx, ny, nz, kw)
        else:
            assert np.all(H.rel_linf(got, ref) <= 1e-6), H.rel_linf(got, ref)
    ens.close()
    for g in boxes:
        g.close()
