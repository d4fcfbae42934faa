"""The TMA stage kernel's bounded waits: an expired wait becomes a status.

Every mbarrier wait of k_stage_tm for a plane's TMA copy is bounded; when
one runs out the block records ERR_WAIT_TIMEOUT in the step-control block,
waits for the copies it did issue, frees its tensor memory and returns, and
the host reads the flag as GPUMHD_E_CUDA.  The test hook withholds the copy
of each block's last plane (a copy nothing ever issues) and shortens the wait
limit to 1e5 clock cycles, so the wait runs out without a fault or a hang.
Afterwards the same context, with the hook off, reproduces the reference's
fixture: it stays usable.
"""
import numpy as np
import pytest

import helpers as H
from muram_main_gb300 import gpumhd

pytestmark = pytest.mark.gpu

SHORT = 100000  # clock cycles, ~50 us


def _ctx(hp, precision):
    p = H.gpu_params(hp, precision)
    p.stage_kernel = 0
    g = gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL)
    assert g.tuning()["stage_kernel"] == 0, "the box must take the TMA stage kernel"
    return g


def _recover(g, d, tol_check):
    g.test_tma_wait(0, False)
    g.upload_state(d["input_U"])
    dts = g.run_steps(int(d["steps"]))
    assert np.allclose(dts, d["dts"].reshape(-1, 3)[:, 0], rtol=1e-6, atol=0)
    tol_check(g.download_state(), d["final_U"])


def _fp64(got, ref):
    assert np.all(H.rel_linf(got, ref) <= 1e-12)


def _fp32(got, ref):
    assert np.all(H.rel_l2(H.interior(got), H.interior(ref)) <= 1e-5)


@pytest.mark.parametrize("precision,capture", [(64, False), (32, True)])
def test_fused_step_wait_timeout(gpu_lib, precision, capture):
    d, hp = H.load_case("periodic")
    g = _ctx(hp, precision)
    g.upload_state(d["input_U"])
    g.test_tma_wait(SHORT, True)
    with pytest.raises(gpumhd.GpumhdError) as e:
        g.run_steps(1, capture=capture)
    assert e.value.code == gpumhd.E_CUDA and "timed out" in str(e.value)
    _recover(g, d, _fp64 if precision == 64 else _fp32)


def test_mhd_residual_wait_timeout(gpu_lib):
    d, hp = H.load_case("periodic")
    g = _ctx(hp, 64)
    g.upload_state(d["s1_c2p_U"])
    g.upload_field(gpumhd.FIELD_PRES, d["s1_c2p_aux"][0])
    g.upload_state(np.zeros_like(d["s1_c2p_U"]), gpumhd.FIELD_RES)
    g.Adjust_Valf_Max()
    g.test_tma_wait(SHORT, True)
    with pytest.raises(gpumhd.GpumhdError) as e:
        g.MHD_Residual()
    assert e.value.code == gpumhd.E_CUDA and "timed out" in str(e.value)
    g.test_tma_wait(0, False)
    g.upload_state(np.zeros_like(d["s1_c2p_U"]), gpumhd.FIELD_RES)
    dt = g.MHD_Residual()
    assert abs(dt / d["s1_res_dt"][0] - 1) <= 1e-12
    assert np.all(H.rel_linf(g.download_state(gpumhd.FIELD_RES), d["s1_res_R"]) <= 1e-12)
