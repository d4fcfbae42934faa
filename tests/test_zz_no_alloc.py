"""The allocation-free CFL time step against the per-routine MHD_Residual.

gpumhd_cfl_dt_noalloc is for callers that own their device arrays and may not
allocate device memory (a MURaM build whose fields belong to the OpenACC
runtime, or a loop that cannot pay for cudaMalloc's synchronisation).  This
test gives it device copies of a ConsToPrim'd state and checks that its dt_mhd
equals the one MHD_Residual returns for the same state, on consecutive calls
with different boxes (the calls share one scratch array).  The file is
collected last so that a run stopping at the first failure has run every
other test first.
"""
import ctypes as C

import numpy as np
import pytest

import helpers as H
from muram_main_gb300 import gpumhd, initial

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _reference_dt(tab, shape, seed, dxs):
    nx, ny, nz = shape
    U = initial.periodic_box(tab, nx, ny, nz, dx=dxs[0], dy=dxs[1], dz=dxs[2], seed=seed)
    g = gpumhd.MuramGPU(gpumhd.default_params(nx, ny, nz, dxs[0], dy=dxs[1], dz=dxs[2]), eos_path=H.EOS_SMALL)
    g.upload_state(U)
    g.ConsToPrim()
    g.Adjust_Valf_Max()
    g.upload_state(np.zeros_like(U), gpumhd.FIELD_RES)
    dt_ref = g.MHD_Residual()
    prim = g.download_state()
    pres = g.download_field(gpumhd.FIELD_PRES)
    inv_va2max = g.limits()[0]
    g.close()
    return dt_ref, prim, pres, inv_va2max


def test_cfl_dt_noalloc_matches_mhd_residual(gpu_lib):
    import torch
    L = gpumhd.load()
    tab = initial.EosTable(H.EOS_SMALL)
    cases = [((20, 12, 10), 21, (3.2e6, 3.2e6, 3.2e6)),
             ((16, 24, 8), 22, (2.4e6, 3.2e6, 4.0e6)),
             ((20, 12, 10), 23, (3.2e6, 3.2e6, 3.2e6))]
    for shape, seed, dxs in cases:  # consecutive calls sharing the scratch array
        dt_ref, prim, pres, inv_va2max = _reference_dt(tab, shape, seed, dxs)
        d_U = torch.from_numpy(prim.reshape(-1).copy()).cuda()
        d_P = torch.from_numpy(pres.reshape(-1).copy()).cuda()
        d_dt = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        dx = (C.c_double * 3)(*dxs)
        torch.cuda.synchronize()
        rc = L.gpumhd_cfl_dt_noalloc(d_U.data_ptr(), d_P.data_ptr(), shape[0], shape[1], shape[2], dx, inv_va2max,
                                     None, d_dt.data_ptr())
        assert rc == gpumhd.OK
        torch.cuda.synchronize()
        dt = float(d_dt.item())
        print(f"noalloc dt {dt!r} vs MHD_Residual {dt_ref!r} for {shape}")
        assert abs(dt / dt_ref - 1.0) <= TOL


def test_cfl_dt_noalloc_rejects_oversized_box(gpu_lib):
    """More z planes than the scratch array holds: refused before any GPU work."""
    import torch
    L = gpumhd.load()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    dx = (C.c_double * 3)(3.2e6, 3.2e6, 3.2e6)
    rc = L.gpumhd_cfl_dt_noalloc(buf.data_ptr(), buf.data_ptr(), 8, 8, 4093, dx, 1e-14, None, out.data_ptr())
    assert rc == gpumhd.E_INVALID
    torch.cuda.synchronize()
    assert float(out.item()) == -1.0


def _mhd_residual_dt(prim, pres, shape, dxs):
    """dt_mhd of the per-routine MHD_Residual for a given primitive state."""
    nx, ny, nz = shape
    g = gpumhd.MuramGPU(gpumhd.default_params(nx, ny, nz, dxs[0], dy=dxs[1], dz=dxs[2]), eos_path=H.EOS_SMALL)
    g.upload_state(prim)
    g.upload_field(gpumhd.FIELD_PRES, pres)
    g.upload_state(np.zeros_like(prim), gpumhd.FIELD_RES)
    g.Adjust_Valf_Max()
    dt = g.MHD_Residual()
    g.close()
    return dt


def _noalloc_dt(L, prim, pres, shape, dxs, inv_va2max):
    import torch
    d_U = torch.from_numpy(prim.reshape(-1).copy()).cuda()
    d_P = torch.from_numpy(pres.reshape(-1).copy()).cuda()
    d_dt = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    dx = (C.c_double * 3)(*dxs)
    torch.cuda.synchronize()
    rc = L.gpumhd_cfl_dt_noalloc(d_U.data_ptr(), d_P.data_ptr(), shape[0], shape[1], shape[2], dx, inv_va2max,
                                 None, d_dt.data_ptr())
    assert rc == gpumhd.OK
    torch.cuda.synchronize()
    return float(d_dt.item())


def test_cfl_dt_noalloc_face_and_corner_ghosts(gpu_lib):
    """Ghost cells that differ from the interior: a fast face ghost (one index
    in a ghost layer) lowers dt in both entry points, a fast edge ghost (two
    indices in ghost layers) changes neither."""
    L = gpumhd.load()
    tab = initial.EosTable(H.EOS_SMALL)
    shape, dxs = (20, 12, 10), (3.2e6, 2.8e6, 3.6e6)
    dt0, prim, pres, inv_va2max = _reference_dt(tab, shape, 31, dxs)
    vfast = 40.0 * float(np.abs(prim[1:4]).max())
    # layout (8, z, y, x) with two ghost layers: x index 1 is a ghost layer
    face = prim.copy()
    face[1, 6, 7, 1] = vfast
    edge = prim.copy()
    edge[2, 6, 1, 1] = 2.0 * vfast
    dt_face_ref = _mhd_residual_dt(face, pres, shape, dxs)
    dt_edge_ref = _mhd_residual_dt(edge, pres, shape, dxs)
    assert dt_face_ref < 0.5 * dt0
    assert abs(dt_edge_ref / dt0 - 1.0) <= TOL
    for _ in range(2):  # two calls in a row on the same scratch
        dt_face = _noalloc_dt(L, face, pres, shape, dxs, inv_va2max)
        dt_edge = _noalloc_dt(L, edge, pres, shape, dxs, inv_va2max)
        print(f"noalloc face-ghost dt {dt_face!r} vs MHD_Residual {dt_face_ref!r}; edge-ghost dt {dt_edge!r} vs {dt0!r}")
        assert abs(dt_face / dt_face_ref - 1.0) <= TOL
        assert abs(dt_edge / dt0 - 1.0) <= TOL
