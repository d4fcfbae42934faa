"""The adjoint of the fused FP64 step against finite differences.

J(U_T) = sum over the top 8 layers of dimension 0 (MURaM's vertical) of a
seeded mask times B_x^2, after a few fixed-dt steps of a periodic box.  The
adjoint's dJ/dU_0 projected on seeded random directions must match central
differences of J computed by the forward step (GPU, and the CPU oracle as the
reference's own path).  The step is piecewise smooth: limiter branches and the
EOS table's bilinear cells have kinks, so the perturbation must stay within
one piece -- 1e-8 of each field's scale does (1e-6 already crosses EOS table
cell edges for some directions), and FP64 rounding keeps the differences
accurate to ~1e-8 there.
"""
import numpy as np
import pytest

import helpers as H
from muram_main_gb300 import gpumhd, initial

pytestmark = pytest.mark.gpu


def fixed_dt_box(nx, ny, nz, seed, frac=0.6):
    tab = initial.EosTable(H.EOS_SMALL)
    U0 = initial.periodic_box(tab, nx, ny, nz, seed=seed)
    g = gpumhd.MuramGPU(gpumhd.default_params(nx, ny, nz, 3.2e6), eos_path=H.EOS_SMALL)
    g.upload_state(U0)
    dt = float(g.run_steps(1)[0]) * frac
    g.close()
    p = gpumhd.default_params(nx, ny, nz, 3.2e6, autostep=0, dt=dt)
    return gpumhd.MuramGPU(p, eos_path=H.EOS_SMALL), U0, dt


def objective(U, mask):
    return float(np.sum(mask * U[5, 2:-2, 2:-2, -10:-2] ** 2))


def objective_grad(U, mask):
    lam = np.zeros_like(U)
    lam[5, 2:-2, 2:-2, -10:-2] = 2.0 * mask * U[5, 2:-2, 2:-2, -10:-2]
    return lam


def J_after(g, U, nsteps, mask):
    g.upload_state(U)
    g.run_steps(nsteps)
    return objective(g.download_state(), mask)


def directions(U, count, seed):
    rng = np.random.default_rng(seed)
    scale = np.sqrt(np.mean(U[:, 2:-2, 2:-2, 2:-2] ** 2, axis=(1, 2, 3)))
    out = []
    for _ in range(count):
        v = np.zeros_like(U)
        v[:, 2:-2, 2:-2, 2:-2] = rng.standard_normal(U[:, 2:-2, 2:-2, 2:-2].shape) * scale[:, None, None, None]
        out.append(initial.fill_ghosts(v, periodic_x=True))
    return out


def test_adjoint_matches_finite_differences(gpu_lib):
    nx, ny, nz, steps = 16, 12, 8, 3
    g, U0, _ = fixed_dt_box(nx, ny, nz, seed=41)
    mask = np.random.default_rng(7).uniform(0.0, 1.0, (nz, ny, 8))
    UT_ref = None
    g.upload_state(U0)
    g.run_steps(steps)
    UT_ref = g.download_state()
    g.upload_state(U0)
    grad = g.adjoint(steps, objective_grad(UT_ref, mask), checkpoint_every=2)
    assert np.all(grad[:, :2] == 0) and np.all(grad[:, :, :, -2:] == 0)
    eps = 1e-8
    errs = []
    for v in directions(U0, 6, seed=3):
        fd = (J_after(g, U0 + eps * v, steps, mask) - J_after(g, U0 - eps * v, steps, mask)) / (2 * eps)
        ad = float(np.sum(grad * v))
        errs.append(abs(ad - fd) / abs(fd))
    print("adjoint vs central differences, relative errors:", np.array2string(np.array(errs), precision=2))
    assert np.median(errs) < 1e-6 and max(errs) < 1e-5, errs
    g.close()


def test_checkpoint_spacing_does_not_change_the_gradient(gpu_lib):
    g, U0, _ = fixed_dt_box(12, 8, 8, seed=5)
    mask = np.random.default_rng(1).uniform(0.0, 1.0, (8, 8, 8))
    g.upload_state(U0)
    g.run_steps(4)
    lam = objective_grad(g.download_state(), mask)
    grads = []
    for k in (1, 3, 4):
        g.upload_state(U0)
        grads.append(g.adjoint(4, lam, checkpoint_every=k))
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[0], grads[2])
    # the context's state is left as it was
    assert np.array_equal(g.download_state()[:, 2:-2, 2:-2, 2:-2], U0[:, 2:-2, 2:-2, 2:-2])
    g.close()


def test_adjoint_against_oracle_differences(gpu_lib):
    """Directional derivatives of the same objective by central differences
    of the CPU oracle (the reference's algorithm in FP64) on the same box."""
    from oracle import oracle as O
    nx, ny, nz, steps = 12, 8, 8, 2
    g, U0, dt = fixed_dt_box(nx, ny, nz, seed=9)
    mask = np.random.default_rng(2).uniform(0.0, 1.0, (nz, ny, 8))
    g.upload_state(U0)
    g.run_steps(steps)
    lam = objective_grad(g.download_state(), mask)
    g.upload_state(U0)
    grad = g.adjoint(steps, lam, checkpoint_every=1)
    eos = O.Eos(H.EOS_SMALL)

    def J_oracle(U):
        p = O.make_params(nx, ny, nz, 3.2e6)
        p.autostep = 0
        p.dt = dt
        st = O.State(p, U)
        st.step(eos, steps)
        return objective(st.U, mask)

    eps = 1e-8
    for v in directions(U0, 3, seed=11):
        fd = (J_oracle(U0 + eps * v) - J_oracle(U0 - eps * v)) / (2 * eps)
        ad = float(np.sum(grad * v))
        print("adjoint", ad, "oracle differences", fd)
        assert abs(ad - fd) <= 1e-5 * abs(fd)
    g.close()


class MuramSteps:
    """torch.autograd.Function over nsteps fused FP64 steps of a box: forward
    runs the steps (fixed dt) from U0, backward calls the library's adjoint."""

    @staticmethod
    def make(torch):
        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, U0, box, nsteps, checkpoint_every):
                box.upload_state(U0.detach().cpu().numpy())
                box.run_steps(nsteps)
                ctx.box, ctx.nsteps, ctx.k = box, nsteps, checkpoint_every
                ctx.save_for_backward(U0)
                return torch.from_numpy(box.download_state())

            @staticmethod
            def backward(ctx, grad_UT):
                (U0,) = ctx.saved_tensors
                ctx.box.upload_state(U0.detach().cpu().numpy())
                g = ctx.box.adjoint(ctx.nsteps, grad_UT.detach().cpu().numpy(), checkpoint_every=ctx.k)
                return torch.from_numpy(g), None, None, None

        return _Fn


def test_torch_autograd_wrapper(gpu_lib):
    torch = pytest.importorskip("torch")
    g, U0, _ = fixed_dt_box(12, 8, 8, seed=13)
    mask = np.random.default_rng(4).uniform(0.0, 1.0, (8, 8, 8))
    Fn = MuramSteps.make(torch)
    U = torch.tensor(U0, dtype=torch.float64, requires_grad=True)
    UT = Fn.apply(U, g, 3, 2)
    J = torch.sum(torch.from_numpy(mask) * UT[5, 2:-2, 2:-2, -10:-2] ** 2)
    J.backward()
    g.upload_state(U0)
    g.run_steps(3)
    UTn = g.download_state()
    Jv = float(J.detach())
    assert abs(Jv - objective(UTn, mask)) <= 1e-12 * abs(Jv)
    g.upload_state(U0)
    ref = g.adjoint(3, objective_grad(UTn, mask), checkpoint_every=2)
    # torch forms dJ/dU_T = 2 * mask * U_T in its own operation order
    assert np.allclose(U.grad.numpy(), ref, rtol=1e-13, atol=0)
    g.close()
