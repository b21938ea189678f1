"""The hand-written adjoint of the implicit step against FP64 central finite differences.

Scene (a reduced config 5): a cube of 4^3 hex cells x 6 tets, per-cell E log-uniform in [1e4, 1e6], bottom
face fixed, random initial velocities, 10 steps, checkpoints every 4; loss = sum |X + u_N - target|^2 with
target = X + 0.1 sin(2 pi X_x) e_z.  Directional derivatives on random directions (E perturbed relatively,
v0 absolutely) must agree with central differences of step 1e-6 to 1e-5 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup():
    import torch

    import ssim_gb300 as g
    from ssim_gb300 import adjoint, mesh

    X, T = mesh.kuhn_box((4, 4, 4))
    fixed = np.where(X[:, 2] == 0.0)[0]
    params = g.default_params(stop_mode=1, rel_tol=1e-14, cg_rtol=1e-13, cg_max_iters=20000, max_newton_iters=25,
                              precond=2, stop_floor=0.0)
    eng = adjoint.RolloutEngine(X, T, fixed, dt=1e-2, nu=0.45, rho=1000.0, params=params, adjoint_rtol=1e-13)
    E = torch.tensor(10.0 ** mesh.uniform(5, T.shape[0], 4.0, 6.0), dtype=torch.float64, device="cuda")
    v0 = torch.tensor(0.5 * mesh.normal(6, X.size).reshape(X.shape), dtype=torch.float64, device="cuda")
    v0[torch.tensor(fixed, device="cuda")] = 0.0
    Xt = torch.tensor(X, dtype=torch.float64, device="cuda")
    target = Xt.clone()
    target[:, 2] += 0.1 * torch.sin(2 * np.pi * Xt[:, 0])
    return eng, E, v0, Xt, target, adjoint


def test_adjoint_matches_central_differences():
    import torch

    eng, E, v0, Xt, target, adjoint = _setup()
    steps, k = 10, 4

    def loss(E_, v0_):
        u = adjoint.rollout(E_, v0_, eng, steps, k)
        return ((Xt + u - target) ** 2).sum()

    Eg = E.clone().requires_grad_(True)
    vg = v0.clone().requires_grad_(True)
    L = loss(Eg, vg)
    L.backward()
    gE, gv = Eg.grad.detach(), vg.grad.detach()
    assert eng.projected == 0
    rng = np.random.default_rng(7)
    h = 1e-6
    for _ in range(4):
        rE = torch.tensor(rng.normal(size=E.shape[0]), device="cuda")
        rv = torch.tensor(rng.normal(size=tuple(v0.shape)), device="cuda")
        with torch.no_grad():
            Lp = loss(E * (1 + h * rE), v0 + h * rv).item()
            Lm = loss(E * (1 - h * rE), v0 - h * rv).item()
        fd = (Lp - Lm) / (2 * h)
        ad = ((gE * E * rE).sum() + (gv * rv).sum()).item()
        assert abs(ad - fd) <= 1e-5 * abs(fd), (ad, fd)


def _rollout_grads(sc, precision, params, adjoint_rtol, steps, k):
    """dL/dE and dL/dv0 of the rollout scene ``sc`` through the adjoint, and the loss."""
    import torch

    from ssim_gb300 import adjoint

    eng = adjoint.RolloutEngine(sc["X"], sc["cells"], sc["fixed"], dt=sc["dt"], nu=sc["nu"], rho=sc["rho"],
                                precision=precision, params=params, adjoint_rtol=adjoint_rtol,
                                adjoint_max_iters=50000)
    E = torch.tensor(sc["E_cells"], dtype=torch.float64, device="cuda", requires_grad=True)
    v0 = torch.tensor(sc["v0"], dtype=torch.float64, device="cuda", requires_grad=True)
    Xt = torch.tensor(sc["X"], dtype=torch.float64, device="cuda")
    target = torch.tensor(sc["target"], dtype=torch.float64, device="cuda")
    L = ((Xt + adjoint.rollout(E, v0, eng, steps, k) - target) ** 2).sum()
    L.backward()
    return eng, E.grad.detach(), v0.grad.detach(), L.item()


def test_mixed_adjoint_matches_fp64_adjoint():
    """The mixed-precision adjoint (forward Newton and adjoint PCG at the benchmark's 1e-6 tolerances, FP32
    Hessian / PCG) against the FP64 adjoint solved tightly, on the rollout scene at 8^3 hex x 6 tets (3,072),
    12 steps, checkpoints every 4: the relative L2 error of each gradient stays below 1e-3."""
    import bench
    import ssim_gb300 as g
    from ssim_gb300 import scenes

    sc = scenes.rollout_cube(8)
    tight = g.default_params(stop_mode=1, rel_tol=1e-12, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=1e-14,
                             cg_max_iters=50000, max_newton_iters=40, precond=2, stop_floor=0.0)
    _, gE, gv, L = _rollout_grads(sc, "fp64", tight, 1e-13, 12, 4)
    eng, gE32, gv32, L32 = _rollout_grads(sc, "mixed", bench.newton_params(g), 1e-6, 12, 4)
    eE = ((gE32 - gE).norm() / gE.norm()).item()
    ev = ((gv32 - gv).norm() / gv.norm()).item()
    print(f"MIXED_ADJOINT grad_E_rel_err={eE:.3e} grad_v0_rel_err={ev:.3e} loss_rel_err={abs(L32 - L) / abs(L):.3e}")
    assert eng.projected == 0
    assert eE <= 1e-3 and ev <= 1e-3, (eE, ev)


def test_adjoint_fd_rollout_cube32():
    """The differentiable rollout at its benchmarked size: 32^3 hex x 6 = 196,608 tets, 40 steps, checkpoints
    every 8 (ssim_gb300.scenes.rollout_cube).  The FP64 adjoint's directional derivatives on random
    directions (seed 7; E perturbed relatively, v0 absolutely) against FP64 central differences of step 1e-6
    (the method of the reference's tests/fem_time_step_diff/main.cpp:47-91), every rollout solved to 1e-12
    relative residual: worst relative error <= 1e-5.  SSIM_GB_ADJOINT_FD_DIRECTIONS sets how many directions
    (default 4; 32 for the full check) and SSIM_GB_ADJOINT_FD_OFFSET which of the seeded sequence come first,
    so the full check can be split over runs."""
    import json
    import os

    import torch

    import ssim_gb300 as g
    from ssim_gb300 import adjoint, scenes

    ndir = int(os.environ.get("SSIM_GB_ADJOINT_FD_DIRECTIONS", "4"))
    offset = int(os.environ.get("SSIM_GB_ADJOINT_FD_OFFSET", "0"))
    sc = scenes.rollout_cube(32)
    steps, k, h = 40, 8, 1e-6
    tight = g.default_params(stop_mode=1, rel_tol=1e-12, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=1e-14,
                             cg_max_iters=50000, max_newton_iters=40, precond=2, stop_floor=0.0)
    eng, gE, gv, L = _rollout_grads(sc, "fp64", tight, 1e-13, steps, k)
    assert eng.projected == 0
    E = torch.tensor(sc["E_cells"], dtype=torch.float64, device="cuda")
    v0 = torch.tensor(sc["v0"], dtype=torch.float64, device="cuda")
    Xt = torch.tensor(sc["X"], dtype=torch.float64, device="cuda")
    target = torch.tensor(sc["target"], dtype=torch.float64, device="cuda")
    fixed = torch.tensor(sc["fixed"], device="cuda")

    def loss(E_, v0_):
        with torch.no_grad():
            return ((Xt + adjoint.rollout(E_, v0_, eng, steps, k) - target) ** 2).sum().item()

    rng = np.random.default_rng(7)
    errs = []
    for d in range(offset + ndir):
        rE = torch.tensor(rng.normal(size=E.shape[0]), device="cuda")
        rv = torch.tensor(rng.normal(size=tuple(v0.shape)), device="cuda")
        rv[fixed] = 0.0
        if d < offset:
            continue
        fd = (loss(E * (1 + h * rE), v0 + h * rv) - loss(E * (1 - h * rE), v0 - h * rv)) / (2 * h)
        ad = ((gE * E * rE).sum() + (gv * rv).sum()).item()
        errs.append(abs(ad - fd) / abs(fd))
    print("ADJOINT_FD " + json.dumps({"workload": sc["name"], "steps": steps, "checkpoint_every": k, "h": h,
                                      "directions": list(range(offset, offset + ndir)), "rel_err": errs,
                                      "max_rel_err": max(errs), "loss": L}))
    assert max(errs) <= 1e-5, errs
