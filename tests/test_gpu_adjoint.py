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
