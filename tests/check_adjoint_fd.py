"""The differentiable-rollout check at full size: the adjoint gradient of the 32^3-cube rollout against
FP64 central finite differences on random directions (run on a GPU; not collected by pytest because one
run takes minutes):

    python tests/check_adjoint_fd.py [--n 32] [--steps 40] [--directions 32] [--checkpoint 8]

Scene: ssim_gb300.scenes.rollout_cube (per-cell E log-uniform in [1e4, 1e6], seed 5; initial velocities
N(0, 0.5^2), seed 6; bottom face fixed; dt = 1e-2); loss = sum |X + u_N - target|^2 with target = X +
0.1 sin(2 pi X_x) e_z.  Directions (seed 7): E perturbed relatively, v0 absolutely, step h = 1e-6; FP64
rollouts solved to 1e-12 relative gradient (PCG 1e-13) so the differences resolve the derivative.
Prints one JSON line with the worst relative error over the directions.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--directions", type=int, default=32)
    ap.add_argument("--checkpoint", type=int, default=8)
    ap.add_argument("--h", type=float, default=1e-6)
    args = ap.parse_args()

    import torch

    import ssim_gb300 as g
    from ssim_gb300 import adjoint, scenes

    sc = scenes.rollout_cube(args.n)
    params = g.default_params(stop_mode=1, rel_tol=1e-12, cg_rtol=1e-13, cg_max_iters=50000, max_newton_iters=40,
                              precond=2, stop_floor=0.0)
    eng = adjoint.RolloutEngine(sc["X"], sc["cells"], sc["fixed"], dt=sc["dt"], nu=sc["nu"], rho=sc["rho"],
                                precision="fp64", params=params, adjoint_rtol=1e-13, adjoint_max_iters=50000)
    E = torch.tensor(sc["E_cells"], dtype=torch.float64, device="cuda")
    v0 = torch.tensor(sc["v0"], dtype=torch.float64, device="cuda")
    Xt = torch.tensor(sc["X"], dtype=torch.float64, device="cuda")
    target = torch.tensor(sc["target"], dtype=torch.float64, device="cuda")

    def loss(E_, v0_):
        u = adjoint.rollout(E_, v0_, eng, args.steps, args.checkpoint)
        return ((Xt + u - target) ** 2).sum()

    t0 = time.perf_counter()
    Eg = E.clone().requires_grad_(True)
    vg = v0.clone().requires_grad_(True)
    L = loss(Eg, vg)
    L.backward()
    gE, gv = Eg.grad.detach(), vg.grad.detach()
    t_grad = time.perf_counter() - t0
    rng = np.random.default_rng(7)
    fixed = torch.tensor(sc["fixed"], device="cuda")
    errs = []
    for _ in range(args.directions):
        rE = torch.tensor(rng.normal(size=E.shape[0]), device="cuda")
        rv = torch.tensor(rng.normal(size=tuple(v0.shape)), device="cuda")
        rv[fixed] = 0.0
        with torch.no_grad():
            Lp = loss(E * (1 + args.h * rE), v0 + args.h * rv).item()
            Lm = loss(E * (1 - args.h * rE), v0 - args.h * rv).item()
        fd = (Lp - Lm) / (2 * args.h)
        ad = ((gE * E * rE).sum() + (gv * rv).sum()).item()
        errs.append(abs(ad - fd) / max(abs(fd), 1e-300))
    print(json.dumps({"workload": sc["name"], "steps": args.steps, "directions": args.directions, "h": args.h,
                      "max_rel_err": max(errs), "median_rel_err": float(np.median(errs)),
                      "projected_fallbacks": eng.projected, "loss": L.item(),
                      "gradient_s": round(t_grad, 2), "total_s": round(time.perf_counter() - t0, 2)}))


if __name__ == "__main__":
    main()
