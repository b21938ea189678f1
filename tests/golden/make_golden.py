"""Generates tests/golden/oracle_small.npz from the FP64 oracle (run: python tests/golden/make_golden.py).

Seeded inputs on a small jittered Kuhn mesh: energy and gradient at a random state, the filtered SPD-
projected and the unfiltered raw Hessian values, the mass values, and three tightly solved Newton steps.
The CPU tests check that the oracle still reproduces these numbers; the GPU tests check the CUDA path
against them.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from ssim_gb300 import mesh  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_small.npz")
SETTINGS = dict(dt=1e-2, E=1e5, nu=0.45, rho=1000.0, gravity=(0.0, 0.0, -9.8))
# twelve Newton iterations with near-exact inner solves: quadratic convergence reaches round-off well before the
# last one, so two correct implementations agree to round-off whatever their stopping decisions
# a fixed 12 tight Newton iterations per step (no early stop: stop_floor 0)
NEWTON = dict(stop_mode=1, rel_tol=1e-14, cg_rtol=1e-13, cg_max_iters=20000, max_newton_iters=12, stop_floor=0.0)


def inputs():
    X, T = mesh.kuhn_box((4, 3, 3), (1.0, 0.75, 0.75))
    X = mesh.jitter_interior(X, 0.02, 21)
    fixed = np.where(X[:, 0] == 0.0)[0]
    u = mesh.uniform(22, X.size, -0.05, 0.05).reshape(X.shape)
    xt = mesh.uniform(23, X.size, -0.05, 0.05).reshape(X.shape)
    return X, T, fixed, u, xt


def oracle_for(X, T, fixed):
    s = SETTINGS
    ts = pyoracle.OracleTimeStep(X, T, s["dt"], s["E"], s["nu"], s["rho"])
    ts.mark_dirichlet(fixed)
    ts.add_gravity(s["gravity"])
    ts.reset()
    return ts


def generate():
    X, T, fixed, u, xt = inputs()
    ts = oracle_for(X, T, fixed)
    ts.prepare_step()
    ts.set("inertia_deform", xt)
    ts.set("next_deform", u)
    energy = ts.update_energy_and_gradients()
    forces = ts.get("forces")
    ts.update_hessian(False, True, True)
    h_spsd = ts.values("sysmatrix")
    ts.update_hessian(False, False, False)
    h_raw = ts.values("sysmatrix")
    mass = ts.values("mass")
    rp, ci = ts.csr_pattern()
    ts2 = oracle_for(X, T, fixed)
    traj = []
    for _ in range(3):
        ts2.prepare_step()
        ts2.compute_step("newton", pyoracle.default_params(**NEWTON))
        ts2.step_next()
        traj.append(ts2.get("deformation"))
    return dict(X=X, cells=T, fixed=fixed, u=u, xt=xt, energy=np.array(energy), forces=forces, h_spsd=h_spsd,
                h_raw=h_raw, mass=mass, row_ptr=rp, col_idx=ci, traj=np.stack(traj))


if __name__ == "__main__":
    d = generate()
    np.savez_compressed(OUT, **d)
    print(OUT, {k: v.shape for k, v in d.items()})
