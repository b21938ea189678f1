"""The linear elasticity model (elast::linear, linear.hpp:7-70) through the same GPU kernels, against the
FP64 oracle: energy and gradient, projected and unprojected Hessians (the make_spsd clamp lifts the three
rotation modes to 1e-3), and a tightly solved Newton trajectory; the mixed path reaches 1e-6."""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import mesh

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _pair(precision="fp64", E=1e5, nu=0.35, rho=1000.0):
    from oracle import pyoracle

    X, T = mesh.kuhn_box((6, 5, 4), (1.2, 1.0, 0.8))
    X = mesh.jitter_interior(X, 0.02, 11)
    ts = g.TimeStep(X, T, 1e-2, E, nu, rho)
    ts.set_precision(precision)
    ts.set_elastic_model("linear")
    ot = pyoracle.OracleTimeStep(X, T, 1e-2, E, nu, rho)
    ot.set_model("linear")
    fixed = np.where(X[:, 2] == 0.0)[0]
    ts.mark_dirichlet_batched(fixed, np.zeros((fixed.size, 3)))
    ot.mark_dirichlet(fixed)
    for t in (ts, ot):
        t.add_gravity((0.0, -9.8, 0.0))
    ts.reset("newton")
    ot.reset()
    return X, ts, ot


def test_linear_energy_gradient():
    X, ts, ot = _pair()
    rng = np.random.default_rng(5)
    u = rng.uniform(-1, 1, X.shape) * 0.1
    xt = rng.uniform(-1, 1, X.shape) * 0.05
    for t in (ts, ot):
        t.prepare_step()
        t.set("inertia_deform", xt)
        t.set("next_deform", u)
    e, eo = ts.update_energy_and_gradients(), ot.update_energy_and_gradients()
    assert abs(e - eo) <= FP64_RTOL * abs(eo)
    assert rel(ts.get("forces"), ot.get("forces")) <= FP64_RTOL
    u2 = u + 0.01 * rng.normal(size=X.shape)
    assert abs(ts.energy_at(u2) - ot.energy_at(u2)) <= FP64_RTOL * abs(ot.energy_at(u2))


@pytest.mark.parametrize("spsd", [False, True])
def test_linear_hessian_values(spsd):
    X, ts, ot = _pair()
    u = np.random.default_rng(6).uniform(-1, 1, X.shape) * 0.15
    for t in (ts, ot):
        t.set("next_deform", u)
        t.update_hessian(False, spsd, True)
    assert rel(ts.values("sysmatrix"), ot.values("sysmatrix")) <= FP64_RTOL


def test_linear_newton_trajectory():
    from oracle import pyoracle

    X, ts, ot = _pair()
    ts.set_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-13, cg_max_iters=20000)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-13, cg_max_iters=20000)
    for _ in range(5):
        ts.step()
        st = ts.stats()
        ot.prepare_step()
        _, sto = ot.compute_step("newton", op)
        ot.step_next()
        assert st["converged"] == 1 and sto["converged"] == 1
    assert rel(ts.get("deformation"), ot.get("deformation")) <= FP64_RTOL


def test_linear_mixed_reaches_residual():
    X, ts, _ = _pair(precision="mixed")
    ts.set_params(stop_mode=1, rel_tol=1e-6)
    for _ in range(3):
        ts.step()
        st = ts.stats()
        assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"]
