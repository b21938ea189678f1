"""GPU parity for mass-spring systems (cloth): the CUDA library through the C ABI against the FP64 oracle's
own spring restatement (the reference has no spring model).

Bars as for the tets: plain FP64 kernel outputs <= 1e-10 relative, tightly solved FP64 trajectories
<= 1e-6 relative between the GPU and the oracle steppers, mixed precision to its stated residual.
"""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import scenes
from oracle import scenes as oscenes

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _small(n=12):
    return scenes.cloth(n, h=0.05, k=1e3, areal_density=0.5, dt=1e-2)


def test_pattern_and_mass():
    sc = _small()
    ts = scenes.build_timestep(sc, stepper="none")
    ot = oscenes.build_oracle(sc)
    rp, ci = ts.csr_pattern()
    rpo, cio = ot.csr_pattern()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    assert rel(ts.values("mass"), ot.values("mass")) == 0.0
    assert rel(ts.values("mass_filtered"), ot.values("mass_filtered")) == 0.0
    assert abs(ts.threshold_abs - ot.threshold_abs) <= 1e-14 * ot.threshold_abs


def test_energy_gradient_hessian():
    sc = _small()
    ts = scenes.build_timestep(sc, stepper="none")
    ot = oscenes.build_oracle(sc)
    rng = np.random.default_rng(21)
    v = rng.uniform(-1, 1, sc["X"].shape)
    u = rng.uniform(-1, 1, sc["X"].shape) * 0.02
    u[:, :2] -= 0.1 * sc["X"][:, :2]  # compress in-plane: some springs shorter than rest
    for t in (ts, ot):
        t.set("velocity", v)
        t.prepare_step()
        t.set("next_deform", u)
    e, eo = ts.update_energy_and_gradients(), ot.update_energy_and_gradients()
    assert abs(e - eo) <= FP64_RTOL * abs(eo)
    assert rel(ts.get("forces"), ot.get("forces")) <= FP64_RTOL
    u2 = u + 0.003 * rng.normal(size=u.shape)
    assert abs(ts.energy_at(u2) - ot.energy_at(u2)) <= FP64_RTOL * abs(ot.energy_at(u2))
    for spsd in (False, True):
        for filt in (False, True):
            ts.update_hessian(False, spsd, filt)
            ot.update_hessian(False, spsd, filt)
            assert rel(ts.values("sysmatrix"), ot.values("sysmatrix")) <= FP64_RTOL, (spsd, filt)
    x = rng.normal(size=u.shape)
    assert rel(ts.spmv(x), ot.spmv(x).reshape(-1, 3)) <= FP64_RTOL


@pytest.mark.parametrize("method", ["newton", "lbfgs", "pd"])
def test_steppers_fp64_match_oracle(method):
    """Three cloth steps (corners pinned, gravity) solved to 1e-9 relative gradient: the GPU stepper and
    the oracle's land on the same state to 1e-6 relative."""
    from oracle import pyoracle

    sc = _small(16)
    params = g.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-11, cg_max_iters=20000,
                              max_lbfgs_iters=50000, max_newton_iters=200, stop_floor=0.0)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-12, cg_max_iters=20000,
                                 max_lbfgs_iters=50000, max_newton_iters=200)
    ts = scenes.build_timestep(sc, precision="fp64", stepper=method, params=params)
    ot = oscenes.build_oracle(sc)
    for _ in range(3):
        ts.prepare_step()
        ts.compute_step()
        st = ts.stats()
        ts.step_next()
        ot.prepare_step()
        _, sto = ot.compute_step(method, op)
        ot.step_next()
        assert st["converged"] == 1, st
        assert sto["converged"] == 1, sto
    u, uo = ts.get("deformation"), ot.get("deformation")
    assert np.abs(uo).max() > 1e-4
    assert rel(u, uo) <= 1e-6
    assert np.all(u[sc["fixed"]] == 0.0)


@pytest.mark.parametrize("method", ["newton", "lbfgs", "pd"])
def test_steppers_mixed_reach_residual(method):
    """Mixed precision (FP32 Hessian/PD matrix and PCG, FP64 spring forces) reaches 1e-6 relative
    residual per step; state within 1e-4 relative of the FP64 oracle solved tightly."""
    from oracle import pyoracle

    sc = _small(24)
    params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_rtol=1e-3, max_lbfgs_iters=50000,
                              max_newton_iters=200)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-12, cg_max_iters=20000,
                                 max_newton_iters=200)
    ts = scenes.build_timestep(sc, precision="mixed", stepper=method, params=params)
    ot = oscenes.build_oracle(sc)
    for _ in range(3):
        ts.step()
        st = ts.stats()
        assert st["converged"] == 1, st
        ot.prepare_step()
        _, sto = ot.compute_step("newton", op)
        ot.step_next()
        assert sto["converged"] == 1
    assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-4


def test_spring_errors():
    sc = _small(4)
    with pytest.raises(ValueError):
        g.TimeStep.springs(sc["X"], sc["cells"], 1e3, vertex_mass=np.ones(3))
    with pytest.raises(ValueError):
        g.TimeStep.springs(sc["X"], sc["cells"], -1.0, mass=1.0)
    with pytest.raises(ValueError):
        g.TimeStep.springs(sc["X"], np.array([[0, 0]]), 1e3, mass=1.0)
    with pytest.raises(ValueError):
        g.TimeStep.springs(sc["X"], np.array([[0, 99]]), 1e3, mass=1.0)
    with pytest.raises(ValueError):
        g.TimeStep.springs(sc["X"], np.zeros((0, 2)), 1e3, mass=1.0)
    ts = g.TimeStep.springs(sc["X"], sc["cells"], 1e3, mass=1e-3)
    with pytest.raises(g.SsimGbError):
        ts.set_material(np.ones(sc["cells"].shape[0]), None)
