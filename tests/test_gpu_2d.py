"""GPU parity for 2D triangles in the plane: the CUDA library through the C ABI against the FP64 oracle's
2D restatement (itself pinned by the reference's 2D element tests).  Bars as for the tets."""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import mesh, scenes
from oracle import scenes as oscenes

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _small(E=1e5, nu=0.4, rho=100.0):
    return scenes.sheet2d(9, 6, E=E, nu=nu, rho=rho)


def _drop_z(ot, which="sysmatrix"):
    A = ot.matrix(which).toarray()
    keep = np.array([k for k in range(A.shape[0]) if k % 3 != 2])
    return A[np.ix_(keep, keep)]


def test_rest_shape_pattern_mass():
    sc = _small()
    ts = scenes.build_timestep(sc, stepper="none")
    ot = oscenes.build_oracle(sc)
    assert ts.dim == 2
    assert rel(ts.rest_volume(), ot.rest_vol()) <= 1e-15
    assert rel(ts.dminv().reshape(-1, 4), ot.dminv().reshape(-1, 9)[:, :4]) <= 1e-15
    rp, ci = ts.csr_pattern()
    rpo, cio = ot.csr_pattern()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    assert rel(ts.values("mass"), ot.values("mass")) <= 1e-15
    rp2, ci2, v2 = ts.csr_2d("mass")
    import scipy.sparse as sp

    M2 = sp.csr_matrix((v2, ci2, rp2), shape=(2 * sc["X2"].shape[0],) * 2).toarray()
    assert rel(M2, _drop_z(ot, "mass")) <= 1e-15
    assert abs(ts.threshold_abs - ot.threshold_abs) <= 1e-14 * ot.threshold_abs


@pytest.mark.parametrize("model", [0, 1])
def test_energy_gradient_hessian(model):
    sc = _small()
    ts = scenes.build_timestep(sc, stepper="none")
    ot = oscenes.build_oracle(sc)
    ts.set_elastic_model(model)
    ot.set_model(model)
    rng = np.random.default_rng(11)
    n = sc["X"].shape[0]
    u = np.zeros((n, 3))
    u[:, :2] = rng.uniform(-1, 1, (n, 2)) * 0.08
    v = np.zeros((n, 3))
    v[:, :2] = rng.uniform(-1, 1, (n, 2))
    for t in (ts, ot):
        t.set("velocity", v)
        t.prepare_step()
        t.set("next_deform", u)
    e, eo = ts.update_energy_and_gradients(), ot.update_energy_and_gradients()
    assert abs(e - eo) <= FP64_RTOL * abs(eo)
    f = ts.get("forces")
    assert rel(f, ot.get("forces")) <= FP64_RTOL
    assert np.all(f[:, 2] == 0)
    u2 = u.copy()
    u2[:, :2] += 0.01 * rng.normal(size=(n, 2))
    assert abs(ts.energy_at(u2) - ot.energy_at(u2)) <= FP64_RTOL * abs(ot.energy_at(u2))
    for spsd in (False, True):
        for filt in (False, True):
            ts.update_hessian(False, spsd, filt)
            ot.update_hessian(False, spsd, filt)
            assert rel(ts.values("sysmatrix"), ot.values("sysmatrix")) <= FP64_RTOL, (spsd, filt)


def test_newton_trajectory_fp64_and_2dof_export():
    from oracle import pyoracle

    sc = _small()
    # the same stopping rule on both sides (relative 1e-11, no absolute floor; PCG 1e-13), so the states agree
    # to well below the 1e-10 bar
    params = g.default_params(stop_mode=1, rel_tol=1e-11, cg_rtol=1e-13, cg_max_iters=20000, stop_floor=0.0)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-11, cg_rtol=1e-13, cg_max_iters=20000, stop_floor=0.0)
    ts = scenes.build_timestep(sc, precision="fp64", stepper="newton", params=params)
    ot = oscenes.build_oracle(sc)
    for _ in range(5):
        ts.step()
        st = ts.stats()
        ot.prepare_step()
        _, sto = ot.compute_step("newton", op)
        ot.step_next()
        assert st["converged"] == 1 and sto["converged"] == 1
        assert abs(st["newton_iters"] - sto["newton_iters"]) <= 1
    u, uo = ts.get("deformation"), ot.get("deformation")
    assert rel(u, uo) <= FP64_RTOL
    assert np.all(u[:, 2] == 0.0) and u[:, 1].min() < -1e-4
    ts.update_hessian(False, True, True)
    ot.update_hessian(False, True, True)
    import scipy.sparse as sp

    rp2, ci2, v2 = ts.csr_2d("sysmatrix")
    H2 = sp.csr_matrix((v2, ci2, rp2), shape=(2 * sc["X2"].shape[0],) * 2).toarray()
    assert rel(H2, _drop_z(ot)) <= FP64_RTOL


@pytest.mark.parametrize("method", ["lbfgs", "pd"])
def test_lbfgs_pd_fp64(method):
    from oracle import pyoracle

    sc = _small()
    params = g.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-11, max_lbfgs_iters=20000, precond=2,
                              stop_floor=0.0)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-9, max_lbfgs_iters=20000, stop_floor=0.0)
    ts = scenes.build_timestep(sc, precision="fp64", stepper=method, params=params)
    ot = oscenes.build_oracle(sc)
    for _ in range(3):
        ts.step()
        st = ts.stats()
        ot.prepare_step()
        _, sto = ot.compute_step(method, op)
        ot.step_next()
        assert st["converged"] == 1 and sto["converged"] == 1
    assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-6


def test_mixed_newton_residual():
    from oracle import pyoracle

    sc = scenes.sheet2d(33, 17)
    params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-2, cg_eta_min=1e-4)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-12)
    ts = scenes.build_timestep(sc, precision="mixed", stepper="newton", params=params)
    ot = oscenes.build_oracle(sc)
    for _ in range(4):
        ts.step()
        st = ts.stats()
        assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"]
        ot.prepare_step()
        ot.compute_step("newton", op)
        ot.step_next()
    assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-5


def test_mixed_lbfgs_fp32_phase():
    """Mixed-precision L-BFGS on triangles runs its early iterations with the FP32 triangle pass
    (strain-relative 2D stable Neo-Hookean on the per-vertex FP32 split) and confirms in FP64: every step
    reaches 1e-6 |g0| and the state matches the all-FP64-evaluation run and the oracle's L-BFGS."""
    from oracle import pyoracle

    sc = scenes.sheet2d(33, 17)
    states = []
    for e32 in (1, 0):
        params = g.default_params(stop_mode=1, rel_tol=1e-6, max_lbfgs_iters=20000, mixed_elem32=e32)
        ts = scenes.build_timestep(sc, precision="mixed", stepper="lbfgs", params=params)
        for _ in range(3):
            ts.step()
            st = ts.stats()
            assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"], st
        states.append(ts.get("deformation"))
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-10, max_lbfgs_iters=20000)
    ot = oscenes.build_oracle(sc)
    for _ in range(3):
        ot.prepare_step()
        ot.compute_step("lbfgs", op)
        ot.step_next()
    uo = ot.get("deformation")
    assert rel(states[0], uo) <= 1e-4 and rel(states[1], uo) <= 1e-4
    # the FP32 triangle pass did run: its iterates differ from the all-FP64-evaluation run's
    assert not np.array_equal(states[0], states[1])


def test_2d_errors():
    X2, T = mesh.unit_square(3, 3)
    with pytest.raises(ValueError):
        g.TimeStep.tri2d(X2, np.array([[0, 1, 99]]), 1e-2, 1e5, 0.4, 100.0)
    with pytest.raises(ValueError):
        g.TimeStep.tri2d(X2, np.array([[0, 1, 2]]) * 0, 1e-2, 1e5, 0.4, 100.0)
    ts = g.TimeStep.tri2d(X2, T, 1e-2, 1e5, 0.4, 100.0)
    import ctypes as C

    import torch

    from ssim_gb300 import _lib

    ub = torch.zeros(27, dtype=torch.float64, device="cuda")
    vb = torch.zeros(27, dtype=torch.float64, device="cuda")
    eb = torch.zeros(T.shape[0], dtype=torch.float64, device="cuda")
    rc = ts._L.ssim_gb_adjoint_step(ts._h, C.c_void_p(ub.data_ptr()), C.c_void_p(vb.data_ptr()),
                                    C.c_void_p(eb.data_ptr()), 1e-6, 10, None, None)
    assert rc == _lib.ERR_STATE
