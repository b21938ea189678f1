"""GPU parity: the CUDA library (through the C ABI) against the FP64 oracle on identical seeded inputs.

Bars: integer / index data bit-exact; plain FP64 path <= 1e-10 relative (per kernel output and on
tightly-solved trajectories); mixed FP32/FP64 path: Newton residual <= 1e-6 relative and its state
error against the FP64 oracle stated in the test.
"""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import mesh, scenes
from oracle import scenes as oscenes

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    den = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / den


def _pair(X, T, dt=1e-2, E=1e6, nu=0.33, rho=1e3, precision="fp64"):
    ts = g.TimeStep(X, T, dt, E, nu, rho)
    ts.set_precision(precision)
    ts.reset("none")
    from oracle import pyoracle

    ot = pyoracle.OracleTimeStep(X, T, dt, E, nu, rho)
    return ts, ot


def _meshes():
    X7, T7 = mesh.unit_box(7, 7, 7)
    Xk, Tk = mesh.kuhn_box((6, 5, 4), (1.2, 1.0, 0.8))
    Xj = mesh.jitter_interior(Xk, 0.02, 11)
    return {"tetra": mesh.tetra(), "unit_box7": (X7, T7), "kuhn_jitter": (Xj, Tk)}


@pytest.mark.parametrize("name", ["tetra", "unit_box7", "kuhn_jitter"])
def test_rest_shape(name):
    X, T = _meshes()[name]
    ts, ot = _pair(X, T)
    assert rel(ts.rest_volume(), ot.rest_vol()) == 0.0
    assert rel(ts.dminv(), ot.dminv()) == 0.0
    rp, ci = ts.csr_pattern()
    rpo, cio = ot.csr_pattern()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)


@pytest.mark.parametrize("name", ["tetra", "unit_box7", "kuhn_jitter"])
def test_energy_gradient(name):
    X, T = _meshes()[name]
    ts, ot = _pair(X, T, rho=10.0)
    rng = np.random.default_rng(5)
    u = rng.uniform(-1, 1, X.shape) * 0.1
    xt = rng.uniform(-1, 1, X.shape) * 0.05
    for t in (ts, ot):
        t.prepare_step()
        t.set("inertia_deform", xt)
        t.set("next_deform", u)
    e = ts.update_energy_and_gradients()
    eo = ot.update_energy_and_gradients()
    assert abs(e - eo) <= FP64_RTOL * abs(eo)
    assert rel(ts.get("forces"), ot.get("forces")) <= FP64_RTOL
    # value-only evaluation at another state
    u2 = u + 0.01 * rng.normal(size=X.shape)
    assert abs(ts.energy_at(u2) - ot.energy_at(u2)) <= FP64_RTOL * abs(ot.energy_at(u2))


@pytest.mark.parametrize("name", ["tetra", "unit_box7", "kuhn_jitter"])
@pytest.mark.parametrize("spsd", [False, True])
@pytest.mark.parametrize("filt", [False, True])
def test_hessian_values(name, spsd, filt):
    X, T = _meshes()[name]
    ts, ot = _pair(X, T, E=1e5, nu=0.45, rho=1000.0)
    fixed = np.where(X[:, 0] == X[:, 0].min())[0]
    ts.mark_dirichlet_batched(fixed, np.zeros((fixed.size, 3)))
    ot.mark_dirichlet(fixed)
    u = np.random.default_rng(6).uniform(-1, 1, X.shape) * 0.15
    ts.set("next_deform", u)
    ot.set("next_deform", u)
    ts.update_hessian(False, spsd, filt)
    ot.update_hessian(False, spsd, filt)
    assert rel(ts.values("sysmatrix"), ot.values("sysmatrix")) <= FP64_RTOL


def test_mass_matrices():
    X, T = _meshes()["kuhn_jitter"]
    ts, ot = _pair(X, T, rho=700.0)
    fixed = np.arange(0, X.shape[0], 7)
    ts.mark_dirichlet_batched(fixed, np.zeros((fixed.size, 3)))
    ot.mark_dirichlet(fixed)
    ot.reset()
    assert rel(ts.values("mass"), ot.values("mass")) <= 1e-15
    assert rel(ts.values("mass_filtered"), ot.values("mass_filtered")) <= 1e-15
    assert abs(ts.threshold_abs - ot.threshold_abs) <= 1e-14 * ot.threshold_abs


@pytest.mark.parametrize("precond", [1, 2])
def test_spmv_and_pcg(precond):
    X, T = _meshes()["kuhn_jitter"]
    ts, ot = _pair(X, T, E=1e5, nu=0.45, rho=1000.0)
    ts.set_params(precond=precond)
    u = np.random.default_rng(7).uniform(-1, 1, X.shape) * 0.05
    for t in (ts, ot):
        t.set("next_deform", u)
        t.update_hessian(False, True, True)
    x = np.random.default_rng(8).normal(size=X.shape)
    assert rel(ts.spmv(x), ot.spmv(x).reshape(-1, 3)) <= FP64_RTOL
    assert rel(ts.spmv(x, "mass"), ot.spmv(x, "mass").reshape(-1, 3)) <= FP64_RTOL
    assert rel(ts.spmv(x, "mass_filtered"), ot.spmv(x, "mass_filtered").reshape(-1, 3)) <= FP64_RTOL
    xs, it, rr = ts.pcg(x, rtol=1e-12, max_iters=5000)
    xo, ito, rro = ot.pcg(x, rtol=1e-12, max_iters=5000, precond=precond)
    assert abs(it - ito) <= 1
    assert rr <= 1e-12 and rro <= 1e-12
    assert rel(xs, xo.reshape(-1, 3)) <= 1e-9


def test_symmetric_storage_export_roundtrip():
    """The symmetric block store exports the reference's full CSR: values symmetric and equal to the
    oracle's full assembly on a mesh with a cell that repeats no vertex order (jittered Kuhn)."""
    X, T = _meshes()["kuhn_jitter"]
    ts, ot = _pair(X, T, E=2e5, nu=0.3, rho=500.0)
    u = np.random.default_rng(12).uniform(-1, 1, X.shape) * 0.2
    for t in (ts, ot):
        t.set("next_deform", u)
        t.update_hessian(False, False, False)
    H = ts.matrix("sysmatrix")
    assert abs(H - H.T).max() == 0.0
    assert rel(H.data, ot.values("sysmatrix")) <= FP64_RTOL


def test_mixed_kernels_close_to_fp64():
    """FP32 Hessian / assembly against the FP64 oracle: relative error stated (<= 1e-5)."""
    X, T = _meshes()["kuhn_jitter"]
    ts, ot = _pair(X, T, E=1e5, nu=0.45, rho=1000.0, precision="mixed")
    u = np.random.default_rng(9).uniform(-1, 1, X.shape) * 0.1
    for t in (ts, ot):
        t.set("next_deform", u)
        t.update_hessian(False, True, True)
    assert rel(ts.values("sysmatrix"), ot.values("sysmatrix")) <= 1e-5
    # energy / gradient stay FP64 in the mixed path
    for t in (ts, ot):
        t.prepare_step()
        t.set("next_deform", u)
    e, eo = ts.update_energy_and_gradients(), ot.update_energy_and_gradients()
    assert abs(e - eo) <= FP64_RTOL * abs(eo)
    assert rel(ts.get("forces"), ot.get("forces")) <= FP64_RTOL


def _run(scene, precision, params, oracle_params, steps, rtol=None):
    ts = scenes.build_timestep(scene, precision=precision, params=params, rtol=rtol)
    ot = oscenes.build_oracle(scene, rtol=rtol)
    hist = []
    for _ in range(steps):
        ts.prepare_step()
        r = ts.compute_step()
        st = ts.stats()
        ts.step_next()
        ot.prepare_step()
        ro, sto = ot.compute_step("newton", oracle_params)
        ot.step_next()
        hist.append((r, ro, st, sto))
    return ts, ot, hist


def test_newton_trajectory_fp64_tight():
    """Plain FP64 Newton on the 6,000-tet cube (top fixed, gravity) for 10 steps, solved tightly:
    the trajectory matches the oracle to 1e-10 relative."""
    scene = scenes.cube10()
    params = g.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-12, cg_max_iters=20000)
    from oracle import pyoracle

    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-12, cg_max_iters=20000)
    ts, ot, hist = _run(scene, "fp64", params, op, 10)
    for r, ro, st, sto in hist:
        assert st["converged"] == 1, st
        assert sto["converged"] == 1, sto
        assert abs(st["newton_iters"] - sto["newton_iters"]) <= 1
    u, uo = ts.get("deformation"), ot.get("deformation")
    assert rel(u, uo) <= FP64_RTOL
    assert rel(ts.get("velocity"), ot.get("velocity")) <= 1e-8
    assert np.all(u[scene["fixed"]] == 0.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_box_scene(precision):
    """The reference's unit_box(11, 11, 11) (5 tets per hex, 5,000 tets) with its harness conventions
    (tests/fem_time_step/main.cpp:54-67: x = 0 face fixed, gravity on y, E 1e6, nu 0.4, rho 10): 5 Newton
    steps to 1e-9 (FP64, matching the oracle's trajectory to 1e-10) or 1e-7 (mixed, within 1e-5 of it; on
    this stiff, light scene a 1e-6 residual leaves state errors up to about 2e-5, wherever in that band the
    iterates of a given PCG matrix happen to stop)."""
    from oracle import pyoracle

    scene = scenes.reference_box()
    if precision == "fp64":
        params = g.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-12, cg_max_iters=20000)
    else:
        params = g.default_params(stop_mode=1, rel_tol=1e-7, cg_forcing=1, cg_rtol=1e-2, cg_eta_min=1e-4)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-9 if precision == "fp64" else 1e-10, cg_rtol=1e-12,
                                 cg_max_iters=20000)
    ts, ot, hist = _run(scene, precision, params, op, 5)
    for r, ro, st, sto in hist:
        assert st["converged"] == 1 and sto["converged"] == 1
    u, uo = ts.get("deformation"), ot.get("deformation")
    assert np.all(u[scene["fixed"]] == 0.0) and u[:, 1].min() < 0
    assert rel(u, uo) <= (FP64_RTOL if precision == "fp64" else 1e-5)


def test_newton_reference_settings_fp64():
    """Reference settings (stop |g| < rtol*sum|M|/3 with rtol 1e-2 default, PCG 1e-8): both converge every
    step and agree to the solver tolerance."""
    scene = scenes.cube10()
    from oracle import pyoracle

    ts, ot, hist = _run(scene, "fp64", g.default_params(), pyoracle.default_params(), 5)
    for r, ro, st, sto in hist:
        assert st["converged"] == 1 and sto["converged"] == 1
        assert r < ts.threshold_abs
    assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-3


def test_newton_mixed_residual():
    """Mixed precision Newton reaches 1e-6 relative residual each step; state error vs the FP64 oracle
    solved to the same residual is below 1e-5 relative."""
    scene = scenes.cube10()
    params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-2, cg_eta_min=1e-4)
    from oracle import pyoracle

    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-12)
    ts, ot, hist = _run(scene, "mixed", params, op, 5)
    for r, ro, st, sto in hist:
        assert st["converged"] == 1
        assert st["grad_norm"] <= 1e-6 * st["grad_norm0"]
    assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-5


def test_determinism_bitwise():
    scene = scenes.cube10()
    outs = []
    for _ in range(2):
        ts = scenes.build_timestep(scene, precision="mixed", params=g.default_params(stop_mode=1, rel_tol=1e-6))
        for _ in range(2):
            ts.step()
        outs.append(ts.get("deformation"))
    assert np.array_equal(outs[0], outs[1])


def test_errors_like_reference():
    X, T = mesh.unit_box(3, 3, 3)
    ts = g.TimeStep(X, T, 1e-2)
    with pytest.raises(ValueError):
        ts.set_poisson(0.5)
    with pytest.raises(ValueError):
        ts.set_time_step(0.0)
    with pytest.raises(ValueError):
        ts.set_threshold(1.0)
    with pytest.raises(ValueError):
        ts.add_ext_force_dof(3, 1.0)
    with pytest.raises(ValueError):
        ts.mark_dirichlet_batched([X.shape[0]], np.zeros((1, 3)))
    bad = T.copy()
    bad[0, 0] = -1
    with pytest.raises(ValueError):
        g.TimeStep(X, bad, 1e-2)
    with pytest.raises(ValueError):
        g.TimeStep(X, T, 1e-2, 1e6, 0.6)  # reset() checks the Poisson ratio (time_step.hpp:371-372)


def test_pyssim_facade_matches_oracle():
    from ssim_gb300.pyssim.fem import TetFiniteElementSolver_Cuda, unit_box

    v, c = unit_box(6, 4, 4)
    vert, elem = v.T.copy(), c.T.copy()
    s = TetFiniteElementSolver_Cuda(vert, elem, 1e-2, 1e5, 0.4, 100.0, "newton")
    s.set_rtol(1e-4)
    fixed = np.where(vert[:, 0] == 0)[0].astype(np.int32)
    s.mark_dirichlet_batched(fixed, np.zeros((3, fixed.size)))
    s.add_gravity(np.array([0, 0, -9.81]))
    s.reset()
    for _ in range(3):
        ms = s.step()
        assert ms > 0
    d = s.deformation()
    assert d.shape == (3, vert.shape[0])
    assert np.abs(d[:, fixed]).max() == 0.0 and d[2].min() < 0
    s.update_hessian(True)
    H = s.hessian()
    assert H.shape == (3 * vert.shape[0],) * 2
    assert abs(H - H.T).max() <= 1e-9 * abs(H).max()
    assert s.mass_matrix().nnz == H.nnz


@pytest.mark.parametrize("method", ["lbfgs", "pd"])
def test_lbfgs_and_pd_fp64(method):
    """L-BFGS (backward_euler.hpp:43-67) and the Laplacian-preconditioned L-BFGS ("PD",
    projective_dynamics.hpp:9-97) on the 6,000-tet cube, FP64, solved to 1e-9 relative gradient: the same
    state as the oracle's steppers to 1e-6 relative."""
    from oracle import pyoracle

    scene = scenes.cube10()
    params = g.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-11, max_lbfgs_iters=20000, precond=2)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-9, max_lbfgs_iters=20000)
    ts = scenes.build_timestep(scene, precision="fp64", stepper=method, params=params)
    ot = oscenes.build_oracle(scene)
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
    assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-6


@pytest.mark.parametrize("history", [3, 12])
def test_lbfgs_history_compact_and_two_loop(history):
    """L-BFGS with up to 8 pairs takes its direction from the compact form of the L-BFGS matrix, with more
    from the two-loop recursion; both are the oracle's two-loop direction, and land on its state."""
    from oracle import pyoracle

    scene = scenes.cube10()
    params = g.default_params(stop_mode=1, rel_tol=1e-9, max_lbfgs_iters=20000, lbfgs_history=history)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-9, max_lbfgs_iters=20000, lbfgs_history=history)
    ts = scenes.build_timestep(scene, precision="fp64", stepper="lbfgs", params=params)
    ot = oscenes.build_oracle(scene)
    for _ in range(2):
        ts.step()
        st = ts.stats()
        ot.prepare_step()
        _, sto = ot.compute_step("lbfgs", op)
        ot.step_next()
        assert st["converged"] == 1 and sto["converged"] == 1
        assert abs(st["newton_iters"] - sto["newton_iters"]) <= max(5, 0.1 * sto["newton_iters"])
    assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-6


@pytest.mark.parametrize("stepper", ["newton", "pd"])
def test_pipelined_pcg_in_mixed_steppers(stepper):
    """Mixed-precision Newton (3x3 blocks) and PD (the Kronecker form) with inexact inner solves (forcing
    eta in [0.05, 0.1]) and pipelined PCG (4) reach the state of Chronopoulos-Gear PCG (2) to 1e-5
    relative, both converged at every step, with the same iteration counts up to 2%."""
    scene = scenes.cube10()
    outs, iters = [], []
    for pers in (2, 4):
        params = g.default_params(stop_mode=1, rel_tol=1e-6, max_lbfgs_iters=20000, precond=2, pcg_persistent=pers,
                                  cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2)
        ts = scenes.build_timestep(scene, precision="mixed", stepper=stepper, params=params)
        it = 0
        for _ in range(3):
            ts.step()
            st = ts.stats()
            assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"], (pers, st)
            it += st["cg_iters_total"]
        outs.append(ts.get("deformation"))
        iters.append(it)
    assert rel(outs[1], outs[0]) <= 1e-5
    assert abs(iters[1] - iters[0]) <= 0.02 * iters[0] + 2


def test_pd_partly_fixed_vertices_fall_back_to_blocks():
    """The PD matrix is read as (scalar) (x) I3 when every block allows; a vertex fixed in z only breaks that
    and the solve falls back to the 3x3 blocks.  Both forms land on the oracle's PD trajectory."""
    from oracle import pyoracle

    scene = scenes.cube10()
    params = g.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-11, max_lbfgs_iters=20000, precond=2,
                              stop_floor=0.0)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-9, max_lbfgs_iters=20000, stop_floor=0.0)
    for partial in (False, True):
        ts = scenes.build_timestep(scene, precision="fp64", stepper="none", params=params)
        ot = oscenes.build_oracle(scene)
        if partial:  # the bottom face may slide in x and y
            X = scene["X"]
            t = ts.dof_type().copy()
            t[np.where(X[:, 2] == 0.0)[0], 2] = 1
            ts.set_dof_type(t)
            ot.set_dof_type(t)
        ts.reset("pd")
        ot.reset()
        for _ in range(2):
            ts.step()
            st = ts.stats()
            ot.prepare_step()
            _, sto = ot.compute_step("pd", op)
            ot.step_next()
            assert st["converged"] == 1 and sto["converged"] == 1
        assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-6, partial


def test_pd_matrix_matches_oracle():
    """The PD stepper's matrix (mass + dt^2 kappa Laplacian, DBC identity) through a PCG solve: the PD
    preconditioner applied to a vector equals the oracle's solve with its PD matrix."""
    from oracle import pyoracle

    scene = scenes.cube10()
    ts = scenes.build_timestep(scene, precision="fp64", stepper="pd", params=g.default_params(precond=2))
    ot = oscenes.build_oracle(scene)
    A = ot.pd_matrix_values()
    assert np.all(np.isfinite(A))
    # first L-BFGS-PD iteration direction is -A^{-1} g: compare after one prepare_step at rest + gravity
    ts.prepare_step()
    ot.prepare_step()
    ts.update_energy_and_gradients()
    ot.update_energy_and_gradients()
    assert rel(ts.get("forces"), ot.get("forces")) <= FP64_RTOL


def test_lbfgs_mixed_reaches_residual():
    scene = scenes.cube10()
    params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_rtol=1e-6, max_lbfgs_iters=20000, precond=2)
    ts = scenes.build_timestep(scene, precision="mixed", stepper="pd", params=params)
    for _ in range(3):
        ts.step()
        st = ts.stats()
        assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"]


def test_lbfgs_mixed_leaves_a_stalled_fp32_phase():
    """Mixed L-BFGS with a target (1e-8 |g0|) below what FP32 element arithmetic resolves and the FP32 phase
    allowed down to the target itself (elem32_switch = 1): the phase ends once its residual stops falling
    near the target (the best |g|, within 1e3 times the target, not halved in max(100, 3 x the phase's
    longest halving interval) iterations), FP64 evaluations finish, every step converges (the
    relative target or the absolute floor stop_floor, whichever is larger) in far fewer than the iteration
    cap, and the state matches the all-FP64-evaluation run's."""
    scene = scenes.cube10()
    states = []
    for e32 in (1, 0):
        params = g.default_params(stop_mode=1, rel_tol=1e-8, max_lbfgs_iters=20000, mixed_elem32=e32,
                                  elem32_switch=1.0)
        ts = scenes.build_timestep(scene, precision="mixed", stepper="lbfgs", params=params)
        for _ in range(2):
            ts.step()
            st = ts.stats()
            assert st["converged"] == 1 and st["grad_norm"] <= 1e-7 * st["grad_norm0"], (e32, st)
            assert st["newton_iters"] < 5000, (e32, st)
        states.append(ts.get("deformation"))
    assert rel(states[0], states[1]) <= 1e-6


def test_forward_euler_matches_oracle():
    """time_step_solver_forward_euler (time_step.hpp:717-736) restated: one explicit update per step."""
    from oracle import pyoracle

    scene = scenes.cube10()
    ts = scenes.build_timestep(scene, precision="fp64", stepper="forward_euler")
    ot = oscenes.build_oracle(scene)
    for _ in range(3):
        ts.prepare_step()
        r = ts.compute_step()
        ts.step_next()
        ot.prepare_step()
        ro, _ = ot.compute_step("forward_euler", pyoracle.default_params())
        ot.step_next()
        assert abs(r - ro) <= 1e-9 * abs(ro)
    assert rel(ts.get("deformation"), ot.get("deformation")) <= FP64_RTOL


def test_h0_stepper_fp64():
    """time_step_solver_h0 (projective_dynamics.hpp:100-150): L-BFGS preconditioned by the projected
    Hessian at the start of the step; converged state equals the oracle's."""
    from oracle import pyoracle

    scene = scenes.cube10()
    params = g.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-11, max_lbfgs_iters=5000, precond=2)
    ts = scenes.build_timestep(scene, precision="fp64", stepper="h0", params=params)
    ot = oscenes.build_oracle(scene)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-9, max_lbfgs_iters=5000)
    for _ in range(3):
        ts.prepare_step()
        ts.compute_step()
        st = ts.stats()
        ts.step_next()
        ot.prepare_step()
        _, sto = ot.compute_step("h0", op)
        ot.step_next()
        assert st["converged"] == 1 and sto["converged"] == 1
    assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-6


def _pcg_case(precision):
    X, T = mesh.kuhn_box((12, 10, 9), (1.2, 1.0, 0.9))
    X = mesh.jitter_interior(X, 0.01, 21)
    ts, _ = _pair(X, T, E=1e5, nu=0.45, rho=1000.0, precision=precision)
    ts.set_params(precond=2)
    u = np.random.default_rng(3).uniform(-1, 1, X.shape) * 0.05
    ts.set("next_deform", u)
    ts.update_hessian(False, True, True)
    b = np.random.default_rng(4).normal(size=X.shape)
    return ts, b


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_persistent_pcg_bitwise_equals_two_launch(precision):
    """Standard PCG in one cooperative launch (grid barriers; the last block to arrive runs the two-launch
    path's reductions and epilogues) reproduces the two-launch loop bit for bit, also under an iteration cap."""
    ts, b = _pcg_case(precision)
    ts.set_params(pcg_persistent=0)
    x0, it0, rr0 = ts.pcg(b, rtol=1e-6, max_iters=5000)
    xc0, itc0, _ = ts.pcg(b, rtol=1e-12, max_iters=7)
    ts.set_params(pcg_persistent=1)
    x1, it1, rr1 = ts.pcg(b, rtol=1e-6, max_iters=5000)
    xc1, itc1, _ = ts.pcg(b, rtol=1e-12, max_iters=7)
    assert it0 == it1 and it0 > 10 and rr0 == rr1 and np.array_equal(x0, x1)
    assert itc0 == itc1 == 7 and np.array_equal(xc0, xc1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("variant", [2, 4])
def test_one_reduction_pcg_matches_two_launch(precision, variant):
    """Chronopoulos-Gear PCG (2) and pipelined PCG (4) in one launch give the two-launch PCG's iterates up
    to rounding: iteration counts within 2, both true residuals at the tolerance, the solutions close; an
    iteration cap stops both at the same iterate up to rounding.  Pipelined PCG in FP32 is checked at a
    1e-3 tolerance (its extra FP32 recurrences stall the residual near 1e-4 on this system)."""
    ts, b = _pcg_case(precision)
    tol = 1e-3 if (variant == 4 and precision == "mixed") else 1e-6
    ts.set_params(pcg_persistent=0)
    x0, it0, rr0 = ts.pcg(b, rtol=tol, max_iters=5000)
    ts.set_params(pcg_persistent=variant)
    x1, it1, rr1 = ts.pcg(b, rtol=tol, max_iters=5000)
    assert it0 > 10 and abs(it0 - it1) <= 2
    bn = np.linalg.norm(b)
    for x in (x0, x1):
        assert np.linalg.norm(b - ts.spmv(x)) <= 1.5 * tol * bn
    # the same iterate up to rounding: FP64 close, FP32 within the tolerance's own scale
    assert rel(x1, x0) <= (1e-9 if precision == "fp64" else max(1e-4, tol))
    ts.set_params(pcg_persistent=0)
    xc0, itc0, _ = ts.pcg(b, rtol=1e-12, max_iters=7)
    ts.set_params(pcg_persistent=variant)
    xc1, itc1, _ = ts.pcg(b, rtol=1e-12, max_iters=7)
    assert itc0 == itc1 == 7
    assert rel(xc1, xc0) <= (1e-12 if precision == "fp64" else 1e-5)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pipelined_pcg_switches_to_chronopoulos_gear(precision):
    """After pcg_pipe_iters iterations the pipelined kernel continues as Chronopoulos-Gear PCG from the same
    state: with the switch at 0 it follows variant 2 (same iteration count, same solution up to rounding);
    with the switch at 10 a tight FP32 solve, where pure pipelined PCG stalls, converges like variant 2,
    its true residual within the gap the 10 pipelined FP32 iterations left (1.6e-5 measured)."""
    ts, b = _pcg_case(precision)
    bn = np.linalg.norm(b)
    ts.set_params(pcg_persistent=2)
    x2, it2, _ = ts.pcg(b, rtol=1e-6, max_iters=5000)
    ts.set_params(pcg_persistent=4, pcg_pipe_iters=0)
    x0, it0, _ = ts.pcg(b, rtol=1e-6, max_iters=5000)
    assert it0 == it2 and rel(x0, x2) <= (1e-12 if precision == "fp64" else 1e-5)
    ts.set_params(pcg_persistent=4, pcg_pipe_iters=10)
    x10, it10, _ = ts.pcg(b, rtol=1e-6, max_iters=5000)
    assert abs(it10 - it2) <= 2
    assert np.linalg.norm(b - ts.spmv(x10)) <= (2e-6 if precision == "fp64" else 5e-5) * bn


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("variant", [1, 2, 4])
def test_persistent_pcg_independent_of_grid(precision, variant):
    """Partial sums are formed per 256-row virtual block and added in a fixed order by whichever block
    arrives last, so the result is bitwise the same whether each block owns one virtual block or several."""
    ts, b = _pcg_case(precision)
    outs = []
    for mb in (0, 3, 1):
        ts.set_params(pcg_persistent=variant, pcg_max_blocks=mb)
        outs.append(ts.pcg(b, rtol=1e-6, max_iters=5000))
    for x, it, rr in outs[1:]:
        assert it == outs[0][1] and rr == outs[0][2] and np.array_equal(x, outs[0][0])


def test_persistent_newton_steps_match_two_launch():
    scene = scenes.cube10()
    outs = []
    for pers in (0, 1, 2):
        ts = scenes.build_timestep(scene, precision="mixed",
                                   params=g.default_params(stop_mode=1, rel_tol=1e-6, pcg_persistent=pers))
        for _ in range(2):
            ts.step()
            st = ts.stats()
            assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"]
        outs.append(ts.get("deformation"))
    assert np.array_equal(outs[1], outs[0])
    assert rel(outs[2], outs[0]) <= 1e-5


def test_grid_barrier_wait_gives_up_and_context_survives():
    """A barrier told to wait for one block more than the grid has (a flag nothing sets) gives up after
    pcg_spin_limit polls: the call fails with DeviceTimeout, and the next solve on the same handle works."""
    X, T = mesh.kuhn_box((6, 5, 4), (1.2, 1.0, 0.8))
    ts, _ = _pair(X, T, E=1e5, nu=0.45, rho=1000.0)
    u = np.random.default_rng(7).uniform(-1, 1, X.shape) * 0.05
    ts.set("next_deform", u)
    ts.update_hessian(False, True, True)
    b = np.random.default_rng(8).normal(size=X.shape)
    for variant in (1, 2, 4):
        ts.set_params(pcg_persistent=variant)
        ref, it_ref, _ = ts.pcg(b, rtol=1e-10, max_iters=5000)
        ts.set_params(pcg_barrier_extra=1, pcg_spin_limit=2000)
        with pytest.raises(g.DeviceTimeout):
            ts.pcg(b, rtol=1e-10, max_iters=5000)
        ts.set_params(pcg_barrier_extra=0, pcg_spin_limit=0)
        x, it, _ = ts.pcg(b, rtol=1e-10, max_iters=5000)
        assert it == it_ref and np.array_equal(x, ref)


def _ncg_pair(precision="fp64"):
    X, T = mesh.kuhn_box((5, 5, 5))
    ts, ot = _pair(X, T, dt=1e-2, E=1e5, nu=0.45, rho=1000.0, precision=precision)
    fixed = np.where(X[:, 2] == 1.0)[0]
    ts.mark_dirichlet_batched(fixed, np.zeros((fixed.size, 3)))
    ot.mark_dirichlet(fixed)
    for t in (ts, ot):
        t.add_gravity((0.0, 0.0, -9.8))
    return X, ts, ot


def _jacobi_factor(ts):
    """L = diag(H_ii^-1/2) on the CSR pattern: L L^T is the Jacobi preconditioner of the current Hessian."""
    ts.prepare_step()
    ts.update_hessian(False, True, True)
    rp, ci = ts.csr_pattern()
    vals = ts.values("sysmatrix")
    L = np.zeros_like(vals)
    rows = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    diag = ci == rows
    L[diag] = 1.0 / np.sqrt(vals[diag])
    return L


@pytest.mark.parametrize("method", ["ncg", "ncg_ext"])
def test_ncg_fp64_matches_oracle(method):
    """Nonlinear CG (Dai-Kou direction, backtracking with parabola fits) on the GPU follows the FP64 oracle's
    iteration: after a fixed number of iterations the states agree to 1e-9 (the two only differ in the
    order of their dot-product sums).  Over more iterations rounding differences grow (perturbing L by
    1e-10 moves the oracle's own count between 34 and 133 iterations on this scene, and unpreconditioned
    NCG between 60 and >1000), so only the preconditioned variant is also run to 1e-6 relative residual,
    where both must converge to the same minimiser.  L is a Jacobi factor set through the API."""
    from oracle import pyoracle

    cases = ((12, 1e-14), (1000, 1e-6)) if method == "ncg_ext" else ((12, 1e-14),)
    for max_it, rel_tol in cases:
        X, ts, ot = _ncg_pair()
        ts.set_params(g.default_params(stop_mode=1, rel_tol=rel_tol, ncg_max_iters=max_it))
        op = pyoracle.default_params(stop_mode=1, rel_tol=rel_tol, ncg_max_iters=max_it)
        ts.reset(method)
        ot.reset()
        if method == "ncg_ext":
            L = _jacobi_factor(ts)
            ts.set_ncg_matrix(L)
            ot.set_ncg_matrix(L)
        ts.prepare_step()
        ts.compute_step()
        st = ts.stats()
        ot.prepare_step()
        _, sto = ot.compute_step(method, op)
        if max_it == 12:
            assert st["newton_iters"] == sto["newton_iters"] == 12
            assert rel(ts.get("next_deform"), ot.get("next_deform")) <= 1e-9
            assert abs(st["energy"] - sto["energy"]) <= 1e-9 * abs(sto["energy"])
        else:
            assert st["converged"] == 1 and sto["converged"] == 1
            assert rel(ts.get("next_deform"), ot.get("next_deform")) <= 1e-4


def test_ncg_preconditioner_reset_and_mixed():
    """reset() restores L = I; the mixed-precision NCG reaches the residual target."""
    X, ts, _ = _ncg_pair(precision="mixed")
    ts.set_params(stop_mode=1, rel_tol=1e-6)
    ts.reset("ncg_ext")
    L = _jacobi_factor(ts)
    ts.set_ncg_matrix(L)
    ts.compute_step()
    st_prec = ts.stats()
    assert st_prec["converged"] == 1 and st_prec["grad_norm"] <= 1e-6 * st_prec["grad_norm0"]
    with pytest.raises(ValueError):
        ts.set_ncg_matrix(L[:-1])
    from ssim_gb300.libssim import fem

    s = fem.tet_ncg_cuda_ext_ai(X, ts.cells(), 1e-2, 1e5, 0.45, 1000.0)
    s.reset()
    s.set_matrix(L)
    with pytest.raises(TypeError):
        s.set_matrix(L.astype(np.float32))


def test_pd_per_element_diffusivity():
    """pd_kappa_mode 2 builds the PD matrix from each element's own Lame parameters: with a per-element E
    field (1e4..1e6) it matches the oracle's mode-2 stepper and converges within 400 L-BFGS iterations, where
    the reference's uniform diffusivity (mode 0) ends the same budget with a larger residual."""
    from oracle import pyoracle

    scene = dict(scenes.cube10())
    scene["E_cells"] = 10.0 ** mesh.uniform(9, scene["cells"].shape[0], 4.0, 6.0)
    res = {}
    for mode in (0, 2):
        params = g.default_params(stop_mode=1, rel_tol=1e-8, cg_rtol=1e-11, max_lbfgs_iters=400, precond=2,
                                  pd_kappa_mode=mode)
        ts = scenes.build_timestep(scene, precision="fp64", stepper="pd", params=params)
        ts.step()
        st = ts.stats()
        res[mode] = (st["converged"], st["newton_iters"], st["grad_norm"] / st["grad_norm0"])
        if mode == 2:
            assert st["converged"] == 1, st
            ot = oscenes.build_oracle(scene)
            ot.set_pd_diffusivity_mode(2)
            ot.prepare_step()
            _, sto = ot.compute_step("pd", pyoracle.default_params(stop_mode=1, rel_tol=1e-8, max_lbfgs_iters=400))
            ot.step_next()
            assert sto["converged"] == 1
            assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-6
    assert res[0][0] == 0 or res[0][1] > res[2][1], res


@pytest.mark.parametrize("scene_name", ["cube10", "bar", "sheet2d"])
def test_mixed_fp32_elements_confirmed_in_fp64(scene_name):
    """Mixed Newton with FP32 element arithmetic in its inner iterations (small-strain forms) and an FP64
    confirmation of the stopping test: every step ends with an FP64 residual <= 1e-6 |g0| (the stats report
    the FP64 evaluation), and the state matches the all-FP64-evaluation mixed run and the FP64 oracle."""
    from oracle import pyoracle

    scene = {"cube10": scenes.cube10, "bar": lambda: scenes.bar(20, 6, 6),
             "sheet2d": lambda: scenes.sheet2d(33, 17)}[scene_name]()
    states = []
    for e32 in (1, 0):
        params = g.default_params(stop_mode=1, rel_tol=1e-6, mixed_elem32=e32)
        ts = scenes.build_timestep(scene, precision="mixed", params=params)
        for _ in range(4):
            ts.prepare_step()
            ts.compute_step()
            st = ts.stats()
            assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"], st
            # the reported residual is the FP64 one: re-evaluating in FP64 gives the same norm
            ts.update_energy_and_gradients()
            assert abs(np.linalg.norm(ts.get("forces")) - st["grad_norm"]) <= 1e-9 * st["grad_norm0"]
            ts.step_next()
        states.append(ts.get("deformation"))
    ot = oscenes.build_oracle(scene)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-12)
    for _ in range(4):
        ot.prepare_step()
        ot.compute_step("newton", op)
        ot.step_next()
    uo = ot.get("deformation")
    assert rel(states[0], uo) <= 1e-4 and rel(states[1], uo) <= 1e-4
    # the FP32 pass did run: its iterates differ from the all-FP64-evaluation run's (within the tolerance)
    assert not np.array_equal(states[0], states[1])


def test_two_handles_step_concurrently_from_threads():
    """One handle per stream, several handles at once: two handles stepped from two host threads at the same
    time give bitwise the states of the same handles stepped one after the other."""
    import threading

    scene = scenes.cube10()
    params = g.default_params(stop_mode=1, rel_tol=1e-8)

    def run(ts, out, k):
        for _ in range(4):
            ts.step()
        out[k] = ts.get("deformation")

    seq = {}
    for k, prec in enumerate(("mixed", "fp64")):
        run(scenes.build_timestep(scene, precision=prec, params=params), seq, k)
    handles = [scenes.build_timestep(scene, precision=prec, params=params) for prec in ("mixed", "fp64")]
    par = {}
    threads = [threading.Thread(target=run, args=(handles[k], par, k)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for k in range(2):
        assert np.array_equal(par[k], seq[k])


def test_reference_harness_scene_step_by_step():
    """The reference's own time-step harness (tests/fem_time_step/main.cpp:39-86: unit_box(24, 6, 6) x 4 in x,
    x = 0 face fixed, gravity on y, rho 10, threshold 1e-3 under the reference's absolute rule) with the
    default Newton settings: the same Newton iteration count every step as the oracle (its loose threshold
    often accepts the inertial prediction), and the same states to the PCG tolerance."""
    from oracle import pyoracle

    sc = scenes.reference_beam()
    ts = scenes.build_timestep(sc, precision="fp64", stepper="newton", params=g.default_params(), rtol=sc["rtol"])
    ot = oscenes.build_oracle(sc, rtol=sc["rtol"])
    op = pyoracle.default_params()
    iters, iters_o = [], []
    for _ in range(20):
        ts.step()
        iters.append(ts.stats()["newton_iters"])
        ot.prepare_step()
        _, sto = ot.compute_step("newton", op)
        ot.step_next()
        iters_o.append(sto["newton_iters"])
    assert iters == iters_o
    assert rel(ts.get("deformation"), ot.get("deformation")) <= 1e-6
