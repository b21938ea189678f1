"""The slice preconditioner (precond 3): per 32-row slice, the block LDL^T factorisation of the slice's
block-tridiagonal part (couplings of vertex u with u - 1 and u + 1), applied as a forward / backward
substitution inside the warp that owns the slice.  Checked against the oracle's restatement of the same
preconditioner (oracle.cpp pcg, precond 3), across the PCG variants, in Newton trajectories and in the H0
stepper, and for the iteration reduction it is there for.
"""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import mesh, scenes
from oracle import scenes as oscenes

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _system(name, precision="fp64"):
    from oracle import pyoracle

    if name == "kuhn_jitter":
        X, T = mesh.kuhn_box((12, 10, 9), (1.2, 1.0, 0.9))
        X = mesh.jitter_interior(X, 0.01, 21)
        E = None
    elif name == "unit_box7":
        X, T = mesh.unit_box(7, 7, 7)
        E = None
    else:  # a beam with the benchmark's column length (34 cells, 35 vertices) and per-cell E
        X, T = mesh.kuhn_box((20, 10, 34), (0.4, 0.2, 0.68))
        E = 10.0 ** mesh.uniform(3, T.shape[0], 4.0, 6.0)
    ts = g.TimeStep(X, T, 1e-2, 1e5, 0.45, 1000.0)
    ts.set_precision(precision)
    ot = pyoracle.OracleTimeStep(X, T, 1e-2, 1e5, 0.45, 1000.0)
    if E is not None:
        ts.set_material(E, None)
        ot.set_material(E, None)
    fixed = np.where(X[:, 0] == 0.0)[0]
    ts.mark_dirichlet_batched(fixed, np.zeros((fixed.size, 3)))
    ot.mark_dirichlet(fixed)
    ts.set_params(precond=3)
    ts.reset("none")
    ot.reset()
    u = np.random.default_rng(3).uniform(-1, 1, X.shape) * 0.02
    for t in (ts, ot):
        t.set("next_deform", u)
        t.update_hessian(False, True, True)
    b = np.random.default_rng(4).normal(size=X.shape)
    b[fixed] = 0.0
    return ts, ot, b


@pytest.mark.parametrize("name", ["kuhn_jitter", "unit_box7", "beam_columns35"])
def test_slice_pcg_matches_oracle(name):
    ts, ot, b = _system(name)
    for variant in (0, 1, 2):
        ts.set_params(precond=3, pcg_persistent=variant)
        xs, it, rr = ts.pcg(b, rtol=1e-12, max_iters=5000)
        xo, ito, rro = ot.pcg(b, rtol=1e-12, max_iters=5000, precond=3)
        assert abs(it - ito) <= 1, (variant, it, ito)
        assert rr <= 1e-12 and rro <= 1e-12
        assert rel(xs, xo.reshape(-1, 3)) <= 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_slice_pcg_variants(precision):
    """With precond 3: the standard persistent PCG is bitwise the two-launch loop; Chronopoulos-Gear agrees
    up to rounding; the pipelined variant runs as Chronopoulos-Gear (bitwise); results do not depend on the
    persistent grid's size."""
    ts, _, b = _system("kuhn_jitter", precision)
    runs = {}
    for variant in (0, 1, 2, 4):
        ts.set_params(precond=3, pcg_persistent=variant)
        runs[variant] = ts.pcg(b, rtol=1e-6, max_iters=5000)
    x0, it0, rr0 = runs[0]
    x1, it1, rr1 = runs[1]
    assert it0 == it1 and rr0 == rr1 and np.array_equal(x0, x1)
    x2, it2, _ = runs[2]
    assert abs(it2 - it0) <= 2 and rel(x2, x0) <= (1e-9 if precision == "fp64" else 1e-4)
    x4, it4, _ = runs[4]
    assert it4 == it2 and np.array_equal(x4, x2)
    for variant in (1, 2):
        outs = []
        for mb in (0, 3, 1):
            ts.set_params(precond=3, pcg_persistent=variant, pcg_max_blocks=mb)
            outs.append(ts.pcg(b, rtol=1e-6, max_iters=5000))
        for x, it, rr in outs[1:]:
            assert it == outs[0][1] and rr == outs[0][2] and np.array_equal(x, outs[0][0])


def test_slice_preconditioner_cuts_iterations():
    """On the beam with 35-vertex columns the slice solve covers most of each column's coupling: fewer PCG
    iterations than block-Jacobi at the Newton solver's forcing tolerances."""
    ts, _, b = _system("beam_columns35", "mixed")
    its = {}
    for pc in (2, 3):
        ts.set_params(precond=pc)
        ts.update_hessian(False, True, True)
        its[pc] = [ts.pcg(b, rtol=tol, max_iters=5000)[1] for tol in (1e-1, 5e-2, 1e-2)]
    assert all(a < b_ for a, b_ in zip(its[3], its[2])), its


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_slice_newton_matches_oracle(precision):
    from oracle import pyoracle

    scene = scenes.cube10()
    if precision == "fp64":
        params = g.default_params(stop_mode=1, rel_tol=1e-9, cg_rtol=1e-12, cg_max_iters=20000, precond=3)
    else:
        params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2,
                                  precond=3)
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-9 if precision == "fp64" else 1e-10, cg_rtol=1e-12,
                                 cg_max_iters=20000, precond=3)
    ts = scenes.build_timestep(scene, precision=precision, params=params)
    ot = oscenes.build_oracle(scene)
    for _ in range(5):
        ts.step()
        st = ts.stats()
        assert st["converged"] == 1
        ot.prepare_step()
        _, sto = ot.compute_step("newton", op)
        ot.step_next()
        assert sto["converged"] == 1
    assert rel(ts.get("deformation"), ot.get("deformation")) <= (FP64_RTOL if precision == "fp64" else 1e-5)


def test_slice_preconditioner_in_h0_stepper():
    """The H0 stepper applies the step-start Hessian by PCG with its preconditioner: with precond 3 the
    slice factors travel with the copied matrix; two steps reach the tolerance."""
    scene = scenes.cube10()
    ts = scenes.build_timestep(scene, precision="fp64", stepper="h0",
                               params=g.default_params(stop_mode=1, rel_tol=1e-6, precond=3,
                                                       max_lbfgs_iters=5000))
    for _ in range(2):
        ts.step()
        st = ts.stats()
        assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"], st
