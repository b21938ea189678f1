"""The FP16 copy of the Jacobi-scaled system matrix (pcg_half_matrix = 1): the mixed Newton's loose PCG
solves run on K~ = S K S (S = diag(K)^-1/2) stored in FP16, both triangles, full block SELL-32.

Checked, against the FP64 oracle's matrix and the FP32 symmetric values on the same state:
* the copy applied in the unscaled space (ssim_gb_spmv, SSIM_GB_SYSMATRIX_HALF) equals K x within the FP16
  rounding of the scaled values: 2e-3 of max|K x| (a scaled value carries 2^-11 relative rounding; a row
  sums about 15 blocks of mixed sign);
* a PCG solve to 5e-2 on the copy leaves a TRUE residual |b - K x| / |b| within the requested tolerance
  plus the copy's rounding (5e-2 + 5e-3) and takes the FP32 path's iteration count within 10% + 2; a solve
  tighter than half_matrix_min_rtol runs on the FP32 values (bitwise the FP32 path's result);
* Newton steps with the copy converge like the FP32 matrix's (the same stopping test on FP64 residuals):
  states within 1e-5, Newton iterations per step within 1, total PCG iterations within 15%;
* the FP16 element blocks of those assemblies (half_hessian_blocks): values within 1e-3 of max|K| of the
  FP32-block assembly at the same state, and Newton steps as above.
"""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import mesh, scenes

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _pair(half):
    from oracle import pyoracle

    X, T = mesh.kuhn_box((12, 6, 5), (1.2, 0.6, 0.5))
    X = mesh.jitter_interior(X, 0.01, 11)
    E = 10.0 ** mesh.uniform(12, T.shape[0], 4.0, 6.0)
    fixed = np.where(X[:, 0] == 0.0)[0]
    ts = g.TimeStep(X, T, 1e-2, 1e5, 0.45, 1000.0)
    ts.set_material(E, None)
    ts.mark_dirichlet_batched(fixed, np.zeros((fixed.size, 3)))
    ts.set_precision("mixed")
    ts.set_params(g.default_params(precond=2, pcg_half_matrix=half, cg_max_iters=20000))
    ts.reset("newton")
    ot = pyoracle.OracleTimeStep(X, T, 1e-2, 1e5, 0.45, 1000.0)
    ot.set_material(E, None)
    ot.mark_dirichlet(fixed)
    ot.reset()
    u = np.random.default_rng(13).uniform(-1, 1, X.shape) * 0.02
    for t in (ts, ot):
        t.set("next_deform", u)
        t.update_hessian(False, True, True)
    return ts, ot, X


def test_half_spmv_matches_matrix():
    ts, ot, X = _pair(1)
    for seed in (14, 15):
        x = np.random.default_rng(seed).normal(size=X.shape)
        y64 = ot.spmv(x).reshape(-1, 3)
        y32 = ts.spmv(x)
        yh = ts.spmv(x, "sysmatrix_half")
        assert rel(y32, y64) <= 1e-5
        assert rel(yh, y64) <= 2e-3, rel(yh, y64)
        assert rel(yh, y32) <= 2e-3
    # FP64 handles have no FP16 copy
    ts64 = g.TimeStep(*mesh.kuhn_box((3, 2, 2), (0.3, 0.2, 0.2)), 1e-2, 1e5, 0.45, 1000.0)
    ts64.reset("newton")
    with pytest.raises(ValueError, match="mixed precision only"):
        ts64.spmv(np.zeros((ts64.num_vertices, 3)), "sysmatrix_half")


def test_half_pcg_true_residual_and_iterations():
    ts_h, ot, X = _pair(1)
    ts_f, _, _ = _pair(0)
    b = np.random.default_rng(16).normal(size=X.shape)
    nb = np.linalg.norm(b)
    xh, ith, rrh = ts_h.pcg(b, rtol=5e-2)
    xf, itf, rrf = ts_f.pcg(b, rtol=5e-2)
    true_h = np.linalg.norm(b.reshape(-1) - ot.spmv(xh)) / nb
    true_f = np.linalg.norm(b.reshape(-1) - ot.spmv(xf)) / nb
    assert rrh <= 5e-2 and rrf <= 5e-2
    assert true_f <= 5e-2 + 1e-4, true_f
    assert true_h <= 5e-2 + 5e-3, (true_h, rrh)
    assert abs(ith - itf) <= 0.1 * itf + 2, (ith, itf)
    # tighter than half_matrix_min_rtol: the FP32 values, bitwise the FP32 handle's solve
    xh2, ith2, _ = ts_h.pcg(b, rtol=1e-6)
    xf2, itf2, _ = ts_f.pcg(b, rtol=1e-6)
    assert ith2 == itf2 and np.array_equal(xh2, xf2)


@pytest.mark.parametrize("name", ["beam_small", "bar_small", "cube10"])
def test_newton_with_half_matrix(name):
    scene = {"beam_small": lambda: scenes.beam(40, 20, 14, h=0.05), "bar_small": lambda: scenes.bar(20, 6, 6),
             "cube10": scenes.cube10}[name]()
    runs = {}
    for half in (1, 0):
        params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2,
                                  precond=2, pcg_half_matrix=half)
        ts = scenes.build_timestep(scene, precision="mixed", params=params)
        newton, cg = [], 0
        for _ in range(4):
            ts.step()
            st = ts.stats()
            assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"], (half, st)
            newton.append(st["newton_iters"])
            cg += st["cg_iters_total"]
        runs[half] = (ts.get("deformation"), newton, cg)
    (uh, nh, ch), (uf, nf, cf) = runs[1], runs[0]
    assert rel(uh, uf) <= 1e-5
    assert all(abs(a - b) <= 1 for a, b in zip(nh, nf)), (nh, nf)
    assert abs(ch - cf) <= 0.15 * cf, (ch, cf)


def _one_newton_iteration(scene, half_blocks):
    params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2, precond=2,
                              pcg_half_matrix=1, half_hessian_blocks=half_blocks, max_newton_iters=1)
    ts = scenes.build_timestep(scene, precision="mixed", params=params)
    ts.prepare_step()
    ts.compute_step()
    return ts


def test_half_hessian_blocks_assembly():
    """half_hessian_blocks = 1: the element blocks of a loose-solve assembly are written in FP16 with a
    power-of-two scale per block and summed in FP32.  The first Newton iteration of the same step on two
    handles assembles at the same state: the FP16-block values differ from the FP32-block values (the FP16
    path ran) by at most 1e-3 of max|K| (a block's values carry 2^-11 of the block's largest magnitude; a
    slot sums up to ~20 of them)."""
    scene = scenes.bar(20, 6, 6)
    k16 = _one_newton_iteration(scene, 1).values("sysmatrix")
    k32 = _one_newton_iteration(scene, 0).values("sysmatrix")
    assert not np.array_equal(k16, k32)
    assert rel(k16, k32) <= 1e-3, rel(k16, k32)


@pytest.mark.parametrize("name", ["beam_small", "bar_small"])
def test_newton_with_half_hessian_blocks(name):
    scene = {"beam_small": lambda: scenes.beam(40, 20, 14, h=0.05), "bar_small": lambda: scenes.bar(20, 6, 6)}[name]()
    runs = {}
    for hb in (1, 0):
        params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2,
                                  precond=2, pcg_half_matrix=1, half_hessian_blocks=hb)
        ts = scenes.build_timestep(scene, precision="mixed", params=params)
        newton, cg = [], 0
        for _ in range(4):
            ts.step()
            st = ts.stats()
            assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"], (hb, st)
            newton.append(st["newton_iters"])
            cg += st["cg_iters_total"]
        runs[hb] = (ts.get("deformation"), newton, cg)
    (u1, n1, c1), (u0, n0, c0) = runs[1], runs[0]
    assert rel(u1, u0) <= 1e-5
    assert all(abs(a - b) <= 1 for a, b in zip(n1, n0)), (n1, n0)
    assert abs(c1 - c0) <= 0.15 * c0, (c1, c0)


def test_half_solves_reported_and_checked():
    """Every Newton solve on the copy is followed by its true residual on the FP32 values (fused with g . d):
    on a well-conditioned beam every step's solves stay on the copy (half_solves = Newton iterations) and the
    checked ratio |g + K d| / (eta |g|) stays near 1."""
    scene = scenes.beam(40, 20, 14, h=0.05)
    params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2, precond=2)
    ts = scenes.build_timestep(scene, precision="mixed", params=params)
    for _ in range(3):
        ts.step()
        st = ts.stats()
        assert st["converged"] == 1 and st["half_solves"] == st["newton_iters"], st
        assert 0.5 < st["half_check"] <= 1.2, st


def test_half_fallback_to_fp32_values():
    """A check that fails (here forced by half_check_slack = 0.5: no solve that stops at its forcing has a true
    residual below half of it) turns the copy off for the handle: one solve on the copy, then the FP32 values,
    the same converged trajectory as a handle that never used the copy; reset() turns it on again."""
    scene = scenes.bar(20, 6, 6)
    base = dict(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2, precond=2)
    ts = scenes.build_timestep(scene, precision="mixed", params=g.default_params(half_check_slack=0.5, **base))
    ref = scenes.build_timestep(scene, precision="mixed", params=g.default_params(pcg_half_matrix=0, **base))
    halves = []
    for _ in range(3):
        ts.step()
        ref.step()
        st = ts.stats()
        assert st["converged"] == 1 and ref.stats()["converged"] == 1
        halves.append(st["half_solves"])
    assert halves == [1, 0, 0], halves
    assert rel(ts.get("deformation"), ref.get("deformation")) <= 1e-5
    ts.reset("newton")
    ts.step()
    assert ts.stats()["half_solves"] == 1


@pytest.mark.parametrize("pipelined", [3, 4])
def test_pipelined_pcg_on_half_matrix(pipelined):
    """pcg_persistent = 3 (automatic, the default) or 4 with the FP16 copy: the pipelined iteration (one
    reducing barrier per iteration) in the copy's scaled space.  Newton steps converge like the
    Chronopoulos-Gear solves on the copy (variant 2): states within 1e-5, Newton iterations per step within 1,
    every solve on the copy."""
    scene = scenes.beam(40, 20, 14, h=0.05)
    runs = {}
    for variant in (pipelined, 2):
        params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2,
                                  precond=2, pcg_persistent=variant)
        ts = scenes.build_timestep(scene, precision="mixed", params=params)
        newton = []
        for _ in range(3):
            ts.step()
            st = ts.stats()
            assert st["converged"] == 1 and st["half_solves"] == st["newton_iters"], (variant, st)
            newton.append(st["newton_iters"])
        runs[variant] = (ts.get("deformation"), newton)
    assert rel(runs[pipelined][0], runs[2][0]) <= 1e-5
    assert all(abs(a - b) <= 1 for a, b in zip(runs[pipelined][1], runs[2][1])), runs
