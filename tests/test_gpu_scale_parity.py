"""GPU against the FP64 oracle at the benchmarked sizes.

For each benchmarked configuration the oracle steps the scene from its initial state with a tight solve
(Newton to 1e-10 relative residual, 1e-11 for the rollout cube, forcing eta = min(0.1, max(1e-12,
|g|/|g0|))), and the GPU steps the same scene: in plain FP64 with the same tight settings (the FP64 parity
bar: states within 1e-10 of the oracle's), and in mixed precision with the benchmark's own solver settings
(Newton to 1e-6 relative; the error against the oracle is stated and held to 1e-5).  The rollout cube
starts from a random velocity field, so its first gradient is large against the solution's scale: there
the benchmark's 1e-6 residual rule alone leaves the state about 3e-4 from the oracle's, in FP64 as in mixed
precision; for it the mixed state is held to the FP64 state of the same rule, and mixed precision solved to
1e-9 (FP64 residual, FP32 Hessian and PCG) is held to 1e-5.  Configurations:

* the 1.02M-tet beam (100 x 50 x 34 hex x 6, per-cell E, gravity), 2 steps; at its size also the energy,
  the gradient and the projected, Dirichlet-filtered Hessian values at the oracle's stepped state
  (time_step.hpp:577-658);
* the full 192,000-tet bar (80 x 20 x 20 x 6, jittered, stretched start), 3 steps;
* the 196,608-tet cube of the differentiable rollout (32^3 x 6, per-cell E, random initial velocities), 3
  steps;
* three instances with 20 or more hex cells per side taken from the 256-cube batch, stepped inside the
  whole batch (6.5M tets) as it is benchmarked, 2 steps.

Each test prints one ``SCALE_PARITY {json}`` line with the measured errors.
"""
import json

import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import scenes
from oracle import scenes as oscenes

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 1e-5
TIGHT = dict(stop_mode=1, rel_tol=1e-10, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=1e-12, cg_max_iters=20000,
             max_newton_iters=40, precond=2, stop_floor=0.0)


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def bench_settings():
    import bench

    return dict(bench.SOLVER, **bench.GPU_ONLY)


def report(name, **vals):
    print("SCALE_PARITY " + json.dumps(dict(config=name, **vals)), flush=True)


def oracle_states(scene, steps, rel_tol):
    from oracle import pyoracle

    ot = oscenes.build_oracle(scene)
    op = pyoracle.default_params(**dict(TIGHT, rel_tol=rel_tol))
    states = []
    for _ in range(steps):
        ot.prepare_step()
        _, st = ot.compute_step("newton", op)
        ot.step_next()
        assert st["converged"] == 1, st
        states.append(ot.get("deformation"))
    return ot, states


def gpu_states(scene, precision, params, steps):
    ts = scenes.build_timestep(scene, precision=precision, params=g.default_params(**params))
    states, stats = [], []
    for _ in range(steps):
        ts.step()
        stats.append(ts.stats())
        states.append(ts.get("deformation"))
    return ts, states, stats


def rollout_scene(n=32):
    sc = scenes.rollout_cube(n)
    return dict(name=sc["name"], X=sc["X"], cells=sc["cells"], dt=sc["dt"], E=1e5, nu=sc["nu"], rho=sc["rho"],
                fixed=sc["fixed"], gravity=(0.0, 0.0, 0.0), u0=None, E_cells=sc["E_cells"], velocity=sc["v0"])


# name: (scene, steps, relative residual of the tight solves)
CASES = {"beam1m": (scenes.beam, 2, 1e-10), "bar192k": (scenes.bar, 3, 1e-10),
         "rollout_cube32": (rollout_scene, 3, 1e-11)}


@pytest.fixture(scope="module")
def oracle_runs():
    return {}


def _oracle(oracle_runs, name):
    if name not in oracle_runs:
        make, steps, tol = CASES[name]
        scene = make()
        ot, states = oracle_states(scene, steps, tol)
        oracle_runs[name] = (scene, ot, states)
    return oracle_runs[name]


@pytest.mark.parametrize("name", list(CASES))
def test_fp64_matches_oracle_at_scale(oracle_runs, name):
    scene, ot, states_o = _oracle(oracle_runs, name)
    tol = CASES[name][2]
    ts, states, stats = gpu_states(scene, "fp64", dict(TIGHT, rel_tol=tol), len(states_o))
    errs = [rel(u, uo) for u, uo in zip(states, states_o)]
    report(name, precision="fp64", settings=f"tight ({tol:g})", rel_err_per_step=errs,
           newton_iters=[s["newton_iters"] for s in stats])
    for s in stats:
        assert s["converged"] == 1, s
    assert np.all(states[-1][scene["fixed"]] == 0.0)
    assert max(errs) <= FP64_RTOL, errs
    if name == "beam1m":
        # the element passes at the oracle's stepped state: energy + gradient (time_step.hpp:577-624) and the
        # SPD-projected, Dirichlet-filtered Hessian values (time_step.hpp:626-658), 23.6M nonzeros; both
        # sides start from the oracle's state, and are evaluated halfway to its inertial prediction
        for f in ("deformation", "prev_deform", "velocity"):
            ts.set(f, ot.get(f))
        u = ot.get("deformation") + 0.5 * scene["dt"] * ot.get("velocity")
        for t in (ts, ot):
            t.prepare_step()
            t.set("next_deform", u)
        e, eo = ts.update_energy_and_gradients(), ot.update_energy_and_gradients()
        g_, go = ts.get("forces"), ot.get("forces")
        # the gradient sums inertia and elastic forces that nearly cancel: held in the 2-norm, its largest
        # entry error reported beside
        ge = float(np.linalg.norm(g_ - go) / np.linalg.norm(go))
        for t in (ts, ot):
            t.update_hessian(False, True, True)
        he = rel(ts.values("sysmatrix"), ot.values("sysmatrix"))
        report(name, precision="fp64", energy_rel_err=abs(e - eo) / abs(eo), gradient_rel_err_2norm=ge,
               gradient_rel_err_max=rel(g_, go), hessian_rel_err=he)
        assert abs(e - eo) <= FP64_RTOL * abs(eo)
        assert ge <= FP64_RTOL and he <= FP64_RTOL


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_benchmark_settings_vs_oracle_at_scale(oracle_runs, name):
    scene, _, states_o = _oracle(oracle_runs, name)
    ts, states, stats = gpu_states(scene, "mixed", bench_settings(), len(states_o))
    errs = [rel(u, uo) for u, uo in zip(states, states_o)]
    report(name, precision="mixed", settings="benchmark (1e-6)", rel_err_per_step=errs,
           rel_residual=[s["grad_norm"] / s["grad_norm0"] for s in stats])
    for s in stats:
        assert s["converged"] == 1 and s["grad_norm"] <= 1e-6 * s["grad_norm0"], s
    if name != "rollout_cube32":
        assert max(errs) <= MIXED_RTOL, errs
        return
    # the stopping rule, not the precision, sets this scene's error: a 1e-6 relative residual leaves state
    # errors of several 1e-4 on this stiff rollout, and two solver paths stop at different points of that
    # band (FP64 under the same rule: 3-4e-4; mixed: up to 8.5e-4 measured), so the bound is a few times the
    # FP64 path's; mixed precision under a tighter rule pins the agreement itself
    _, states64, _ = gpu_states(scene, "fp64", bench_settings(), len(states_o))
    errs64 = [rel(u, uo) for u, uo in zip(states64, states_o)]
    _, states9, stats9 = gpu_states(scene, "mixed", dict(bench_settings(), rel_tol=1e-9), len(states_o))
    errs9 = [rel(u, uo) for u, uo in zip(states9, states_o)]
    report(name, fp64_benchmark_settings_rel_err=errs64, mixed_rel_tol_1e9_rel_err=errs9)
    for s in stats9:
        assert s["converged"] == 1, s
    assert max(errs) <= 4 * max(errs64) + MIXED_RTOL, (errs, errs64)
    assert max(errs9) <= MIXED_RTOL, errs9


def test_batch_instances_k20_in_full_batch():
    """Three instances with k >= 20 hex cells per side, stepped inside the benchmarked 256-cube batch (one
    handle, per-instance stopping), against the oracle stepping each alone."""
    from oracle import pyoracle

    batch = scenes.batch_cubes()
    big = [i for i in range(len(batch["k"])) if batch["k"][i] >= 20][:3]
    assert len(big) == 3
    steps = 2
    op = pyoracle.default_params(**TIGHT)
    ref = {}
    for i in big:
        ot = oscenes.batch_instance_oracle(batch, i)
        for _ in range(steps):
            ot.prepare_step()
            _, st = ot.compute_step("newton", op)
            ot.step_next()
            assert st["converged"] == 1, st
        ref[i] = ot.get("deformation")
    off = batch["vertex_offsets"]
    out = {}
    for precision, params in (("fp64", TIGHT), ("mixed", bench_settings())):
        ts = scenes.build_batch_timestep(batch, precision=precision, params=g.default_params(**params))
        for _ in range(steps):
            ts.step()
            assert ts.stats()["converged"] == 1
        u = ts.get("deformation")
        out[precision] = {int(i): rel(u[off[i]:off[i + 1]], ref[i]) for i in big}
        ts.close()
    report("batch256_k>=20", instances={int(i): int(batch["k"][i]) for i in big}, fp64=out["fp64"],
           mixed=out["mixed"])
    assert max(out["fp64"].values()) <= FP64_RTOL, out
    assert max(out["mixed"].values()) <= MIXED_RTOL, out
