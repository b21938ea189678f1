"""Batched instances: a disjoint union of cubes stepped by one GPU time-step object, each instance against
the oracle stepping it alone."""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import scenes
from oracle import scenes as oscenes

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_batch_matches_instances_fp64():
    from oracle import pyoracle

    batch = scenes.batch_cubes(n=5, kmin=2, kmax=4, seed=14)
    params = g.default_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-12, cg_max_iters=20000, precond=2,
                              stop_floor=0.0)
    ts = scenes.build_batch_timestep(batch, precision="fp64", params=params)
    ots = [oscenes.batch_instance_oracle(batch, i) for i in range(5)]
    op = pyoracle.default_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-12, cg_max_iters=20000, precond=2,
                                 stop_floor=0.0)
    for _ in range(3):
        ts.step()
        assert ts.stats()["converged"] == 1
        gi, gi0 = ts.instance_residuals()
        assert np.all(gi <= 1e-10 * gi0)
        for ot in ots:
            ot.prepare_step()
            _, st = ot.compute_step("newton", op)
            ot.step_next()
            assert st["converged"] == 1
    u = ts.get("deformation")
    off = batch["vertex_offsets"]
    for i, ot in enumerate(ots):
        assert rel(u[off[i]:off[i + 1]], ot.get("deformation")) <= 1e-8, i


def test_batch_mixed_per_instance_residual():
    batch = scenes.batch_cubes(n=16, kmin=2, kmax=6, seed=15)
    params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-2, cg_eta_min=1e-3, precond=2)
    ts = scenes.build_batch_timestep(batch, precision="mixed", params=params)
    for _ in range(3):
        ts.step()
        assert ts.stats()["converged"] == 1
        gi, gi0 = ts.instance_residuals()
        assert np.all(gi <= 1e-6 * gi0)
    fixed = batch["fixed"]
    assert np.abs(ts.get("deformation")[fixed]).max() == 0.0
