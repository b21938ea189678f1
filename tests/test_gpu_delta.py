"""The mixed Newton's iterations after the FP32 phase as FP32 increments from the FP64 evaluation at the
switch (mixed_delta = 1, the default) against the same iterations evaluated in FP64 (mixed_delta = 0).

The increment form (elem_math.cuh snh_increment; checked on the host in tests/test_host_math.py) rounds
relative to the increment since the switch, so the forces it reports are FP64-quality: every step's
reported residual must equal a fresh FP64 evaluation of the gradient at the returned state to 1e-9 of
|g0|, the energy to 1e-10 relative, and the states of the two settings must agree to the solver tolerance.
"""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import scenes

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", ["beam_small", "bar_small", "cube10"])
def test_increment_phase_reports_fp64_residuals(name):
    scene = {"beam_small": lambda: scenes.beam(40, 20, 14, h=0.05), "bar_small": lambda: scenes.bar(20, 6, 6),
             "cube10": scenes.cube10}[name]()
    states = {}
    for delta in (1, 0):
        params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2,
                                  precond=2, mixed_delta=delta)
        ts = scenes.build_timestep(scene, precision="mixed", params=params)
        for _ in range(4):
            ts.prepare_step()
            ts.compute_step()
            st = ts.stats()
            assert st["converged"] == 1 and st["grad_norm"] <= 1e-6 * st["grad_norm0"], st
            e = ts.update_energy_and_gradients()  # FP64 at the returned state
            assert abs(np.linalg.norm(ts.get("forces")) - st["grad_norm"]) <= 1e-9 * st["grad_norm0"], (delta, st)
            assert abs(e - st["energy"]) <= 1e-10 * abs(e), (delta, e, st["energy"])
            ts.step_next()
        states[delta] = ts.get("deformation")
    assert rel(states[1], states[0]) <= 1e-5
