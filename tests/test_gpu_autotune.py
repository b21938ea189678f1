"""The launch-shape autotuner (ssim_gb_autotune): a sweep on the handle's own data that applies the fastest
block sizes, PCG variant / grid and assembly path, cached per process by problem shape.

Checked: the choices come from the candidate sets and the sweep timed them; a second handle of the same
shape takes the cached choice without timing; the forces view and the deformation are left as they were;
and a tuned handle steps to the same states as an untuned one up to the solver tolerance (tuning changes
launch shapes and the PCG variant, not the equations), in both precisions and for a batch of instances;
and a saved tuning applied with ssim_gb_set_tuning, with out-of-set values rejected.
"""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import scenes

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _params():
    return g.default_params(stop_mode=1, rel_tol=1e-8, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=1e-3, precond=2)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_autotune_choices_cache_and_states(precision):
    scene = scenes.bar(24, 8, 8)
    ts = scenes.build_timestep(scene, precision=precision, params=_params())
    ts.step()
    u, f = ts.get("deformation"), ts.get("forces")
    t = ts.autotune()
    assert t["from_cache"] == 0 and t["candidates"] >= 8
    if precision == "mixed":
        assert t["elem_block"] in (64, 128, 256) and t["gather_block"] in (128, 256, 512)
        assert t["elem_regcap"] in (0, 1)
        assert t["pcg_persistent"] in (1, 2, 3)
        assert t["pcg_persistent"] != 3 or t["pcg_half_matrix"] == 1
    else:
        assert t["pcg_persistent"] in (0, 2)
    assert t["hessian_block"] in (32, 64, 128) and t["assembly_block"] in (128, 256, 512)
    assert t["fused_assembly"] in (0, 1) and t["pcg_solve_ms"] > 0 and t["pcg_iterations"] > 0
    if precision == "mixed":
        assert t["pcg_half_matrix"] in (0, 1) and (t["pcg_half_matrix"] == 0 or t["pcg_persistent"] in (2, 3))
    assert np.array_equal(ts.get("deformation"), u) and np.array_equal(ts.get("forces"), f)
    p = ts.params
    assert (p.pcg_persistent, p.pcg_max_blocks, p.fused_assembly) == (t["pcg_persistent"], t["pcg_max_blocks"],
                                                                      t["fused_assembly"])
    assert p.pcg_half_matrix == t["pcg_half_matrix"]
    # a second handle of the same shape: the cached choice
    ts2 = scenes.build_timestep(scene, precision=precision, params=_params())
    t2 = ts2.autotune()
    assert t2["from_cache"] == 1
    for k in ("elem_block", "hessian_block", "assembly_block", "gather_block", "pcg_persistent", "pcg_max_blocks",
              "fused_assembly", "pcg_half_matrix", "elem_regcap"):
        assert t2[k] == t[k]
    # tuned and untuned handles step to the same states up to the tolerance
    ref = scenes.build_timestep(scene, precision=precision, params=_params())
    for _ in range(3):
        ts2.step()
        ref.step()
        assert ts2.stats()["converged"] == 1 and ref.stats()["converged"] == 1
    assert rel(ts2.get("deformation"), ref.get("deformation")) <= 1e-6


def test_autotune_batch():
    batch = scenes.batch_cubes(n=12, kmin=3, kmax=8, seed=23)
    ts = scenes.build_batch_timestep(batch, precision="mixed", params=_params())
    t = ts.autotune()
    assert t["candidates"] >= 8
    ref = scenes.build_batch_timestep(batch, precision="mixed", params=_params())
    for _ in range(2):
        ts.step()
        ref.step()
    gi, gi0 = ts.instance_residuals()
    assert np.all(gi <= 1e-8 * gi0)
    assert rel(ts.get("deformation"), ref.get("deformation")) <= 1e-6


def test_set_tuning_applies_a_saved_choice():
    """ssim_gb_set_tuning: a tuning from an earlier sweep applied to a fresh handle without timing
    anything; values outside the candidate sets are rejected and leave the handle as it was."""
    scene = scenes.bar(24, 8, 8)
    ts = scenes.build_timestep(scene, precision="mixed", params=_params())
    saved = {"elem_block": 256, "hessian_block": 32, "assembly_block": 512, "gather_block": 128,
             "pcg_persistent": 2, "pcg_max_blocks": 0, "fused_assembly": 0, "pcg_half_matrix": 1, "elem_regcap": 1}
    ts.set_tuning(saved)
    p = ts.params
    assert (p.pcg_persistent, p.pcg_max_blocks, p.fused_assembly, p.pcg_half_matrix) == (2, 0, 0, 1)
    ref = scenes.build_timestep(scene, precision="mixed", params=_params())
    for _ in range(2):
        ts.step()
        ref.step()
        assert ts.stats()["converged"] == 1
    assert rel(ts.get("deformation"), ref.get("deformation")) <= 1e-6
    for bad in ({"elem_block": 96}, {"hessian_block": 256}, {"assembly_block": 64}, {"gather_block": 1024},
                {"pcg_persistent": 5}, {"pcg_max_blocks": -1}, {"fused_assembly": 2}, {"pcg_half_matrix": 2},
                {"elem_regcap": 3}):
        with pytest.raises(ValueError, match="invalid tuning"):
            ts.set_tuning(dict(saved, **bad))
    p = ts.params
    assert (p.pcg_persistent, p.pcg_max_blocks, p.fused_assembly, p.pcg_half_matrix) == (2, 0, 0, 1)


def test_register_capped_element_pass_is_bitwise_the_same():
    """elem_regcap changes the element pass's register allocation, not its arithmetic: two handles that
    differ only in it step to bitwise equal states."""
    scene = scenes.bar(20, 6, 6)
    base = {"elem_block": 128, "hessian_block": 64, "assembly_block": 256, "gather_block": 256,
            "pcg_persistent": 2, "pcg_max_blocks": 0, "fused_assembly": 0, "pcg_half_matrix": 1}
    states = []
    for cap in (0, 1):
        ts = scenes.build_timestep(scene, precision="mixed", params=_params())
        ts.set_tuning(dict(base, elem_regcap=cap))
        for _ in range(2):
            ts.step()
        states.append(ts.get("deformation"))
    assert np.array_equal(states[0], states[1])
