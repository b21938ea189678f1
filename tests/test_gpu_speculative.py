"""The speculative assembly (speculative_hessian = 1): the mixed Newton assembles the next iteration's Hessian
at the full step u + d on a second stream while the line search runs, from the same FP32 positions that the
accepted full step produces.  Checked: the trajectories with and without it are bitwise equal (the same
matrices, the same solves), whether the line search takes the full step (the matrix made ahead is used:
spec_hits > 0) or backtracks (it is discarded and the matrix assembled again); in both precisions of the
element blocks; and the FP64 path, which never speculates, is unaffected.
"""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import scenes

pytestmark = pytest.mark.gpu


def _run(scene, spec, precision="mixed", steps=3, **kw):
    params = g.default_params(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2, precond=2,
                              speculative_hessian=spec, **kw)
    ts = scenes.build_timestep(scene, precision=precision, params=params)
    stats = []
    for _ in range(steps):
        ts.step()
        stats.append(ts.stats())
    return ts.get("deformation"), stats


@pytest.mark.parametrize("name", ["beam_small", "bar_small"])
@pytest.mark.parametrize("blocks", [1, 0])
def test_speculative_assembly_is_bitwise_the_same(name, blocks):
    scene = {"beam_small": lambda: scenes.beam(40, 20, 14, h=0.05), "bar_small": lambda: scenes.bar(20, 6, 6)}[name]()
    u1, st1 = _run(scene, 1, half_hessian_blocks=blocks)
    u0, st0 = _run(scene, 0, half_hessian_blocks=blocks)
    assert np.array_equal(u1, u0)
    for a, b in zip(st1, st0):
        assert a["converged"] == 1 and (a["newton_iters"], a["cg_iters_total"]) == (b["newton_iters"], b["cg_iters_total"])
        assert b["spec_hits"] == 0
    assert sum(a["spec_hits"] for a in st1) > 0


def test_speculation_discarded_on_backtracking():
    """With the Armijo constant at 0.6 a Newton step on a near-quadratic energy never passes at alpha = 1
    (it decreases the energy by about half of alpha g.d) and passes at 0.5: every speculative matrix is
    thrown away and assembled again; the trajectory is still bitwise the unspeculative one."""
    scene = scenes.beam(40, 20, 14, h=0.05)
    u1, st1 = _run(scene, 1, steps=1, armijo=0.6)
    u0, st0 = _run(scene, 0, steps=1, armijo=0.6)
    assert np.array_equal(u1, u0)
    ls = sum(a["ls_steps_total"] for a in st1)
    newton = sum(a["newton_iters"] for a in st1)
    hits = sum(a["spec_hits"] for a in st1)
    assert st1[0]["converged"] == 1
    assert ls > newton, "no backtracking in this run: the discard path was not exercised"
    assert hits < newton


def test_fp64_never_speculates():
    scene = scenes.bar(20, 6, 6)
    _, st = _run(scene, 1, precision="fp64", steps=1)
    assert st[0]["converged"] == 1 and st[0]["spec_hits"] == 0
