"""The fused element-Hessian + assembly kernel against the two-kernel path (element blocks to memory, then
per-slot assembly) and against the FP64 oracle.

Both paths sum the same element blocks (time_step.hpp:626-658) into the same slots; only the order of the
floating-point sums differs.  Checked: the system values with and without the SPD projection and the
Dirichlet filter, the block-Jacobi preconditioner through a PCG solve, meshes with jitter, per-element
material and a batch of small cubes (whose slots collect up to 24 contributions in one chunk), and that
repeated evaluations are bitwise identical (the kernel has no atomics).
"""
import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import mesh, scenes

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _scenes():
    return {
        "cube10": scenes.cube10(),
        "bar_small": scenes.bar(20, 6, 6),
        "batch": scenes.batch_cubes(n=12, kmin=2, kmax=6, seed=21),
        "unit_box": scenes.reference_box(9),
    }


def _values(sc, precision, fused, spsd, filt, u):
    params = g.default_params(fused_assembly=fused)
    if sc.get("vertex_offsets") is not None:
        ts = scenes.build_batch_timestep(sc, precision=precision, params=params)
    else:
        ts = scenes.build_timestep(sc, precision=precision, params=params)
    ts.set("next_deform", u)
    ts.update_hessian(False, spsd, filt)
    return ts, ts.values("sysmatrix")


@pytest.mark.parametrize("name", ["cube10", "bar_small", "batch", "unit_box"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_matches_two_kernel_path(name, precision):
    sc = _scenes()[name]
    u = np.random.default_rng(8).uniform(-1, 1, sc["X"].shape) * 0.05
    tol = 1e-13 if precision == "fp64" else 2e-6
    for spsd, filt in ((True, True), (False, True), (True, False)):
        ts_f, vf = _values(sc, precision, 1, spsd, filt, u)
        ts_2, v2 = _values(sc, precision, 0, spsd, filt, u)
        assert rel(vf, v2) <= tol, (spsd, filt, rel(vf, v2))
        # the same kernel twice: bitwise
        ts_f.update_hessian(False, spsd, filt)
        assert np.array_equal(ts_f.values("sysmatrix"), vf)
    # the preconditioner rows come with the fused values: the same PCG solution
    b = np.random.default_rng(9).normal(size=sc["X"].shape)
    xf, _, _ = ts_f.pcg(b, rtol=1e-10 if precision == "fp64" else 1e-5, max_iters=20000)
    x2, _, _ = ts_2.pcg(b, rtol=1e-10 if precision == "fp64" else 1e-5, max_iters=20000)
    assert rel(xf, x2) <= (1e-8 if precision == "fp64" else 1e-3)


def test_fused_fp64_matches_oracle():
    """FP64 fused values against the oracle on a jittered box with per-element E (1e-10, as the other
    Hessian parity tests)."""
    from oracle import pyoracle

    X, T = mesh.kuhn_box((7, 5, 6), (1.4, 1.0, 1.2))
    X = mesh.jitter_interior(X, 0.02, 31)
    E = 10.0 ** mesh.uniform(32, T.shape[0], 4.0, 6.0)
    ts = g.TimeStep(X, T, 1e-2, 1e5, 0.45, 1000.0)
    ts.set_material(E, None)
    ts.set_params(g.default_params(fused_assembly=1))
    ts.reset("none")
    ot = pyoracle.OracleTimeStep(X, T, 1e-2, 1e5, 0.45, 1000.0)
    ot.set_material(E, None)
    ot.reset()
    fixed = np.where(X[:, 2] == 0.0)[0]
    ts.mark_dirichlet_batched(fixed, np.zeros((fixed.size, 3)))
    ot.mark_dirichlet(fixed)
    u = np.random.default_rng(10).uniform(-1, 1, X.shape) * 0.2
    for spsd in (True, False):
        ts.set("next_deform", u)
        ot.set("next_deform", u)
        ts.update_hessian(False, spsd, True)
        ot.update_hessian(False, spsd, True)
        assert rel(ts.values("sysmatrix"), ot.values("sysmatrix")) <= 1e-10
