"""The FP64 oracle's mass-spring system (cloth), checked on the CPU.

The reference has no spring model, so there is nothing of its own to pin
against: the oracle's spring energy is checked against its closed form, its
gradient and Hessian against central differences of the energy (the
reference's own pinning method for the tets, tests/fem_time_step_diff/main.cpp),
the projective-dynamics matrix against a dense construction, and the
steppers against one another on a tight tolerance.
"""
import numpy as np
import pytest

from ssim_gb300 import scenes
from oracle import scenes as oscenes


def _dense(ts, which="sysmatrix"):
    return ts.matrix(which).toarray()


def test_spring_pair_known_answer(oracle):
    """Two vertices, one spring of rest length 1 stretched to 1.5: E = 1/2 m |u - x~|^2 + dt^2 k/2 (0.5)^2."""
    X = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    k, m, dt = 40.0, 0.3, 0.05
    ts = oracle.OracleTimeStep.springs(X, np.array([[0, 1]]), k, mass=m, time_step=dt)
    ts.prepare_step()  # zero velocity and load: x~ = 0
    u = np.array([[-0.25, 0, 0], [0.25, 0, 0]])
    e = ts.energy_at(u)
    want = 0.5 * m * 2 * 0.25**2 + dt * dt * k / 2 * 0.25
    assert e == pytest.approx(want, rel=1e-14)
    ts.set("next_deform", u)
    ts.update_energy_and_gradients()
    g = ts.get("forces")
    f = dt * dt * k * 0.5  # spring tension times dt^2
    assert np.allclose(g, [[-m * 0.25 - f, 0, 0], [m * 0.25 + f, 0, 0]], rtol=1e-13, atol=0)


def test_spring_fd_gradient_and_hessian(oracle):
    """Central differences of the energy (gradient) and of the gradient (unprojected Hessian) on a
    5x5 cloth with a random state, no Dirichlet dofs."""
    sc = scenes.cloth(5, h=0.1, k=50.0, areal_density=2.0, dt=0.05)
    ts = oracle.OracleTimeStep.springs(sc["X"], sc["cells"], sc["k"], vertex_mass=sc["vertex_mass"],
                                       time_step=sc["dt"])
    rng = np.random.default_rng(7)
    ts.set("velocity", rng.uniform(-1, 1, size=sc["X"].shape))
    ts.prepare_step()
    u = rng.uniform(-1, 1, size=sc["X"].shape) * 0.04
    base = u.reshape(-1)
    delta = 1e-6
    ts.set("next_deform", u)
    ts.update_energy_and_gradients()
    g = ts.get("forces").reshape(-1)
    ts.update_hessian(make_spsd=False)
    H = _dense(ts)
    n = base.size
    fd = np.zeros(n)
    Hfd = np.zeros((n, n))
    for q in range(n):
        up, um = base.copy(), base.copy()
        up[q] += delta
        um[q] -= delta
        fd[q] = (ts.energy_at(up) - ts.energy_at(um)) / (2 * delta)
        ts.set("next_deform", up)
        ts.update_energy_and_gradients()
        gp = ts.get("forces").reshape(-1)
        ts.set("next_deform", um)
        ts.update_energy_and_gradients()
        gm = ts.get("forces").reshape(-1)
        Hfd[:, q] = (gp - gm) / (2 * delta)
    assert np.max(np.abs(fd - g)) < 1e-7 * max(1.0, np.max(np.abs(g)))
    assert np.max(np.abs(Hfd - H)) < 1e-6 * np.max(np.abs(H))
    assert np.allclose(H, H.T, rtol=0, atol=1e-14 * np.max(np.abs(H)))


def test_spring_projected_hessian_is_psd(oracle):
    """make_spsd clamps the compressed springs' transverse stiffness: the projected matrix minus the
    lumped mass is positive semi-definite on a compressed random state."""
    sc = scenes.cloth(4, h=0.1, k=50.0, areal_density=2.0, dt=0.05)
    ts = oracle.OracleTimeStep.springs(sc["X"], sc["cells"], sc["k"], vertex_mass=sc["vertex_mass"],
                                       time_step=sc["dt"])
    ts.prepare_step()
    u = -0.3 * sc["X"] + np.random.default_rng(3).uniform(-1, 1, size=sc["X"].shape) * 0.01
    ts.set("next_deform", u)
    ts.update_energy_and_gradients()
    ts.update_hessian(make_spsd=True)
    K = _dense(ts) - _dense(ts, "mass")
    assert np.linalg.eigvalsh(0.5 * (K + K.T)).min() > -1e-12 * np.abs(K).max()
    ts.update_hessian(make_spsd=False)
    K = _dense(ts) - _dense(ts, "mass")
    assert np.linalg.eigvalsh(0.5 * (K + K.T)).min() < -1e-6 * np.abs(K).max()


def test_spring_pd_matrix_dense(oracle):
    """Projective-dynamics matrix of a spring system: M + dt^2 sum_s k (e_i - e_j)(e_i - e_j)^T (x) I3."""
    sc = scenes.cloth(4, h=0.1, k=50.0, areal_density=2.0, dt=0.05)
    ts = oracle.OracleTimeStep.springs(sc["X"], sc["cells"], sc["k"], vertex_mass=sc["vertex_mass"],
                                       time_step=sc["dt"])
    nv = sc["X"].shape[0]
    Lap = np.zeros((nv, nv))
    for i, j in sc["cells"]:
        Lap[i, i] += 1
        Lap[j, j] += 1
        Lap[i, j] -= 1
        Lap[j, i] -= 1
    want = np.kron(np.diag(sc["vertex_mass"]) + sc["dt"] ** 2 * sc["k"] * Lap, np.eye(3))
    rp, ci = ts.csr_pattern()
    vals = ts.pd_matrix_values()
    got = np.zeros_like(want)
    for r in range(3 * nv):
        for q in range(rp[r], rp[r + 1]):
            got[r, ci[q]] = vals[q]
    assert np.allclose(got, want, rtol=1e-15, atol=0)


def test_spring_steppers_agree(oracle):
    """Newton, L-BFGS and projective dynamics reach the same minimiser of one cloth step on a tight
    tolerance (corners pinned, gravity)."""
    sc = scenes.cloth(8, h=0.05, k=1e3, areal_density=0.5, dt=1e-2)
    outs = {}
    for method in ("newton", "lbfgs", "pd"):
        ts = oscenes.build_oracle(sc, rtol=1e-10)
        p = oracle.default_params(max_newton_iters=100000, max_lbfgs_iters=100000)
        for _ in range(2):
            ts.prepare_step()
            _, st = ts.compute_step(method, p)
            assert st["converged"] == 1, (method, st)
            ts.step_next()
        outs[method] = ts.get("deformation")
    scale = np.abs(outs["newton"]).max()
    assert scale > 1e-4
    for m in ("lbfgs", "pd"):
        assert np.abs(outs[m] - outs["newton"]).max() < 1e-6 * scale, m
