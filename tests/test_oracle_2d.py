"""The FP64 oracle's 2D triangle path, pinned by the reference's own 2D element tests.

tests/fem_intro/main.cpp:157-297 (elast.linear2, elast.snh2) check the 2D models at F = I and by central
differences at F = [[1, 0.3], [0.2, 3]]; the time-step level (no reference instance for 2D) is checked by
central differences of the incremental potential, the way tests/fem_time_step_diff/main.cpp checks 3D.
"""
import numpy as np
import pytest

from ssim_gb300 import mesh

F2 = np.array([[1.0, 0.3], [0.2, 3.0]])


def _fd_hessian(stress, H, d):
    for i in range(2):
        for j in range(2):
            Fp, Fm = F2.copy(), F2.copy()
            Fp[i, j] += d
            Fm[i, j] -= d
            Pp, Pm = stress(Fp), stress(Fm)
            for k in range(2):
                for l in range(2):
                    h = H[i * 2 + j, k * 2 + l]
                    fd = (Pp[k, l] - Pm[k, l]) / (2 * d)
                    yield h, fd


def test_snh2_known_answer_and_fd(oracle):
    """elast.snh2 (:229-297): E=1e6, nu=0.3; Psi(I) = P(I) = 0 (1e-7); FD of Psi vs P (delta 1e-6, 1e-3);
    FD of P vs H (relative 1e-3)."""
    lam, mu = oracle.lame(1e6, 0.3)
    e, P = oracle.snh2_stress(np.eye(2), lam, mu)
    assert abs(e) < 1e-7 and np.abs(P).max() < 1e-7
    assert abs(oracle.snh2_energy(np.eye(2), lam, mu)) < 1e-7
    _, P = oracle.snh2_stress(F2, lam, mu)
    d = 1e-6
    for i in range(2):
        for j in range(2):
            Fp, Fm = F2.copy(), F2.copy()
            Fp[i, j] += d
            Fm[i, j] -= d
            fd = (oracle.snh2_energy(Fp, lam, mu) - oracle.snh2_energy(Fm, lam, mu)) / (2 * d)
            assert abs(P[i, j] - fd) < 1e-3
    H = oracle.snh2_hessian(F2, lam, mu)
    for h, fd in _fd_hessian(lambda F: oracle.snh2_stress(F, lam, mu)[1], H, d):
        den = max(abs(h), abs(fd))
        if den > 0:
            assert abs(h - fd) / den < 1e-3
    assert np.allclose(H, H.T)


def test_linear2_known_answer_and_fd(oracle):
    """elast.linear2 (:157-227): E=1e6, nu=0.4; Psi(I) = P(I) = 0; FD (delta 1e-3, absolute 1e-3)."""
    lam, mu = oracle.lame(1e6, 0.4)
    e, P = oracle.linear2_stress(np.eye(2), lam, mu)
    assert abs(e) < 1e-7 and np.abs(P).max() < 1e-7
    _, P = oracle.linear2_stress(F2, lam, mu)
    d = 1e-3
    for i in range(2):
        for j in range(2):
            Fp, Fm = F2.copy(), F2.copy()
            Fp[i, j] += d
            Fm[i, j] -= d
            fd = (oracle.linear2_stress(Fp, lam, mu)[0] - oracle.linear2_stress(Fm, lam, mu)[0]) / (2 * d)
            assert abs(P[i, j] - fd) < 1e-3
    H = oracle.linear2_hessian(lam, mu)
    for h, fd in _fd_hessian(lambda F: oracle.linear2_stress(F, lam, mu)[1], H, d):
        assert abs(h - fd) < 1e-3


def test_2d_snh_delta_is_the_root():
    """stable_neohookean.hpp:93-100: delta solves (2t+1) d^2 + (2t+2) d - 2t = 0 and makes Psi(I) = 0 with
    P(I) = 0: dPsi/dF at I is mu (1 - 1/(2 + delta)) I + lambda (1 - alpha) I = 0."""
    for E, nu in [(1e6, 0.3), (1e5, 0.45), (3e4, 0.1)]:
        lam = E * nu / ((1 + nu) * (1 - 2 * nu))
        mu = E / (2 * (1 + nu))
        t = mu / lam
        dl = (-(2 * t + 2) + np.sqrt((2 * t + 2) ** 2 + 8 * t * (2 * t + 1))) / (2 * (2 * t + 1))
        assert abs((2 * t + 1) * dl * dl + (2 * t + 2) * dl - 2 * t) < 1e-14
        alpha = (1 - 1 / (2 + dl)) * mu / lam + 1
        assert abs(mu * (1 - 1 / (2 + dl)) + lam * (1 - alpha)) < 1e-8 * mu


def test_2d_integrals(oracle):
    """p1_element_2d (bilinears.hpp:45-96): the consistent mass sums to rho x area, every Laplacian row of
    the PD matrix minus the mass sums to zero."""
    X, T = mesh.unit_square(5, 4)
    ts = oracle.OracleTimeStep.tri2d(X, T, 1e-2, 1e5, 0.4, 700.0)
    M = ts.matrix("mass").toarray()
    assert M[0::3, 0::3].sum() == pytest.approx(700.0, rel=1e-14)
    A = ts.pd_matrix_values()
    rp, ci = ts.csr_pattern()
    Pd = np.zeros_like(M)
    for r in range(M.shape[0]):
        Pd[r, ci[rp[r]:rp[r + 1]]] = A[rp[r]:rp[r + 1]]
    assert np.abs((Pd - M).sum(axis=1)).max() < 1e-9 * np.abs(Pd).max()


def test_2d_time_step_fd(oracle):
    """FD gradient and Hessian (make_spsd off) of the 2D incremental potential on unit_square(4, 3) with a
    random state: the 3D check of tests/fem_time_step_diff/main.cpp:95-172 in the plane."""
    X, T = mesh.unit_square(4, 3)
    ts = oracle.OracleTimeStep.tri2d(X, T, 1e-2, 1e5, 0.4, 100.0)
    rng = np.random.default_rng(3)
    v = np.zeros((X.shape[0], 3))
    v[:, :2] = rng.uniform(-1, 1, (X.shape[0], 2))
    ts.set("velocity", v)
    ts.prepare_step()
    u = np.zeros((X.shape[0], 3))
    u[:, :2] = rng.uniform(-1, 1, (X.shape[0], 2)) * 0.05
    base = u.reshape(-1)
    ts.set("next_deform", u)
    ts.update_energy_and_gradients()
    g = ts.get("forces").reshape(-1)
    assert np.all(g[2::3] == 0)
    ts.update_hessian(make_spsd=False)
    H = ts.matrix().toarray()
    d = 1e-6
    for q in [k for k in range(base.size) if k % 3 != 2]:
        up, um = base.copy(), base.copy()
        up[q] += d
        um[q] -= d
        fd = (ts.energy_at(up) - ts.energy_at(um)) / (2 * d)
        assert abs(fd - g[q]) < 1e-6 * max(1.0, np.abs(g).max())
        ts.set("next_deform", up)
        ts.update_energy_and_gradients()
        gp = ts.get("forces").reshape(-1)
        ts.set("next_deform", um)
        ts.update_energy_and_gradients()
        gm = ts.get("forces").reshape(-1)
        col = (gp - gm) / (2 * d)
        assert np.abs(col - H[:, q]).max() < 1e-5 * np.abs(H).max()


def test_2d_newton_converges_in_plane(oracle):
    """A hanging 2D sheet (x = 0 edge fixed, gravity -y) under tight Newton: converges every step, z stays 0."""
    X, T = mesh.unit_square(8, 6)
    ts = oracle.OracleTimeStep.tri2d(X, T, 1e-2, 1e5, 0.4, 100.0)
    ts.mark_dirichlet(np.where(X[:, 0] == 0.0)[0])
    ts.add_gravity((0.0, -9.8, 0.0))
    ts.reset()
    p = oracle.default_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-12)
    for _ in range(4):
        ts.prepare_step()
        _, st = ts.compute_step("newton", p)
        ts.step_next()
        assert st["converged"] == 1
    u = ts.get("deformation")
    assert np.all(u[:, 2] == 0.0) and u[:, 1].min() < -1e-4
