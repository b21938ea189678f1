"""Pins of the FP64 oracle against the reference's own tests.

ssim ships no golden vectors; its correctness pins are known-answer and
finite-difference tests.  Each test here restates one of them (file:line of the
reference's tests/ tree) against the oracle, with the reference's tolerances.
"""
import numpy as np
import pytest

F_FD = np.array([[1, 0.3, 0.2], [0.2, 2, 0.1], [0.1, 0.3, 1]], dtype=np.float64)


def test_snh_rest_known_answer(oracle):
    """tests/fem_intro/main.cpp:95-106: energy and PK1 vanish at F = I (tol 1e-7)."""
    lam, mu = oracle.lame(1e6, 0.3)
    e, P = oracle.snh_stress(np.eye(3), lam, mu)
    assert abs(e) < 1e-7
    assert np.abs(P).max() < 1e-7
    assert abs(oracle.snh_energy(np.eye(3), lam, mu)) < 1e-7


def test_snh_stress_fd(oracle):
    """tests/fem_intro/main.cpp:108-126: central FD of the energy vs PK1 (delta 1e-6, tol 1e-3)."""
    lam, mu = oracle.lame(1e6, 0.3)
    _, P = oracle.snh_stress(F_FD, lam, mu)
    d = 1e-6
    for i in range(3):
        for j in range(3):
            Fp, Fm = F_FD.copy(), F_FD.copy()
            Fp[i, j] += d
            Fm[i, j] -= d
            fd = (oracle.snh_energy(Fp, lam, mu) - oracle.snh_energy(Fm, lam, mu)) / (2 * d)
            assert abs(P[i, j] - fd) < 1e-3


def test_snh_hessian_fd(oracle):
    """tests/fem_intro/main.cpp:128-153: central FD of PK1 vs the 9x9 Hessian (relative 1e-3)."""
    lam, mu = oracle.lame(1e6, 0.3)
    H = oracle.snh_hessian(F_FD, lam, mu)
    d = 1e-6
    for i in range(3):
        for j in range(3):
            Fp, Fm = F_FD.copy(), F_FD.copy()
            Fp[i, j] += d
            Fm[i, j] -= d
            Pp = oracle.snh_stress(Fp, lam, mu)[1]
            Pm = oracle.snh_stress(Fm, lam, mu)[1]
            for k in range(3):
                for l in range(3):
                    h = H[i * 3 + j, k * 3 + l]
                    fd = (Pp[k, l] - Pm[k, l]) / (2 * d)
                    den = max(abs(h), abs(fd))
                    if den == 0:
                        continue
                    assert abs(h - fd) / den < 1e-3, (i, j, k, l, h, fd)
    assert np.allclose(H, H.T, rtol=0, atol=1e-9 * np.abs(H).max())


def test_linear_known_answer_and_fd(oracle):
    """tests/fem_intro/main.cpp:13-83 (elast.linear3): E=1e6, nu=0.4; energy and PK1 vanish at F = I (1e-7);
    central FD of the energy vs PK1 and of PK1 vs the Hessian at the same F, delta 1e-3, tol 1e-3 (the
    reference compares H(i*3+j, k*3+l) with the FD of P(l, k); the model is symmetric in F and F^T)."""
    lam, mu = oracle.lame(1e6, 0.4)
    e, P = oracle.linear_stress(np.eye(3), lam, mu)
    assert abs(e) < 1e-7 and np.abs(P).max() < 1e-7
    d = 1e-3
    _, P = oracle.linear_stress(F_FD, lam, mu)
    H = oracle.linear_hessian(lam, mu)
    for i in range(3):
        for j in range(3):
            Fp, Fm = F_FD.copy(), F_FD.copy()
            Fp[i, j] += d
            Fm[i, j] -= d
            ep, Pp = oracle.linear_stress(Fp, lam, mu)
            em, Pm = oracle.linear_stress(Fm, lam, mu)
            assert abs(P[i, j] - (ep - em) / (2 * d)) < 1e-3 * max(1.0, abs(P[i, j]))
            for k in range(3):
                for l in range(3):
                    fd = (Pp[l, k] - Pm[l, k]) / (2 * d)
                    assert abs(H[i * 3 + j, k * 3 + l] - fd) < 1e-3 * max(1.0, abs(fd))


def test_linear_projected_stiffness(oracle):
    """The make_spsd clamp (time_step.hpp:50-56) lifts the linear model's three rotation (skew) modes from 0
    to 1e-3 and leaves the 2 mu / 2 mu + 3 lambda modes: the element stiffness differs from the
    unprojected one exactly by 1e-3 times the pfpx contraction of the skew projector."""
    lam, mu = oracle.lame(1e5, 0.3)
    Dm, _ = oracle.dminv([0, 0, 0], [1, 0.1, 0], [0.2, 1, 0], [0, 0.1, 1.1])
    K0 = oracle.element_stiffness(np.eye(3), Dm, lam, mu, make_spsd=False, model=1)
    K1 = oracle.element_stiffness(np.eye(3), Dm, lam, mu, make_spsd=True, model=1)
    T = np.zeros((9, 9))
    for i in range(3):
        for j in range(3):
            T[i * 3 + j, j * 3 + i] = 1
    Pskew = 0.5 * (np.eye(9) - T)
    D = np.zeros((9, 12))  # pfpx: dF(r,c)/dx(v,s) = delta_rs grad N_v[c]
    g = np.zeros((4, 3))
    g[1:] = np.asarray(Dm)
    g[0] = -g[1:].sum(0)
    for r in range(3):
        for c in range(3):
            for v in range(4):
                D[r * 3 + c, v * 3 + r] = g[v, c]
    assert np.allclose(K1 - K0, 1e-3 * D.T @ Pskew @ D, rtol=0, atol=1e-9 * np.abs(K0).max())


def test_deform_rest_identity_and_volume(oracle):
    """tests/fem_intro/main.cpp:311-333: F == I at rest, sum of rest volumes == 1 on unit_box()."""
    X, cells = oracle.unit_box(2, 2, 2)
    ts = oracle.OracleTimeStep(X, cells, 1e-2, 1e6, 0.33, 1.0)
    ts.update_energy_and_gradients()
    F = ts.def_grad()
    assert np.abs(F - np.eye(3)).max() < 1e-12
    assert abs(ts.rest_vol().sum() - 1.0) < 1e-6


def test_integration_mass_and_laplace(oracle):
    """tests/fem_local_global/main.cpp:166-197: sum of local mass == 1, sum of local Laplacian == 0."""
    X, cells = oracle.unit_box(2, 2, 2)
    ts = oracle.OracleTimeStep(X, cells, 1e-2, 1e6, 0.33, 1.0)
    assert abs(ts.local_mass(1.0).sum() - 1.0) < 1e-6
    assert abs(ts.local_laplace(1.0).sum()) < 1e-6
    # the assembled consistent mass holds three copies (one per dof) of the local mass
    assert abs(ts.values("mass").sum() / 3.0 - 1.0) < 1e-12


def test_gather_3d(oracle):
    """tests/fem_local_global/main.cpp:85-164: gathered forces / Hessian vs brute force.

    The composer's weights are the rest volumes (global_composer.hpp:36-128)."""
    X, cells = oracle.unit_box(2, 2, 2)
    ts = oracle.OracleTimeStep(X, cells, 1e-2, 1e6, 0.33, 1.0)
    nE, nV = cells.shape[0], X.shape[0]
    w = ts.rest_vol()
    lf = np.arange(nE * 12, dtype=np.float64).reshape(nE, 4, 3)
    f = ts.gather_force(lf, alpha=0.2)
    gt = np.zeros((nV, 3))
    for i in range(nE):
        for j in range(4):
            gt[cells[i, j]] += lf[i, j] * w[i] * 0.2
    assert np.allclose(f, gt, rtol=1e-14, atol=0)
    K = np.arange(nE * 144, dtype=np.float64).reshape(nE, 12, 12)
    rp, ci = ts.csr_pattern()
    dense = np.zeros((3 * nV, 3 * nV))
    for i in range(nE):
        dofs = (3 * cells[i][:, None] + np.arange(3)[None, :]).reshape(-1)
        dense[np.ix_(dofs, dofs)] -= K[i] * w[i]
    base = np.array([dense[r, ci[k]] for r in range(3 * nV) for k in range(rp[r], rp[r + 1])])
    vals = ts.gather_hessian(K, 1.0, base=base)
    assert np.abs(vals).max() < 1e-9 * np.abs(base).max()


def _fd_check(oracle, X, cells, deform, inertia, delta=1e-4):
    ts = oracle.OracleTimeStep(X, cells, 1e-2, 1e6, 0.33, 0.0)
    ts.prepare_step()
    if inertia is not None:
        ts.set("inertia_deform", inertia)
    ts.set("next_deform", deform)
    ts.update_energy_and_gradients()
    g = ts.get("forces").reshape(-1)
    n = g.size
    fd = np.zeros(n)
    base = deform.reshape(-1)
    for k in range(n):
        up, um = base.copy(), base.copy()
        up[k] += delta
        um[k] -= delta
        fd[k] = (ts.energy_at(up) - ts.energy_at(um)) / (2 * delta)
    ts.set("next_deform", deform)
    ts.update_energy_and_gradients()
    ts.update_hessian()  # make_spsd = false, filter = true (time_step.hpp:626)
    H = ts.matrix("sysmatrix").toarray()
    Hfd = np.zeros((n, n))
    for k in range(n):
        up, um = base.copy(), base.copy()
        up[k] += delta
        um[k] -= delta
        ts.set("next_deform", up)
        ts.update_energy_and_gradients()
        gp = ts.get("forces").reshape(-1)
        ts.set("next_deform", um)
        ts.update_energy_and_gradients()
        gm = ts.get("forces").reshape(-1)
        Hfd[:, k] = (gp - gm) / (2 * delta)
    return g, fd, H, Hfd


def test_time_step_fd_tetra(oracle):
    """tests/fem_time_step_diff/main.cpp:19-92: FD gradient and Hessian of the incremental potential
    on tetra(), E=1e6, nu=0.33, rho=0, the deformation of :34-45 and a random inertia target."""
    X, cells = oracle.tetra()
    deform = np.array([[-0.1, -0.1, -0.1], [0.1, -0.1, -0.1], [-0.1, 0.1, -0.1], [0.1, 0.1, -0.1]])
    inertia = np.random.default_rng(0).uniform(-1, 1, size=(4, 3))
    g, fd, H, Hfd = _fd_check(oracle, X, cells, deform, inertia)
    assert np.sum((fd - g) ** 2) < 1e-4
    assert np.sum((Hfd - H) ** 2) < 1e-4


def test_time_step_fd_unit_box(oracle):
    """tests/fem_time_step_diff/main.cpp:95-172: the same on unit_box(7,7,7) with random u * 0.3."""
    X, cells = oracle.unit_box(7, 7, 7)
    deform = np.random.default_rng(1).uniform(-1, 1, size=X.shape) * 0.3
    g, fd, H, Hfd = _fd_check(oracle, X, cells, deform, None)
    assert np.sum((fd - g) ** 2) < 1e-4
    assert np.sum((Hfd - H) ** 2) < 1e-4


# ---------------------------------------------------------------- oracle self-consistency
def test_jacobi_eigen_vs_lapack(oracle):
    rng = np.random.default_rng(2)
    for _ in range(20):
        A = rng.normal(size=(9, 9))
        A = A + A.T
        w, V = oracle.sym_eigen(A)
        assert np.allclose(np.sort(w), np.linalg.eigvalsh(A), rtol=0, atol=1e-12 * np.abs(A).max())
        assert np.allclose(V @ np.diag(w) @ V.T, A, rtol=0, atol=1e-12 * np.abs(A).max())


def test_project_spd_vs_lapack(oracle):
    lam, mu = oracle.lame(1e5, 0.45)
    rng = np.random.default_rng(3)
    for _ in range(20):
        F = np.eye(3) + 0.4 * rng.normal(size=(3, 3))
        H = oracle.snh_hessian(F, lam, mu)
        w, V = np.linalg.eigh(H)
        ref = V @ np.diag(np.maximum(w, 1e-3)) @ V.T
        assert np.allclose(oracle.project_spd(H), ref, rtol=0, atol=1e-10 * np.abs(H).max())


def test_element_stiffness_is_pfpx_contraction(oracle):
    """time_step.hpp:58 with compute_pfpx_3 (internal_physic.hpp:107-160)."""
    lam, mu = oracle.lame(1e5, 0.45)
    rng = np.random.default_rng(4)
    xs = rng.normal(size=(4, 3))
    Dm, vol = oracle.dminv(*xs)
    F = np.eye(3) + 0.2 * rng.normal(size=(3, 3))
    # pfpx [9, 12]: row r*3+c of F, column v*3+a
    D = np.zeros((4, 3))
    D[1:] = Dm
    D[0] = -Dm.sum(axis=0)
    P = np.zeros((9, 12))
    for r in range(3):
        for c in range(3):
            for v in range(4):
                P[r * 3 + c, v * 3 + r] = D[v, c]
    for spsd in (False, True):
        H = oracle.snh_hessian(F, lam, mu)
        if spsd:
            H = oracle.project_spd(H)
        ref = P.T @ H @ P
        K = oracle.element_stiffness(F, Dm, lam, mu, spsd)
        assert np.allclose(K, ref, rtol=0, atol=1e-10 * np.abs(ref).max())


def test_csr_pattern_matches_coo_to_csr(oracle):
    """The pattern equals COO->CSR of the composer's triplets (global_composer.hpp:81-92):
    sorted unique columns, full symmetric storage, explicit zeros kept."""
    import scipy.sparse as sp

    X, cells = oracle.unit_box(4, 3, 5)
    ts = oracle.OracleTimeStep(X, cells, 1e-2, 1e6, 0.33, 1.0)
    rp, ci = ts.csr_pattern()
    rows, cols = [], []
    for c in cells:
        for i in range(4):
            for j in range(4):
                for a in range(3):
                    for b in range(3):
                        rows.append(3 * c[i] + a)
                        cols.append(3 * c[j] + b)
    n = 3 * X.shape[0]
    M = sp.coo_matrix((np.ones(len(rows)), (rows, cols)), shape=(n, n)).tocsr()
    M.sum_duplicates()
    M.sort_indices()
    assert np.array_equal(M.indptr.astype(np.int32), rp)
    assert np.array_equal(M.indices.astype(np.int32), ci)


def test_newton_step_converges_and_matches_direct_solve(oracle):
    """One backward-Euler step with Newton + Jacobi-PCG: converged, and the last Newton update
    solves the projected system."""
    X, cells = oracle.unit_box(5, 4, 4)
    ts = oracle.OracleTimeStep(X, cells, 1e-2, 1e5, 0.4, 1000.0)
    fixed = np.where(X[:, 0] == 0)[0]
    ts.mark_dirichlet(fixed)
    ts.add_gravity([0, 0, -9.8])
    ts.set_threshold(1e-6)
    ts.reset()
    for _ in range(3):
        ts.prepare_step()
        r, st = ts.compute_step("newton", oracle.default_params(cg_rtol=1e-10))
        assert st["converged"] == 1
        assert r < ts.threshold_abs
        ts.step_next()
    assert np.abs(ts.get("deformation")[fixed]).max() == 0.0
    assert ts.get("deformation")[:, 2].min() < 0
