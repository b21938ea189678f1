"""CPU checks of the PCG recurrences the persistent kernels implement (kernels_sparse.cu), restated with numpy
on a small SPD system with a 3x3 block-Jacobi preconditioner: standard PCG, Chronopoulos-Gear PCG, and
pipelined PCG with u = M r and M s formed from r and s, with and without the switch to Chronopoulos-Gear.
In FP64 all produce the standard PCG iterates; in FP32 the pipelined recurrences drift further from the true
residual than Chronopoulos-Gear's, which is why pipelined PCG is not the default."""
import numpy as np
import pytest


def _system(nv=60, seed=0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    n = 3 * nv
    B = rng.normal(size=(n, n)) / np.sqrt(n)
    A = B @ B.T + np.diag(rng.uniform(0.05, 2.0, size=n))  # SPD, moderately conditioned
    Minv = np.zeros_like(A)
    for v in range(nv):
        s = slice(3 * v, 3 * v + 3)
        Minv[s, s] = np.linalg.inv(A[s, s])
    b = rng.normal(size=n)
    return A.astype(dtype), Minv.astype(dtype), b.astype(dtype)


def _after(st, g, d, iters):
    """cgcg_after: beta = g / g_old, alpha = g / (d - beta g / alpha_old)."""
    if iters == 0:
        beta, alpha = 0.0, g / d
    else:
        beta = g / st["g"]
        alpha = g / (d - beta * g / st["alpha"])
    st.update(g=g, alpha=alpha)
    return alpha, beta


def pcg(A, Minv, b, iters):
    x = np.zeros_like(b)
    r = b.copy()
    z = Minv @ r
    p = z.copy()
    rz = r @ z
    xs = []
    for _ in range(iters):
        q = A @ p
        alpha = rz / (p @ q)
        x = x + alpha * p
        r = r - alpha * q
        z = Minv @ r
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        xs.append(x.copy())
    return xs


def cgcg(A, Minv, b, iters):
    x = np.zeros_like(b)
    r = b.copy()
    u = Minv @ r
    p = np.zeros_like(b)
    s = np.zeros_like(b)
    st, xs = {}, []
    for k in range(iters):
        w = A @ u  # phase A
        alpha, beta = _after(st, r @ u, w @ u, k)
        p = u + beta * p  # phase B
        s = w + beta * s
        x = x + alpha * p
        r = r - alpha * s
        u = Minv @ r
        xs.append(x.copy())
    return xs


def pipelined(A, Minv, b, iters, switch=None):
    """pipe_persistent_kernel: prologue w = A u0, m = M w; phase k: n = A m, z = n + beta z, s = w + beta s,
    p = M r + beta p, x += alpha p, r -= alpha s, w -= alpha z, m = M w; after `switch` iterations the
    Chronopoulos-Gear phases continue from (x, r, p, s, w)."""
    x = np.zeros_like(b)
    r = b.copy()
    u = Minv @ r
    w = A @ u
    m = Minv @ w
    p = np.zeros_like(b)
    s = np.zeros_like(b)
    z = np.zeros_like(b)
    st, xs = {}, []
    gam, dlt = r @ u, w @ u
    for k in range(iters):
        alpha, beta = _after(st, gam, dlt, k)
        if switch is None or k < switch:
            n = A @ m
            z = n if k == 0 else n + beta * z
            s = w if k == 0 else w + beta * s
            uu = Minv @ r
            p = uu if k == 0 else uu + beta * p
            x = x + alpha * p
            r = r - alpha * s
            w = w - alpha * z
            m = Minv @ w
            un = Minv @ r
            gam, dlt = r @ un, w @ un
        else:
            uu = Minv @ r  # u from r at the switch, as the kernel writes it
            p = uu if k == 0 else uu + beta * p
            s = w if k == 0 else w + beta * s
            x = x + alpha * p
            r = r - alpha * s
            u = Minv @ r
            w = A @ u
            gam, dlt = r @ u, w @ u
        xs.append(x.copy())
    return xs


@pytest.mark.parametrize("switch", [None, 0, 5])
def test_recurrences_give_the_pcg_iterates_in_fp64(switch):
    A, Minv, b = _system()
    ref = pcg(A, Minv, b, 25)
    for xs in (cgcg(A, Minv, b, 25), pipelined(A, Minv, b, 25, switch)):
        for k in range(25):
            assert np.linalg.norm(xs[k] - ref[k]) <= 1e-9 * np.linalg.norm(ref[k]), k


def test_pipelined_fp32_drifts_more_than_chronopoulos_gear():
    """True residual after 60 FP32 iterations on an ill-conditioned system: pipelined PCG stalls above
    Chronopoulos-Gear PCG; switching to Chronopoulos-Gear early keeps the pipelined drift small."""
    A64, M64, b64 = _system(nv=80, seed=3)
    # widen the spectrum: scale some dofs strongly (condition number ~1e6 before preconditioning)
    d = np.geomspace(1.0, 1e3, A64.shape[0])
    A64 = (A64 * d[:, None]) * d[None, :]
    M64 = np.zeros_like(A64)
    for v in range(A64.shape[0] // 3):
        sl = slice(3 * v, 3 * v + 3)
        M64[sl, sl] = np.linalg.inv(A64[sl, sl])
    A, M, b = A64.astype(np.float32), M64.astype(np.float32), b64.astype(np.float32)

    def true_res(xs):
        return np.linalg.norm(b64 - A64 @ xs[-1].astype(np.float64)) / np.linalg.norm(b64)

    r_cg = true_res(cgcg(A, M, b, 60))
    r_pipe = true_res(pipelined(A, M, b, 60))
    r_switch = true_res(pipelined(A, M, b, 60, switch=5))
    assert np.isfinite([r_cg, r_pipe, r_switch]).all()
    # measured: 1.7e-5, 1.6e-2, 9.5e-5
    assert r_pipe > 100 * r_cg
    assert r_switch < 0.1 * r_pipe
