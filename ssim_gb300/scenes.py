"""Seeded synthetic workloads with the shapes, sizes and value distributions of the benchmark configs.

Each scene returns a dict with the mesh, the material, the boundary and the
time-stepping settings; ``build_timestep`` turns it into a GPU ``TimeStep`` and
the tests set the same dict up on the oracle (oracle/scenes.py).  No public dataset is involved.
"""
from __future__ import annotations

import numpy as np

from . import mesh


def cube10():
    """Plain FP64 cube: [0,1]^3, 10^3 hex x 6 tets (6,000 tets, 1,331 vertices), E=1e5, nu=0.45,
    rho=1000, top face (z=1) fixed, gravity -9.8 e_z, dt=1e-2, 10 steps, Newton + Jacobi-PCG 1e-8."""
    X, T = mesh.kuhn_box((10, 10, 10))
    return dict(
        name="cube10_kuhn_6000tets",
        X=X,
        cells=T,
        dt=1e-2,
        E=1e5,
        nu=0.45,
        rho=1000.0,
        fixed=np.where(X[:, 2] == 1.0)[0],
        gravity=(0.0, 0.0, -9.8),
        steps=10,
        u0=None,
        E_cells=None,
    )


def reference_box(nx=11):
    """The reference's own CPU scene shape (tests/fem_time_step/main.cpp:39-67) on unit_box(nx,nx,nx):
    x = 0 face fixed, gravity -9.8 on y, E=1e6, nu=0.4, rho=10, dt=1e-2."""
    X, T = mesh.unit_box(nx, nx, nx)
    return dict(
        name=f"unit_box{nx}_5tet",
        X=X,
        cells=T,
        dt=1e-2,
        E=1e6,
        nu=0.4,
        rho=10.0,
        fixed=np.where(X[:, 0] == 0.0)[0],
        gravity=(0.0, -9.8, 0.0),
        steps=10,
        u0=None,
        E_cells=None,
    )


def reference_beam(nx=6):
    """The reference's own time-step harness (tests/fem_time_step/main.cpp:39-86): unit_box(4nx, nx, nx)
    stretched 4x along x ([0,4] x [0,1]^2; nx = 6: 864 vertices, 2,875 tets), the first nx^2 vertices (the
    x = 0 face) fixed, gravity -9.8 on y, dt = 1e-2, E = 1e6, nu = 0.4, rho = 10, threshold 1e-3 (the
    reference's absolute rule), 200 steps."""
    X, T = mesh.unit_box(4 * nx, nx, nx)
    X = X.copy()
    X[:, 0] *= 4.0
    return dict(
        name=f"reference_beam_unit_box{4 * nx}x{nx}x{nx}_{T.shape[0]}tets",
        X=X,
        cells=T,
        dt=1e-2,
        E=1e6,
        nu=0.4,
        rho=10.0,
        fixed=np.arange(nx * nx),
        gravity=(0.0, -9.8, 0.0),
        steps=200,
        rtol=1e-3,
        u0=None,
        E_cells=None,
    )


def bar(nx=80, ny=20, nz=20, seed=2):
    """Single large bar: 80x20x20 hex over [0,4]x[0,1]^2 (h=0.05) x 6 = 192,000 tets; interior vertices
    jittered U(-0.1h, 0.1h) (SplitMix64 seed 2); E=1e6, nu=0.4, rho=1000; initial state stretched 1.5x
    along x (u0 = 0.5 X_x e_x); left face (x=0) fixed; dt=5e-3; 20 steps; stop at 1e-6 relative residual."""
    h = 4.0 / nx
    X, T = mesh.kuhn_box((nx, ny, nz), (4.0, ny * h, nz * h))
    X = mesh.jitter_interior(X, 0.1 * h, seed)
    u0 = np.zeros_like(X)
    u0[:, 0] = 0.5 * X[:, 0]
    return dict(
        name=f"bar_{nx}x{ny}x{nz}_{T.shape[0]}tets",
        X=X,
        cells=T,
        dt=5e-3,
        E=1e6,
        nu=0.4,
        rho=1000.0,
        fixed=np.where(X[:, 0] == 0.0)[0],
        gravity=(0.0, 0.0, 0.0),
        steps=20,
        u0=u0,
        E_cells=None,
    )


def beam(nx=100, ny=50, nz=34, h=0.02, seed=3):
    """1.02M-tet beam: 100x50x34 hex (h=0.02, [0,2]x[0,1]x[0,0.68]) x 6 tets; per-cell E log-uniform in
    [1e4, 1e6] (SplitMix64 seed 3), nu=0.45, rho=1000; left face (x=0) fixed; gravity -9.8 e_z; dt=1e-2."""
    X, T = mesh.kuhn_box((nx, ny, nz), (nx * h, ny * h, nz * h))
    E_cells = 10.0 ** mesh.uniform(seed, T.shape[0], 4.0, 6.0)
    return dict(
        name=f"beam_{nx}x{ny}x{nz}_{T.shape[0]}tets",
        X=X,
        cells=T,
        dt=1e-2,
        E=1e5,
        nu=0.45,
        rho=1000.0,
        fixed=np.where(X[:, 0] == 0.0)[0],
        gravity=(0.0, 0.0, -9.8),
        steps=10,
        u0=None,
        E_cells=E_cells,
    )


def cloth_springs(n):
    """Spring list of an n x n vertex grid (vertex (i, j) = i * n + j): structural (grid edges,
    2 n (n-1)), shear (both quad diagonals, 2 (n-1)^2) and bend (every second vertex along the rows and
    columns, 2 n (n-2)) springs, in that order."""
    idx = np.arange(n * n, dtype=np.int32).reshape(n, n)
    parts = [
        (idx[:, :-1], idx[:, 1:]),  # structural, along j
        (idx[:-1, :], idx[1:, :]),  # structural, along i
        (idx[:-1, :-1], idx[1:, 1:]),  # shear
        (idx[:-1, 1:], idx[1:, :-1]),  # shear
        (idx[:, :-2], idx[:, 2:]),  # bend, along j
        (idx[:-2, :], idx[2:, :]),  # bend, along i
    ]
    return np.concatenate([np.stack([a.reshape(-1), b.reshape(-1)], axis=1) for a, b in parts]).astype(np.int32)


def cloth(n=512, h=0.01, k=1e3, areal_density=0.5, dt=1e-2, steps=10):
    """Mass-spring cloth: n x n vertex grid in the z = 0 plane with spacing h (512^2 vertices, h = 1 cm:
    a 5.11 m square sheet), structural + shear + bend springs (1,567,746 for n = 512) of stiffness k = 1e3
    N/m, rest lengths from the grid, lumped vertex masses areal_density x h^2 (0.5 kg/m^2, a heavy fabric),
    the four corners pinned, gravity -9.8 e_z, dt = 1e-2 s, 10 steps."""
    g = np.arange(n, dtype=np.float64) * h
    X = np.zeros((n * n, 3))
    X[:, 0] = np.repeat(g, n)
    X[:, 1] = np.tile(g, n)
    S = cloth_springs(n)
    return dict(
        name=f"cloth_{n}x{n}_{S.shape[0]}springs",
        X=X,
        cells=S,
        springs=True,
        k=k,
        vertex_mass=np.full(n * n, areal_density * h * h),
        dt=dt,
        fixed=np.array([0, n - 1, n * (n - 1), n * n - 1]),
        gravity=(0.0, 0.0, -9.8),
        steps=steps,
        u0=None,
        E_cells=None,
    )


def sheet2d(nx=41, ny=21, E=1e5, nu=0.4, rho=100.0, seed=7):
    """2D sheet: unit_square(nx, ny) scaled to [0, 2] x [0, 1] with interior vertices jittered by
    U(-0.1h, 0.1h) (SplitMix64 seed 7), x = 0 edge fixed, gravity -9.8 e_y, dt = 1e-2, 10 steps."""
    X2, T = mesh.unit_square(nx, ny)
    X2 = X2 * np.array([2.0, 1.0])
    h = 1.0 / (ny - 1)
    inner = (X2[:, 0] > 0) & (X2[:, 0] < 2.0) & (X2[:, 1] > 0) & (X2[:, 1] < 1.0)
    jit = (mesh.uniform(seed, 2 * X2.shape[0], -0.1 * h, 0.1 * h)).reshape(-1, 2)
    X2 = X2 + jit * inner[:, None]
    return dict(
        name=f"sheet2d_{nx}x{ny}_{T.shape[0]}tris",
        X=np.concatenate([X2, np.zeros((X2.shape[0], 1))], axis=1),
        X2=X2,
        cells=T,
        tri2d=True,
        dt=1e-2,
        E=E,
        nu=nu,
        rho=rho,
        fixed=np.where(X2[:, 0] == 0.0)[0],
        gravity=(0.0, -9.8, 0.0),
        steps=10,
        u0=None,
        E_cells=None,
    )


def build_timestep(scene, precision="fp64", stepper="newton", params=None, rtol=None):
    """A GPU TimeStep set up for ``scene`` (material, Dirichlet face, gravity, initial state)."""
    from .timestep import TimeStep

    if scene.get("springs"):
        ts = TimeStep.springs(scene["X"], scene["cells"], scene["k"], vertex_mass=scene["vertex_mass"],
                              time_step=scene["dt"])
    elif scene.get("tri2d"):
        ts = TimeStep.tri2d(scene["X2"], scene["cells"], scene["dt"], scene["E"], scene["nu"], scene["rho"])
    else:
        ts = TimeStep(scene["X"], scene["cells"], scene["dt"], scene["E"], scene["nu"], scene["rho"])
    ts.set_precision(precision)
    if scene.get("E_cells") is not None:
        ts.set_material(scene["E_cells"], scene.get("nu_cells"))
    if len(scene["fixed"]):
        ts.mark_dirichlet_batched(scene["fixed"], np.zeros((len(scene["fixed"]), 3)))
    if any(scene["gravity"]):
        ts.add_gravity(scene["gravity"])
    if rtol is not None:
        ts.set_threshold(rtol)
    if params is not None:
        ts.set_params(params)
    ts.reset(stepper)
    if scene.get("u0") is not None:
        ts.set("deformation", scene["u0"])
        ts.set("prev_deform", scene["u0"])
    if scene.get("velocity") is not None:
        ts.set("velocity", scene["velocity"])
    return ts


def batch_cubes(n=256, kmin=4, kmax=24, seed=4, dt=1e-2, rho=1000.0):
    """Batched instances: n unit cubes with per-side hex counts k ~ U{kmin..kmax} (6 tets per hex), E
    log-uniform in [1e4, 1e6], nu ~ U[0.3, 0.48] and one initial velocity per cube with N(0, 0.5^2)
    components (SplitMix64 stream ``seed``); bottom face (z = 0) fixed; no gravity; dt = 1e-2."""
    ks = kmin + np.floor(mesh.uniform(seed, n, 0.0, 1.0) * (kmax - kmin + 1)).astype(int)
    E = 10.0 ** mesh.uniform(seed, n, 4.0, 6.0, offset=n)
    nu = mesh.uniform(seed, n, 0.3, 0.48, offset=2 * n)
    v0 = 0.5 * mesh.normal(seed, 3 * n, offset=3 * n).reshape(n, 3)
    Xs, Ts, voff, E_cells, nu_cells, fixed, vel = [], [], [0], [], [], [], []
    for i, k in enumerate(ks):
        X, T = mesh.kuhn_box((int(k), int(k), int(k)))
        Ts.append(T + voff[-1])
        Xs.append(X)
        fixed.append(np.where(X[:, 2] == 0.0)[0] + voff[-1])
        vel.append(np.tile(v0[i], (X.shape[0], 1)))
        E_cells.append(np.full(T.shape[0], E[i]))
        nu_cells.append(np.full(T.shape[0], nu[i]))
        voff.append(voff[-1] + X.shape[0])
    return dict(
        name=f"batch{n}_cubes_k{kmin}-{kmax}",
        X=np.concatenate(Xs), cells=np.concatenate(Ts).astype(np.int32), vertex_offsets=np.array(voff, dtype=np.int32),
        k=ks, E_inst=E, nu_inst=nu, v0_inst=v0, E_cells=np.concatenate(E_cells), nu_cells=np.concatenate(nu_cells),
        fixed=np.concatenate(fixed), velocity=np.concatenate(vel), dt=dt, E=1e5, nu=0.4, rho=rho,
        gravity=(0.0, 0.0, 0.0), steps=10, u0=None,
    )


def rollout_cube(n=32, seed=5, v0_seed=6):
    """Differentiable rollout: [0,1]^3 with n^3 hex x 6 tets (n = 32: 196,608 tets), per-cell E log-uniform
    in [1e4, 1e6] (SplitMix64 seed 5), nu = 0.45, rho = 1000, bottom face (z = 0) fixed, initial vertex
    velocities N(0, 0.5^2) per component (seed 6, zero on the fixed face), dt = 1e-2, 40 steps; the loss
    target is the rest shape displaced by 0.1 sin(2 pi x) e_z."""
    X, T = mesh.kuhn_box((n, n, n))
    fixed = np.where(X[:, 2] == 0.0)[0]
    v0 = 0.5 * mesh.normal(v0_seed, X.size).reshape(X.shape)
    v0[fixed] = 0.0
    target = X.copy()
    target[:, 2] += 0.1 * np.sin(2 * np.pi * X[:, 0])
    return dict(
        name=f"rollout_cube{n}_{T.shape[0]}tets", X=X, cells=T, fixed=fixed, dt=1e-2, nu=0.45, rho=1000.0,
        E_cells=10.0 ** mesh.uniform(seed, T.shape[0], 4.0, 6.0), v0=v0, target=target, steps=40,
        checkpoint_every=8,
    )


def build_batch_timestep(batch, precision="mixed", params=None):
    """One GPU TimeStep over the disjoint union of the batch's cubes (per-cell material, per-instance
    stopping test)."""
    from .timestep import TimeStep

    ts = TimeStep(batch["X"], batch["cells"], batch["dt"], batch["E"], batch["nu"], batch["rho"])
    ts.set_precision(precision)
    ts.set_material(batch["E_cells"], batch["nu_cells"])
    ts.mark_dirichlet_batched(batch["fixed"], np.zeros((len(batch["fixed"]), 3)))
    ts.set_instances(batch["vertex_offsets"])
    if params is not None:
        ts.set_params(params)
    ts.reset("newton")
    ts.set("velocity", batch["velocity"])
    return ts
