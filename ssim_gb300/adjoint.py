"""Differentiable backward-Euler rollouts: a torch.autograd.Function over the GPU time step.

Forward: N steps from rest with per-cell Young's modulus E and initial vertex velocities v0, checkpointing
(u_n, v_n) every ``checkpoint_every`` steps.  Backward: segment by segment from the last, restore the
checkpoint, recompute the segment's states, then run ssim_gb_adjoint_step (the hand-written adjoint of the
implicit step, kernels_adjoint.cu) from the segment's last step to its first.  The gradients returned are
dL/dE (per cell) and dL/dv0 (per vertex).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .timestep import TimeStep


class RolloutEngine:
    """A GPU time step configured for a scene whose material and initial velocity are the inputs."""

    def __init__(self, X, cells, fixed, dt=1e-2, nu=0.45, rho=1000.0, gravity=(0.0, 0.0, 0.0), precision="fp64",
                 params=None, adjoint_rtol=1e-10, adjoint_max_iters=20000):
        self.ts = TimeStep(X, cells, dt, 1e5, nu, rho)
        self.ts.set_precision(precision)
        self.fixed = np.asarray(fixed, dtype=np.int32)
        if self.fixed.size:
            self.ts.mark_dirichlet_batched(self.fixed, np.zeros((self.fixed.size, 3)))
        if any(gravity):
            self.ts.add_gravity(gravity)
        if params is not None:
            self.ts.set_params(params)
        self.nu = nu
        self.num_cells = cells.shape[0]
        self.num_vertices = X.shape[0]
        self.adjoint_rtol = adjoint_rtol
        self.adjoint_max_iters = adjoint_max_iters
        self.cg_iters = 0
        self.projected = 0

    def _field_out(self, name, t):
        self.ts._c(self.ts._L.ssim_gb_get_field_device(self.ts._h, _lib.FIELDS[name], C.c_void_p(t.data_ptr())))

    def _field_in(self, name, t):
        self.ts._c(self.ts._L.ssim_gb_set_field_device(self.ts._h, _lib.FIELDS[name], C.c_void_p(t.data_ptr())))

    def start(self, E_cells, v0):
        import torch

        self.ts.set_material(np.asarray(E_cells.detach().cpu().numpy(), dtype=np.float64), None)
        self.ts.reset("newton")
        z = torch.zeros((self.num_vertices, 3), dtype=torch.float64, device="cuda")
        for f in ("deformation", "prev_deform"):
            self._field_in(f, z)
        self._field_in("velocity", v0.detach().to(torch.float64).contiguous())

    def state(self):
        import torch

        u = torch.empty((self.num_vertices, 3), dtype=torch.float64, device="cuda")
        v = torch.empty_like(u)
        self._field_out("deformation", u)
        self._field_out("velocity", v)
        return u, v

    def restore(self, u, v):
        self._field_in("deformation", u)
        self._field_in("prev_deform", u)
        self._field_in("velocity", v)

    def step(self):
        self.ts.step()

    def adjoint_step(self, u_next, ubar, vbar, ebar):
        self._field_in("next_deform", u_next)
        it, proj = C.c_int32(), C.c_int32()
        self.ts._c(
            self.ts._L.ssim_gb_adjoint_step(
                self.ts._h, C.c_void_p(ubar.data_ptr()), C.c_void_p(vbar.data_ptr()), C.c_void_p(ebar.data_ptr()),
                self.adjoint_rtol, self.adjoint_max_iters, C.byref(it), C.byref(proj),
            )
        )
        self.cg_iters += it.value
        self.projected += proj.value


def _function():
    import torch

    class ImplicitRollout(torch.autograd.Function):
        """u_N = rollout(E, v0): N backward-Euler steps; backward by the adjoint with checkpoints."""

        @staticmethod
        def forward(ctx, E_cells, v0, engine, num_steps, checkpoint_every):
            engine.start(E_cells, v0)
            ckpts = []
            for n in range(num_steps):
                if n % checkpoint_every == 0:
                    ckpts.append(engine.state())
                engine.step()
            u_final, _ = engine.state()
            ctx.engine, ctx.ckpts, ctx.n, ctx.k = engine, ckpts, num_steps, checkpoint_every
            return u_final

        @staticmethod
        def backward(ctx, grad_u):
            eng, n_steps, k = ctx.engine, ctx.n, ctx.k
            ubar = grad_u.detach().to(torch.float64).contiguous().clone()
            vbar = torch.zeros_like(ubar)
            ebar = torch.zeros(eng.num_cells, dtype=torch.float64, device="cuda")
            for s in reversed(range(len(ctx.ckpts))):
                s0, s1 = s * k, min(s * k + k, n_steps)
                eng.restore(*ctx.ckpts[s])
                states = []
                for _ in range(s0, s1):
                    eng.step()
                    states.append(eng.state()[0])
                for j in reversed(range(s1 - s0)):
                    eng.adjoint_step(states[j], ubar, vbar, ebar)
            return ebar, vbar, None, None, None

    return ImplicitRollout


_FN = None


def implicit_rollout_function():
    """The autograd Function class behind ``rollout`` (created on first use: torch is imported lazily)."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN


def rollout(E_cells, v0, engine: RolloutEngine, num_steps: int, checkpoint_every: int = 8):
    """Final displacement u_N [V,3] (torch, cuda, float64), differentiable w.r.t. E_cells and v0."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(E_cells, v0, engine, num_steps, checkpoint_every)
