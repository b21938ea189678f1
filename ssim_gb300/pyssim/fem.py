"""``pyssim.fem`` facade (pyssim/fem/__init__.py:7-157) over the GB300 ``libssim`` mirror.

``TetFiniteElementSolver_Cuda`` and ``TetFiniteElementSolver_Host`` keep the reference's constructor
(vertices, elements, time_step=1e-2, young_modulus=1e6, poisson_ratio=0.33, density=1e2, method) and
methods; both run on the GPU.  Extra keywords: ``precision`` and ``params``.
"""
from __future__ import annotations

from typing import Literal, Tuple

import numpy as np

from ..libssim import fem as _fem


def unit_box(nx: int, ny: int, nz: int) -> Tuple[np.ndarray, np.ndarray]:
    return _fem.unit_box(nx, ny, nz)


_METHODS = {
    "newton": _fem.tet_newton_cuda,
    "lbfgs": _fem.tet_lbfgs_cuda,
    "lbfgs_pd": _fem.tet_lbfgs_pd,
}


class TetFiniteElementSolver_Cuda:
    def __init__(
        self,
        vertices: np.ndarray,
        elements: np.ndarray,
        time_step: float = 1e-2,
        young_modulus: float = 1e6,
        poisson_ratio: float = 0.33,
        density: float = 1e2,
        method: Literal["lbfgs", "lbfgs_pd", "newton"] = "newton",
        precision: str = "fp64",
        params=None,
    ):
        if method not in _METHODS:
            raise ValueError(f"Unknown method: {method}")
        self.solver = _METHODS[method](
            vertices, elements, time_step, young_modulus, poisson_ratio, density, precision=precision, params=params
        )

    def reset(self):
        self.solver.reset()

    def prepare_step(self):
        self.solver.prepare_step()

    def compute_step(self):
        self.solver.compute_step()

    def step_next(self):
        return self.solver.step_next()

    def step(self):
        return self.solver.step()

    def mark_dirichlet(self, node_idx: int, targ_deform: np.ndarray):
        self.solver.mark_dirichlet(node_idx, targ_deform)

    def mark_dirichlet_batched(self, verts: np.ndarray, targ_deform: np.ndarray):
        self.solver.mark_dirichlet_batched(verts, targ_deform)

    def mark_general_batched(self, verts: np.ndarray):
        self.solver.mark_general_batched(verts)

    def set_rtol(self, rtol: float):
        self.solver.set_rtol(rtol)

    def add_gravity(self, gravity: np.ndarray):
        self.solver.add_gravity(gravity)

    def vertices(self) -> np.ndarray:
        return self.solver.vertices()

    def cells(self) -> np.ndarray:
        return self.solver.cells()

    def deformation(self) -> np.ndarray:
        return self.solver.deformation()

    def forces(self) -> np.ndarray:
        return self.solver.forces()

    def update_energy_and_gradients(self):
        return self.solver.update_energy_and_gradients()

    def update_hessian(self, make_spsd=True):
        self.solver.update_hessian(make_spsd)

    def update_hessian_unfiltered(self, make_spsd=True):
        self.solver.update_hessian_unfiltered(make_spsd)

    def mass_matrix(self):
        return self.solver.mass_matrix()

    def hessian(self):
        return self.solver.hessian()

    def hessian_nonzeros(self) -> np.ndarray:
        return self.solver.hessian_nonzeros()


class TetFiniteElementSolver_Host(TetFiniteElementSolver_Cuda):
    """Same interface as the reference's CPU solver class; computes on the GPU."""


def ImplicitStep():
    """The ``torch.autograd.Function`` class of a differentiable backward-Euler rollout (forward: N implicit
    steps from per-element Young's moduli and initial velocities; backward: the hand-written adjoint with
    checkpoint recomputation).  See ``rollout``."""
    from .. import adjoint

    return adjoint.implicit_rollout_function()


def rollout(E_cells, v0, engine, num_steps: int, checkpoint_every: int = 8):
    """Final displacement after ``num_steps`` implicit steps, differentiable w.r.t. E_cells [T] and v0 [V,3]
    (torch CUDA float64 tensors); ``engine`` is an ``ssim_gb300.adjoint.RolloutEngine``."""
    from .. import adjoint

    return adjoint.rollout(E_cells, v0, engine, num_steps, checkpoint_every)
