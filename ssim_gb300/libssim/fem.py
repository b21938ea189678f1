"""``libssim.fem`` classes (bindings/src/fem_host.cpp:178-226, bindings/src/fem_cuda.cu:209-250) on the GPU.

The reference binds one wrapper class per stepper; the ``_cuda`` names run on the GPU with cuBLAS /
cuSPARSE and the plain names on the CPU.  Here every class runs on the GB300 kernels (there is no CPU
path); the plain names are kept so scripts written for either flavour run unchanged.  Constructor:
``(vert [V,3] float64, cell [T,4] int32, time_step, youngs_modulus, poisson_ratio, density)`` plus the
keyword extensions ``precision`` ("fp64" | "mixed") and ``params`` (solver settings).
"""
from __future__ import annotations

import time

import numpy as np

from .. import mesh as _mesh
from ..timestep import TimeStep


def unit_box(nx: int, ny: int, nz: int):
    """fem_host.cpp:216-219: (vertices [3, V], cells [4, T]) of ssim::mesh::unit_box."""
    X, T = _mesh.unit_box(nx, ny, nz)
    return np.ascontiguousarray(X.T), np.ascontiguousarray(T.T)


class _TimeStepWrapper:
    """timestep_wrapper / timestep_wrapper_cuda (fem_host.cpp:70-172, fem_cuda.cu:61-169)."""

    _stepper = "newton"

    def __init__(self, vert, cell, time_step, youngs_modulus, poisson_ratio, density, precision="fp64", params=None):
        vert = np.asarray(vert)
        cell = np.asarray(cell)
        if vert.ndim != 2 or vert.shape[1] != 3 or vert.dtype != np.float64:
            raise TypeError("vert must be a float64 array of shape [V, 3]")
        if cell.ndim != 2 or cell.shape[1] != 4 or cell.dtype != np.int32:
            raise TypeError("cell must be an int32 array of shape [T, 4]")
        self.step_ = TimeStep(vert, cell, time_step, youngs_modulus, poisson_ratio, density)
        self.step_.set_precision(precision)
        if params is not None:
            self.step_.set_params(params)
        self.has_reset_ = False

    def reset(self):
        self.step_.reset(self._stepper)
        self.has_reset_ = True

    def prepare_step(self):
        if not self.has_reset_:
            self.step_.reset(self._stepper)
            print("Warning: prepare_step() called before reset(), bad logic.", flush=True)
            self.has_reset_ = True
        self.step_.prepare_step()

    def compute_step(self):
        self.step_.compute_step()

    def step_next(self):
        self.step_.step_next()

    def step(self) -> float:
        """prepare + compute + next; returns the wall time in milliseconds (fem_host.cpp:102-111)."""
        t0 = time.perf_counter()
        self.prepare_step()
        self.compute_step()
        self.step_next()
        self.step_.synchronize()
        return (time.perf_counter() - t0) * 1e3

    def mark_dirichlet(self, node_idx, targ_deform):
        self.step_.mark_dirichlet_batched(np.array([node_idx]), np.asarray(targ_deform, dtype=np.float64).reshape(1, 3))

    def mark_dirichlet_batched(self, verts, targ_deform):
        """targ_deform is [3, n] as the reference takes it (an Eigen::Matrix3Xd)."""
        t = np.asarray(targ_deform, dtype=np.float64)
        v = np.asarray(verts).reshape(-1)
        if t.shape != (3, v.size):
            raise ValueError("targ_deform must have shape [3, len(verts)]")
        self.step_.mark_dirichlet_batched(v, np.ascontiguousarray(t.T))

    def mark_general_batched(self, verts):
        self.step_.mark_general_batched(verts)

    def set_rtol(self, rtol):
        self.step_.set_threshold(rtol)

    def add_gravity(self, gravity):
        self.step_.add_gravity(gravity)

    # The getters return [3, V] / [4, T] arrays with the memory of the reference's Eigen Matrix3Xd /
    # Matrix4Xi results (column-major: one vertex's x, y, z adjacent), i.e. the transposed view of a fresh
    # [V, 3] copy: no second copy per call.
    def vertices(self):
        return self.step_.vertices().T

    def cells(self):
        return self.step_.cells().T

    def deformation(self):
        return self.step_.deformation().T

    def forces(self):
        return self.step_.forces().T

    def update_energy_and_gradients(self):
        return self.step_.update_energy_and_gradients(True)

    def update_hessian(self, make_spsd=True):
        self.step_.update_hessian(False, make_spsd, True)

    def update_hessian_unfiltered(self, make_spsd=True):
        self.step_.update_hessian(False, make_spsd, False)

    def mass_matrix(self):
        return self.step_.matrix("mass")

    def hessian(self):
        return self.step_.matrix("sysmatrix")

    def hessian_nonzeros(self):
        return self.step_.values("sysmatrix")


class tet_newton_cuda(_TimeStepWrapper):
    _stepper = "newton"


class tet_newton(_TimeStepWrapper):
    _stepper = "newton"


class tet_lbfgs_cuda(_TimeStepWrapper):
    _stepper = "lbfgs"


class tet_lbfgs(_TimeStepWrapper):
    _stepper = "lbfgs"


class tet_lbfgs_pd(_TimeStepWrapper):
    _stepper = "pd"


class tet_ncg_cuda_ext_ai(_TimeStepWrapper):
    """timestep_ncg (fem_cuda.cu:171-207): nonlinear CG preconditioned by x = L L^T g, L on the system
    matrix's CSR pattern; reset() installs L = I, set_matrix(values) sets its nonzeros (CSR order of
    ``hessian()``)."""

    _stepper = "ncg_ext"

    def set_matrix(self, values):
        v = np.asarray(values)
        if v.dtype != np.float64 or v.ndim != 1:
            raise TypeError("values must be a float64 vector")  # nb::arg().noconvert() in the reference
        self.step_.set_ncg_matrix(v)
