"""Python view of one GPU time-step object (ssim::fem::basic_time_step, time_step.hpp:168-715).

Method names follow the reference class; arrays cross the boundary as host
numpy copies in the reference's layouts ([V,3] float64 fields, [T,4] int32
cells, scipy CSR matrices).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, dptr, iptr


class TimeStep:
    """basic_time_step<double, cuda, 3, 4, stable_neohookean, ...> on the GPU.

    Construction mirrors ``basic_time_step(mesh, dt=1e-3, E=1e6, nu=0.33, rho=1e3)``
    (time_step.hpp:260-265) and runs ``reset()``.  ``precision`` selects the
    Hessian / assembly / inner-PCG arithmetic: "fp64" (the reference's) or
    "mixed" (FP32 there, FP64 energy, gradient, state and reductions).
    """

    def __init__(self, vertices, cells, time_step=1e-3, youngs=1e6, poisson=0.33, density=1e3, precision="fp64"):
        L = _lib.lib()
        self._L = L
        X = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        T = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1, 4)
        self.num_vertices, self.num_cells = X.shape[0], T.shape[0]
        self.n = 3 * self.num_vertices
        h = C.c_void_p()
        check(
            L.ssim_gb_create(dptr(X), X.shape[0], iptr(T), T.shape[0], time_step, youngs, poisson, density, C.byref(h))
        )
        self._h = h
        self._X, self._cells = X, T
        self._stepper = _lib.STEPPER_NONE
        if precision != "fp64":
            self.set_precision(precision)
            self.reset()

    @classmethod
    def tri2d(cls, vertices, triangles, time_step, youngs, poisson, density, precision="fp64"):
        """2D triangles in the plane (ssim_gb_create_2d): vertices [V, 2], triangles [T, 3].  Fields stay
        [V, 3] with z identically zero; csr_2d() gives the reference's 2-dof matrices."""
        self = cls.__new__(cls)
        L = _lib.lib()
        self._L = L
        X2 = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 2)
        T = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
        self.num_vertices, self.num_cells = X2.shape[0], T.shape[0]
        self.n = 3 * self.num_vertices
        h = C.c_void_p()
        check(L.ssim_gb_create_2d(dptr(X2), X2.shape[0], iptr(T), T.shape[0], time_step, youngs, poisson, density,
                                  C.byref(h)))
        self._h = h
        self._X = np.concatenate([X2, np.zeros((X2.shape[0], 1))], axis=1)
        self._cells = T
        self._stepper = _lib.STEPPER_NONE
        if precision != "fp64":
            self.set_precision(precision)
            self.reset()
        return self

    @property
    def dim(self) -> int:
        d = C.c_int32()
        self._c(self._L.ssim_gb_get_dim(self._h, C.byref(d)))
        return d.value

    def csr_2d(self, which="sysmatrix"):
        """(row_ptr [2V+1], col_idx, values) of a 2D handle's matrix in the reference's 2-dof layout."""
        nnz2 = self.nnz * 4 // 9
        rp = np.zeros(2 * self.num_vertices + 1, dtype=np.int32)
        ci = np.zeros(nnz2, dtype=np.int32)
        v = np.zeros(nnz2)
        self._c(self._L.ssim_gb_get_csr_2d(self._h, _lib.MATRICES[which], iptr(rp), iptr(ci), dptr(v)))
        return rp, ci, v

    @classmethod
    def springs(cls, vertices, springs, stiffness, vertex_mass=None, mass=None, time_step=1e-2, precision="fp64"):
        """A mass-spring system (ssim_gb_create_springs): springs [S, 2] vertex pairs (rest lengths from the
        vertices), uniform stiffness, vertex masses [V] (or one mass for all)."""
        self = cls.__new__(cls)
        L = _lib.lib()
        self._L = L
        X = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        Sp = np.ascontiguousarray(springs, dtype=np.int32).reshape(-1, 2)
        self.num_vertices, self.num_cells = X.shape[0], Sp.shape[0]
        self.n = 3 * self.num_vertices
        m = None
        if vertex_mass is not None:
            m = np.ascontiguousarray(vertex_mass, dtype=np.float64).reshape(-1)
            if m.size != X.shape[0]:
                raise ValueError("vertex_mass must have one entry per vertex")
        h = C.c_void_p()
        check(
            L.ssim_gb_create_springs(dptr(X), X.shape[0], iptr(Sp), Sp.shape[0], stiffness,
                                     dptr(m) if m is not None else None, mass if mass is not None else 0.0,
                                     time_step, C.byref(h))
        )
        self._h = h
        self._X, self._cells = X, Sp
        self._stepper = _lib.STEPPER_NONE
        if precision != "fp64":
            self.set_precision(precision)
            self.reset()
        return self

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.ssim_gb_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, status):
        check(status, self._h)

    # ---------------------------------------------------------------- configuration
    def set_precision(self, precision):
        p = {"fp64": _lib.FP64, "mixed": _lib.MIXED}[precision] if isinstance(precision, str) else int(precision)
        self._c(self._L.ssim_gb_set_precision(self._h, p))
        return self

    def set_time_step(self, v):
        self._c(self._L.ssim_gb_set_time_step(self._h, v))
        return self

    def set_youngs(self, v):
        self._c(self._L.ssim_gb_set_youngs(self._h, v))
        return self

    def set_poisson(self, v):
        self._c(self._L.ssim_gb_set_poisson(self._h, v))
        return self

    def set_density(self, v):
        self._c(self._L.ssim_gb_set_density(self._h, v))
        return self

    def set_damping(self, v):
        self._c(self._L.ssim_gb_set_damping(self._h, v))
        return self

    def set_threshold(self, v):
        self._c(self._L.ssim_gb_set_threshold(self._h, v))
        return self

    def set_material(self, youngs=None, poisson=None):
        self._Em = None if youngs is None else np.ascontiguousarray(youngs, dtype=np.float64).reshape(-1)
        self._nm = None if poisson is None else np.ascontiguousarray(poisson, dtype=np.float64).reshape(-1)
        for a in (self._Em, self._nm):
            if a is not None and a.size != self.num_cells:
                raise ValueError("per-cell material arrays must have one entry per cell")
        pe = None if self._Em is None else dptr(self._Em)
        pn = None if self._nm is None else dptr(self._nm)
        self._c(self._L.ssim_gb_set_material(self._h, pe, pn))
        return self

    @property
    def params(self) -> _lib.Params:
        p = _lib.Params()
        self._c(self._L.ssim_gb_get_params(self._h, C.byref(p)))
        return p

    def set_params(self, params: _lib.Params | None = None, **kw):
        p = params if params is not None else self.params
        for k, v in kw.items():
            if not hasattr(p, k):
                raise KeyError(f"unknown solver parameter {k!r}")
            setattr(p, k, v)
        self._c(self._L.ssim_gb_set_params(self._h, C.byref(p)))
        return self

    def set_stream(self, stream_handle: int | None):
        self._c(self._L.ssim_gb_set_stream(self._h, stream_handle))

    # ---------------------------------------------------------------- boundary
    def mark_dirichlet_batched(self, verts, targ_deform=None):
        """Dirichlet dofs at ``verts`` with targets [n,3] (or [3,n] as the reference binding takes)."""
        v = np.ascontiguousarray(verts, dtype=np.int32).reshape(-1)
        if targ_deform is None:
            t = np.zeros((v.size, 3))
        else:
            t = np.asarray(targ_deform, dtype=np.float64)
            if t.shape == (3, v.size) and v.size != 3:
                t = t.T
            t = np.ascontiguousarray(t).reshape(v.size, 3)
        self._c(self._L.ssim_gb_mark_dirichlet_batched(self._h, iptr(v), v.size, dptr(t)))

    def mark_general_batched(self, verts):
        v = np.ascontiguousarray(verts, dtype=np.int32).reshape(-1)
        self._c(self._L.ssim_gb_mark_general_batched(self._h, iptr(v), v.size))

    def set_dof_type(self, types):
        t = np.ascontiguousarray(types, dtype=np.int8).reshape(-1)
        if t.size != self.n:
            raise ValueError("dof types must be [V,3]")
        self._c(self._L.ssim_gb_set_dof_type(self._h, t.ctypes.data_as(C.POINTER(C.c_int8))))

    def dof_type(self):
        t = np.zeros(self.n, dtype=np.int8)
        self._c(self._L.ssim_gb_get_dof_type(self._h, t.ctypes.data_as(C.POINTER(C.c_int8))))
        return t.reshape(-1, 3)

    def add_ext_force_dof(self, dof, accel):
        self._c(self._L.ssim_gb_add_ext_force_dof(self._h, int(dof), float(accel)))

    def add_gravity(self, g):
        g = np.ascontiguousarray(g, dtype=np.float64).reshape(3)
        self._c(self._L.ssim_gb_add_gravity(self._h, dptr(g)))

    # ---------------------------------------------------------------- loop
    def reset(self, stepper: int | str | None = None):
        if isinstance(stepper, str):
            stepper = {"newton": 0, "lbfgs": 1, "pd": 2, "none": 3, "forward_euler": 4, "h0": 5, "ncg": 6,
                       "ncg_ext": 7}[stepper]
        if stepper is not None:
            self._stepper = int(stepper)
        self._c(self._L.ssim_gb_reset(self._h, self._stepper))

    def prepare_step(self):
        self._c(self._L.ssim_gb_prepare_step(self._h))

    def compute_step(self) -> float:
        r = C.c_double()
        self._c(self._L.ssim_gb_compute_step(self._h, C.byref(r)))
        return r.value

    def step_next(self):
        self._c(self._L.ssim_gb_step_next(self._h))

    def step(self) -> float:
        ms = C.c_double()
        self._c(self._L.ssim_gb_step(self._h, C.byref(ms)))
        return ms.value

    def restore(self):
        self._c(self._L.ssim_gb_restore(self._h))

    def stats(self) -> dict:
        s = _lib.StepStats()
        self._c(self._L.ssim_gb_get_step_stats(self._h, C.byref(s)))
        return s.as_dict()

    def set_elastic_model(self, model: str | int):
        """"stable_neohookean" (default) or "linear": the reference's ElastModel template argument."""
        self._c(self._L.ssim_gb_set_elastic_model(self._h, _lib.MODELS.get(model, model)))

    def set_ncg_matrix(self, values=None):
        """Values of the NCG preconditioner factor L (x = L L^T g) in the CSR order of ``csr_pattern``;
        None restores the identity."""
        if values is None:
            self._c(self._L.ssim_gb_set_ncg_matrix(self._h, None))
            return
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if v.size != self.nnz:
            raise ValueError(f"expected {self.nnz} values, got {v.size}")
        self._c(self._L.ssim_gb_set_ncg_matrix(self._h, dptr(v)))

    def solve_log(self) -> list[int]:
        """PCG iterations of every solve since the last reset."""
        n = C.c_int32()
        self._c(self._L.ssim_gb_get_solve_log(self._h, None, 0, C.byref(n)))
        buf = np.zeros(max(1, n.value), dtype=np.int32)
        self._c(self._L.ssim_gb_get_solve_log(self._h, iptr(buf), n.value, C.byref(n)))
        return buf[: n.value].tolist()

    def check_convergence(self) -> bool:
        c = C.c_int32()
        self._c(self._L.ssim_gb_check_convergence(self._h, C.byref(c)))
        return bool(c.value)

    @property
    def threshold_abs(self) -> float:
        v = C.c_double()
        self._c(self._L.ssim_gb_threshold_abs(self._h, C.byref(v)))
        return v.value

    def synchronize(self):
        self._c(self._L.ssim_gb_synchronize(self._h))

    # ---------------------------------------------------------------- energy / Hessian
    def update_energy_and_gradients(self, is_deform_grad_updated=False) -> float:
        e = C.c_double()
        self._c(self._L.ssim_gb_update_energy_and_gradients(self._h, int(is_deform_grad_updated), C.byref(e)))
        return e.value

    def update_hessian(self, is_deform_grad_updated=False, make_spsd=False, filter_dbc=True):
        self._c(self._L.ssim_gb_update_hessian(self._h, int(is_deform_grad_updated), int(make_spsd), int(filter_dbc)))

    def energy_at(self, deform) -> float:
        u = np.ascontiguousarray(deform, dtype=np.float64).reshape(-1)
        e = C.c_double()
        self._c(self._L.ssim_gb_energy_at(self._h, dptr(u), C.byref(e)))
        return e.value

    # ---------------------------------------------------------------- state
    def get(self, field: str) -> np.ndarray:
        out = np.empty(self.n)
        self._c(self._L.ssim_gb_get_field(self._h, _lib.FIELDS[field], dptr(out)))
        return out.reshape(-1, 3)

    def set(self, field: str, value):
        v = np.ascontiguousarray(value, dtype=np.float64).reshape(-1)
        if v.size != self.n:
            raise ValueError(f"{field} must be [V,3]")
        self._c(self._L.ssim_gb_set_field(self._h, _lib.FIELDS[field], dptr(v)))

    def device_ptr(self, field: str) -> int:
        p = C.c_void_p()
        self._c(self._L.ssim_gb_field_device_ptr(self._h, _lib.FIELDS[field], C.byref(p)))
        return p.value

    def deformation(self):
        return self.get("deformation")

    def forces(self):
        return self.get("forces")

    def vertices(self):
        return self._X.copy()

    def cells(self):
        return self._cells.copy()

    @property
    def nnz(self) -> int:
        v = C.c_int64()
        self._c(self._L.ssim_gb_sizes(self._h, None, None, None, C.byref(v)))
        return v.value

    def csr_pattern(self):
        rp = np.zeros(self.n + 1, dtype=np.int32)
        ci = np.zeros(self.nnz, dtype=np.int32)
        self._c(self._L.ssim_gb_get_csr_pattern(self._h, iptr(rp), iptr(ci)))
        return rp, ci

    def values(self, which="sysmatrix") -> np.ndarray:
        out = np.zeros(self.nnz)
        self._c(self._L.ssim_gb_get_matrix_values(self._h, _lib.MATRICES[which], dptr(out)))
        return out

    def matrix(self, which="sysmatrix"):
        import scipy.sparse as sp

        rp, ci = self.csr_pattern()
        return sp.csr_matrix((self.values(which), ci, rp), shape=(self.n, self.n))

    def rest_volume(self) -> np.ndarray:
        out = np.zeros(self.num_cells)
        self._c(self._L.ssim_gb_get_rest_volume(self._h, dptr(out)))
        return out

    def dminv(self) -> np.ndarray:
        d = self.dim
        out = np.zeros(self.num_cells * d * d)
        self._c(self._L.ssim_gb_get_dminv(self._h, dptr(out)))
        return out.reshape(-1, d, d)

    def spmv(self, x, which="sysmatrix") -> np.ndarray:
        xv = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        y = np.zeros(self.n)
        self._c(self._L.ssim_gb_spmv(self._h, _lib.MATRICES[which], dptr(xv), dptr(y)))
        return y.reshape(-1, 3)

    def pcg(self, b, rtol=1e-8, max_iters=10000):
        bv = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
        x = np.zeros(self.n)
        it, rr = C.c_int32(), C.c_double()
        self._c(self._L.ssim_gb_pcg(self._h, dptr(bv), dptr(x), rtol, max_iters, C.byref(it), C.byref(rr)))
        return x.reshape(-1, 3), it.value, rr.value

    # ---------------------------------------------------------------- batched instances
    def set_instances(self, vertex_offsets):
        off = np.ascontiguousarray(vertex_offsets, dtype=np.int32).reshape(-1)
        self._c(self._L.ssim_gb_set_instances(self._h, iptr(off), off.size - 1))
        self._ninst = off.size - 1

    def instance_residuals(self):
        g = np.zeros(self._ninst)
        g0 = np.zeros(self._ninst)
        self._c(self._L.ssim_gb_get_instance_residuals(self._h, dptr(g), dptr(g0)))
        return g, g0

    # ---------------------------------------------------------------- profiling
    def autotune(self) -> dict:
        """One-time sweep of launch shapes on this handle's data (ssim_gb_autotune): block sizes of the element
        pass, the Hessian, the assembly and the gather, the PCG variant and grid, fused or two-kernel assembly;
        the fastest is applied and cached for the process by problem shape.  Returns the chosen shapes and
        their timings."""
        t = _lib.Tuning()
        self._c(self._L.ssim_gb_autotune(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, tuning: dict):
        """Applies a tuning found earlier (ssim_gb_set_tuning): the shape and PCG keys of an autotune() result;
        missing keys are 0 (the compiled defaults, the two-launch or standard PCG, unfused assembly, the FP32
        matrix in every solve)."""
        t = _lib.Tuning()
        for k in ("elem_block", "hessian_block", "assembly_block", "gather_block", "pcg_persistent",
                  "pcg_max_blocks", "fused_assembly", "pcg_half_matrix", "elem_regcap"):
            setattr(t, k, int(tuning.get(k, 0)))
        self._c(self._L.ssim_gb_set_tuning(self._h, C.byref(t)))

    def profile(self, enable: bool = True):
        self._c(self._L.ssim_gb_profile_enable(self._h, int(enable)))

    def profile_read(self, kernel: str = "pcg_spmv") -> dict:
        n, ms, b = C.c_int64(), C.c_double(), C.c_double()
        self._c(
            self._L.ssim_gb_profile_read(self._h, _lib.PROFILE_KERNELS[kernel], C.byref(n), C.byref(ms), C.byref(b))
        )
        return {"launches": n.value, "total_ms": ms.value, "bytes_per_launch": b.value}
