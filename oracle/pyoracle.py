"""ctypes wrapper of the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker / the timed CPU
baseline.  The product package never imports it.

The oracle restates ssim's FEM time-stepping path in C++ (``oracle.cpp``); see
that file for the reference file:line each function follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

ORC_DEFORMATION, ORC_PREV_DEFORM, ORC_INERTIA_DEFORM, ORC_NEXT_DEFORM = 0, 1, 2, 3
ORC_VELOCITY, ORC_EXT_ACCEL, ORC_FORCES, ORC_DBC_VALUES = 4, 5, 6, 7
ORC_SYSMATRIX, ORC_MASS, ORC_MASS_FILTERED = 0, 1, 2

_BUFFERS = {
    "deformation": ORC_DEFORMATION,
    "prev_deform": ORC_PREV_DEFORM,
    "inertia_deform": ORC_INERTIA_DEFORM,
    "next_deform": ORC_NEXT_DEFORM,
    "velocity": ORC_VELOCITY,
    "ext_accel": ORC_EXT_ACCEL,
    "forces": ORC_FORCES,
    "dbc_values": ORC_DBC_VALUES,
}


class OrcParams(C.Structure):
    _fields_ = [
        ("max_newton_iters", C.c_int),
        ("armijo", C.c_double),
        ("ls_shrink", C.c_double),
        ("max_ls_iters", C.c_int),
        ("cg_max_iters", C.c_int),
        ("cg_rtol", C.c_double),
        ("cg_forcing", C.c_int),
        ("cg_eta_min", C.c_double),
        ("stop_mode", C.c_int),
        ("rel_tol", C.c_double),
        ("precond", C.c_int),
        ("lbfgs_history", C.c_int),
        ("lbfgs_armijo", C.c_double),
        ("max_lbfgs_iters", C.c_int),
        ("ls_energy_slack", C.c_double),
        ("ncg_max_iters", C.c_int),
        ("ncg_step0", C.c_double),
        ("ncg_eta", C.c_double),
        ("ncg_expand", C.c_int),
        ("stop_floor", C.c_double),
    ]


class OrcStats(C.Structure):
    _fields_ = [
        ("converged", C.c_int),
        ("newton_iters", C.c_int),
        ("cg_iters_total", C.c_int),
        ("ls_steps_total", C.c_int),
        ("grad_norm", C.c_double),
        ("grad_norm0", C.c_double),
        ("energy", C.c_double),
        ("last_change", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (g++ -O3 -fopenmp)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
        os.path.join(_HERE, "oracle.cpp")
    ):
        build()
    L = C.CDLL(_LIB_PATH)
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    i8p = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")
    vp = C.c_void_p
    sig = {
        "orc_unit_box_sizes": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "orc_unit_box": (None, [C.c_int, C.c_int, C.c_int, dp, ip]),
        "orc_tetra": (None, [dp, ip]),
        "orc_lame": (None, [C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "orc_snh_energy": (C.c_double, [dp, C.c_double, C.c_double]),
        "orc_snh_stress": (C.c_double, [dp, C.c_double, C.c_double, dp]),
        "orc_snh_hessian": (None, [dp, C.c_double, C.c_double, dp]),
        "orc_sym_eigen": (C.c_int, [C.c_int, dp, dp, dp]),
        "orc_project_spd": (None, [dp, C.c_double, dp]),
        "orc_dminv": (None, [dp, dp, dp, dp, dp, C.POINTER(C.c_double)]),
        "orc_element_stiffness": (None, [dp, dp, C.c_double, C.c_double, C.c_int, dp]),
        "orc_default_params": (None, [C.POINTER(OrcParams)]),
        "orc_create": (vp, [dp, C.c_int, ip, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]),
        "orc_create_2d": (vp, [dp, C.c_int, ip, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]),
        "orc_snh2_energy": (C.c_double, [dp, C.c_double, C.c_double]),
        "orc_snh2_stress": (C.c_double, [dp, C.c_double, C.c_double, dp]),
        "orc_snh2_hessian": (None, [dp, C.c_double, C.c_double, dp]),
        "orc_linear2_stress": (C.c_double, [dp, C.c_double, C.c_double, dp]),
        "orc_linear2_hessian": (None, [C.c_double, C.c_double, dp]),
        "orc_element_stiffness_2d": (None, [dp, dp, C.c_double, C.c_double, C.c_int, C.c_int, dp]),
        "orc_create_springs": (
            vp,
            [dp, C.c_int, ip, C.c_int, C.c_double, C.c_void_p, C.c_double, C.c_double],
        ),
        "orc_destroy": (None, [vp]),
        "orc_num_vertices": (C.c_int, [vp]),
        "orc_num_cells": (C.c_int, [vp]),
        "orc_nnz": (C.c_int, [vp]),
        "orc_threshold_abs": (C.c_double, [vp]),
        "orc_set_time_step": (C.c_int, [vp, C.c_double]),
        "orc_set_youngs": (C.c_int, [vp, C.c_double]),
        "orc_set_poisson": (C.c_int, [vp, C.c_double]),
        "orc_set_density": (C.c_int, [vp, C.c_double]),
        "orc_set_damping": (C.c_int, [vp, C.c_double]),
        "orc_set_threshold": (C.c_int, [vp, C.c_double]),
        "orc_set_material": (None, [vp, vp, vp]),
        "orc_set_dof_type": (None, [vp, i8p]),
        "orc_get_dof_type": (None, [vp, i8p]),
        "orc_add_ext_force_dof": (C.c_int, [vp, C.c_int, C.c_double]),
        "orc_set_pd_diffusivity_mode": (None, [vp, C.c_int]),
        "orc_reset": (None, [vp]),
        "orc_prepare_step": (None, [vp]),
        "orc_update_energy_and_gradients": (C.c_double, [vp, C.c_int]),
        "orc_energy_at": (C.c_double, [vp, dp]),
        "orc_update_hessian": (None, [vp, C.c_int, C.c_int, C.c_int]),
        "orc_compute_step_newton": (C.c_double, [vp, C.POINTER(OrcParams), C.POINTER(OrcStats)]),
        "orc_compute_step_lbfgs": (C.c_double, [vp, C.POINTER(OrcParams), C.POINTER(OrcStats)]),
        "orc_compute_step_pd": (C.c_double, [vp, C.POINTER(OrcParams), C.POINTER(OrcStats)]),
        "orc_compute_step_h0": (C.c_double, [vp, C.POINTER(OrcParams), C.POINTER(OrcStats)]),
        "orc_compute_step_forward_euler": (C.c_double, [vp, C.POINTER(OrcParams), C.POINTER(OrcStats)]),
        "orc_compute_step_ncg": (C.c_double, [vp, C.POINTER(OrcParams), C.POINTER(OrcStats)]),
        "orc_compute_step_ncg_prec": (C.c_double, [vp, C.POINTER(OrcParams), C.POINTER(OrcStats)]),
        "orc_set_ncg_matrix": (None, [vp, C.c_void_p]),
        "orc_set_model": (None, [vp, C.c_int]),
        "orc_linear_stress": (C.c_double, [dp, C.c_double, C.c_double, dp]),
        "orc_linear_hessian": (None, [C.c_double, C.c_double, dp]),
        "orc_element_stiffness_model": (None, [dp, dp, C.c_double, C.c_double, C.c_int, C.c_int, dp]),
        "orc_step_next": (None, [vp]),
        "orc_restore": (None, [vp]),
        "orc_check_convergence": (C.c_int, [vp]),
        "orc_get": (None, [vp, C.c_int, dp]),
        "orc_set": (None, [vp, C.c_int, dp]),
        "orc_get_dminv": (None, [vp, dp]),
        "orc_get_rest_vol": (None, [vp, dp]),
        "orc_get_def_grad": (None, [vp, dp]),
        "orc_get_local_stiffness": (None, [vp, dp]),
        "orc_get_csr": (None, [vp, ip, ip]),
        "orc_get_values": (None, [vp, C.c_int, dp]),
        "orc_spmv": (None, [vp, C.c_int, dp, dp]),
        "orc_pd_matrix_values": (None, [vp, vp]),
        "orc_pcg": (C.c_int, [vp, dp, dp, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_double)]),
        "orc_gather_force": (None, [vp, dp, C.c_double, dp]),
        "orc_gather_hessian": (None, [vp, dp, C.c_double, dp]),
        "orc_num_threads": (C.c_int, []),
        "orc_local_mass": (None, [vp, C.c_double, dp]),
        "orc_local_laplace": (None, [vp, C.c_double, dp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


# ---------------------------------------------------------------- meshes
def unit_box(nx=2, ny=2, nz=2):
    """ssim::mesh::unit_box (vertex counts; 5 tets per cell).  Returns X [V,3], cells [T,4]."""
    L = lib()
    nv, nt = C.c_int(), C.c_int()
    L.orc_unit_box_sizes(nx, ny, nz, C.byref(nv), C.byref(nt))
    X = np.zeros((nv.value, 3))
    cells = np.zeros((nt.value, 4), dtype=np.int32)
    L.orc_unit_box(nx, ny, nz, X, cells)
    return X, cells


def tetra():
    X = np.zeros((4, 3))
    cells = np.zeros((1, 4), dtype=np.int32)
    lib().orc_tetra(X, cells)
    return X, cells


# ---------------------------------------------------------------- element math
def lame(E, nu):
    lam, mu = C.c_double(), C.c_double()
    lib().orc_lame(E, nu, C.byref(lam), C.byref(mu))
    return lam.value, mu.value


def snh_energy(F, lam, mu):
    return lib().orc_snh_energy(_f64(F, (9,)), lam, mu)


def snh_stress(F, lam, mu):
    P = np.zeros(9)
    e = lib().orc_snh_stress(_f64(F, (9,)), lam, mu, P)
    return e, P.reshape(3, 3)


def snh_hessian(F, lam, mu):
    H = np.zeros(81)
    lib().orc_snh_hessian(_f64(F, (9,)), lam, mu, H)
    return H.reshape(9, 9)


def snh2_energy(F, lam, mu):
    return lib().orc_snh2_energy(_f64(F).reshape(-1), lam, mu)


def snh2_stress(F, lam, mu):
    P = np.zeros(4)
    e = lib().orc_snh2_stress(_f64(F).reshape(-1), lam, mu, P)
    return e, P.reshape(2, 2)


def snh2_hessian(F, lam, mu):
    H = np.zeros(16)
    lib().orc_snh2_hessian(_f64(F).reshape(-1), lam, mu, H)
    return H.reshape(4, 4)


def linear2_stress(F, lam, mu):
    P = np.zeros(4)
    e = lib().orc_linear2_stress(_f64(F).reshape(-1), lam, mu, P)
    return e, P.reshape(2, 2)


def linear2_hessian(lam, mu):
    H = np.zeros(16)
    lib().orc_linear2_hessian(lam, mu, H)
    return H.reshape(4, 4)


def element_stiffness_2d(F, Dminv, lam, mu, make_spsd=True, model=0):
    K = np.zeros(81)
    lib().orc_element_stiffness_2d(_f64(F).reshape(-1), _f64(Dminv).reshape(-1), lam, mu, int(make_spsd),
                                   int(model), K)
    return K.reshape(9, 9)


def linear_stress(F, lam, mu):
    P = np.zeros(9)
    e = lib().orc_linear_stress(_f64(F, (9,)), lam, mu, P)
    return e, P.reshape(3, 3)


def linear_hessian(lam, mu):
    H = np.zeros(81)
    lib().orc_linear_hessian(lam, mu, H)
    return H.reshape(9, 9)


def sym_eigen(A):
    A = _f64(A)
    n = A.shape[0]
    w = np.zeros(n)
    V = np.zeros((n, n))
    lib().orc_sym_eigen(n, A.reshape(-1), w, V.reshape(-1))
    return w, V


def project_spd(H, eps=1e-3):
    Hp = np.zeros(81)
    lib().orc_project_spd(_f64(H, (81,)), eps, Hp)
    return Hp.reshape(9, 9)


def dminv(x0, x1, x2, x3):
    D = np.zeros(9)
    v = C.c_double()
    lib().orc_dminv(_f64(x0), _f64(x1), _f64(x2), _f64(x3), D, C.byref(v))
    return D.reshape(3, 3), v.value


def element_stiffness(F, Dminv, lam, mu, make_spsd=True, model=0):
    K = np.zeros(144)
    lib().orc_element_stiffness_model(_f64(F, (9,)), _f64(Dminv, (9,)), lam, mu, int(make_spsd), int(model), K)
    return K.reshape(12, 12)


def default_params(**kw) -> OrcParams:
    p = OrcParams()
    lib().orc_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def num_threads() -> int:
    return lib().orc_num_threads()


# ---------------------------------------------------------------- time step
class OracleTimeStep:
    """basic_time_step restated on the CPU in FP64 (time_step.hpp:168-715)."""

    def __init__(self, X, cells, time_step=1e-3, youngs=1e6, poisson=0.33, density=1e3):
        L = lib()
        self._L = L
        X = _f64(X).reshape(-1, 3)
        cells = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1, 4)
        self.nv, self.nt = X.shape[0], cells.shape[0]
        self.n = 3 * self.nv
        self._h = L.orc_create(X.reshape(-1), self.nv, cells.reshape(-1), self.nt, time_step, youngs, poisson, density)
        self.X, self.cells = X, cells

    @classmethod
    def tri2d(cls, X2, tris, time_step=1e-3, youngs=1e6, poisson=0.33, density=1e3):
        """2D triangles in the plane (basic_time_step with PhysicalDim 2, TopologyDim 3): X2 [V, 2],
        tris [T, 3]; state vectors are [V, 3] with z identically zero."""
        L = lib()
        self = cls.__new__(cls)
        self._L = L
        X2 = _f64(X2).reshape(-1, 2)
        T = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
        self.nv, self.nt = X2.shape[0], T.shape[0]
        self.n = 3 * self.nv
        self._h = L.orc_create_2d(X2.reshape(-1), self.nv, T.reshape(-1), self.nt, time_step, youngs, poisson,
                                  density)
        self.X = np.concatenate([X2, np.zeros((self.nv, 1))], axis=1)
        self.cells = T
        return self

    @classmethod
    def springs(cls, X, springs, stiffness, vertex_mass=None, mass=None, time_step=1e-2):
        """A mass-spring system (no reference counterpart): rest lengths from X, lumped vertex masses
        (vertex_mass[nv], or `mass` each), energy 1/2|x - x~|_M^2 + dt^2 sum k/2 (|x_i - x_j| - L)^2."""
        L = lib()
        self = cls.__new__(cls)
        self._L = L
        X = _f64(X).reshape(-1, 3)
        sp = np.ascontiguousarray(springs, dtype=np.int32).reshape(-1, 2)
        self.nv, self.nt = X.shape[0], sp.shape[0]
        self.n = 3 * self.nv
        vm = None if vertex_mass is None else _f64(vertex_mass).reshape(-1)
        if vm is not None and vm.size != self.nv:
            raise ValueError("vertex_mass must have one entry per vertex")
        m = float(mass) if mass is not None else 0.0
        self._vm = vm
        self._h = L.orc_create_springs(
            X.reshape(-1), self.nv, sp.reshape(-1), self.nt, float(stiffness),
            None if vm is None else vm.ctypes.data, m, float(time_step),
        )
        self.X, self.cells = X, sp
        return self

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.orc_destroy(h)
            self._h = None

    # setters
    def _chk(self, rc, what):
        if rc != 0:
            raise ValueError(what)
        return self

    def set_time_step(self, v):
        return self._chk(self._L.orc_set_time_step(self._h, v), "Time step must be positive.")

    def set_youngs(self, v):
        return self._chk(self._L.orc_set_youngs(self._h, v), "Young's modulus must be positive.")

    def set_poisson(self, v):
        return self._chk(self._L.orc_set_poisson(self._h, v), "Poisson's ratio must be in (0, 0.5).")

    def set_density(self, v):
        return self._chk(self._L.orc_set_density(self._h, v), "Density must be positive.")

    def set_damping(self, v):
        return self._chk(self._L.orc_set_damping(self._h, v), "Damping must be in [0, 1).")

    def set_threshold(self, v):
        return self._chk(self._L.orc_set_threshold(self._h, v), "Threshold must be positive.")

    def set_material(self, E_elem=None, nu_elem=None):
        self._Ee = None if E_elem is None else _f64(E_elem).reshape(-1)
        self._ne = None if nu_elem is None else _f64(nu_elem).reshape(-1)
        pe = None if self._Ee is None else self._Ee.ctypes.data
        pn = None if self._ne is None else self._ne.ctypes.data
        self._L.orc_set_material(self._h, pe, pn)

    def set_pd_diffusivity_mode(self, mode):
        self._L.orc_set_pd_diffusivity_mode(self._h, int(mode))

    def set_dof_type(self, types):
        self._L.orc_set_dof_type(self._h, np.ascontiguousarray(types, dtype=np.int8).reshape(-1))

    def dof_type(self):
        t = np.zeros(self.n, dtype=np.int8)
        self._L.orc_get_dof_type(self._h, t)
        return t.reshape(-1, 3)

    def mark_dirichlet(self, verts, values=None):
        t = self.dof_type().reshape(-1, 3).copy()
        t[np.asarray(verts)] = 1
        self.set_dof_type(t)
        dv = self.get("dbc_values")
        if values is not None:
            dv[np.asarray(verts)] = np.asarray(values, dtype=np.float64).reshape(-1, 3)
        self.set("dbc_values", dv)

    def add_ext_force_dof(self, dof, a):
        return self._chk(self._L.orc_add_ext_force_dof(self._h, dof, a), "|dof_idx| must be less than PhysicalDim.")

    def add_gravity(self, g):
        for d in range(3):
            self.add_ext_force_dof(d, float(g[d]))

    # loop
    def reset(self):
        self._L.orc_reset(self._h)

    def prepare_step(self):
        self._L.orc_prepare_step(self._h)

    def update_energy_and_gradients(self, F_updated=False):
        return self._L.orc_update_energy_and_gradients(self._h, int(F_updated))

    def energy_at(self, u):
        return self._L.orc_energy_at(self._h, _f64(u).reshape(-1))

    def update_hessian(self, F_updated=False, make_spsd=False, filter_dbc=True):
        self._L.orc_update_hessian(self._h, int(F_updated), int(make_spsd), int(filter_dbc))

    def compute_step(self, method="newton", params: OrcParams | None = None):
        p = params if params is not None else default_params()
        st = OrcStats()
        fn = {
            "newton": self._L.orc_compute_step_newton,
            "lbfgs": self._L.orc_compute_step_lbfgs,
            "pd": self._L.orc_compute_step_pd,
            "h0": self._L.orc_compute_step_h0,
            "forward_euler": self._L.orc_compute_step_forward_euler,
            "ncg": self._L.orc_compute_step_ncg,
            "ncg_ext": self._L.orc_compute_step_ncg_prec,
        }[method]
        r = fn(self._h, C.byref(p), C.byref(st))
        return r, st.as_dict()

    def set_model(self, model):
        """Elastic model: "stable_neohookean" (0) or "linear" (1)."""
        self._L.orc_set_model(self._h, {"stable_neohookean": 0, "linear": 1}.get(model, model))

    def set_ncg_matrix(self, values=None):
        """Values of the NCG preconditioner factor L in the system matrix's CSR order (None: identity)."""
        if values is None:
            self._L.orc_set_ncg_matrix(self._h, None)
            return
        self._ncg_vals = _f64(values).reshape(-1)
        assert self._ncg_vals.size == self.nnz
        self._L.orc_set_ncg_matrix(self._h, self._ncg_vals.ctypes.data)

    def step_next(self):
        self._L.orc_step_next(self._h)

    def restore(self):
        self._L.orc_restore(self._h)

    def check_convergence(self):
        return bool(self._L.orc_check_convergence(self._h))

    # accessors
    @property
    def threshold_abs(self):
        return self._L.orc_threshold_abs(self._h)

    @property
    def nnz(self):
        return self._L.orc_nnz(self._h)

    def get(self, name):
        out = np.zeros(self.n)
        self._L.orc_get(self._h, _BUFFERS[name], out)
        return out.reshape(-1, 3)

    def set(self, name, value):
        self._L.orc_set(self._h, _BUFFERS[name], _f64(value).reshape(-1))

    def dminv(self):
        out = np.zeros(self.nt * 9)
        self._L.orc_get_dminv(self._h, out)
        return out.reshape(-1, 3, 3)

    def rest_vol(self):
        out = np.zeros(self.nt)
        self._L.orc_get_rest_vol(self._h, out)
        return out

    def def_grad(self):
        out = np.zeros(self.nt * 9)
        self._L.orc_get_def_grad(self._h, out)
        return out.reshape(-1, 3, 3)

    def local_stiffness(self):
        L = 3 * self.cells.shape[1]
        out = np.zeros(self.nt * L * L)
        self._L.orc_get_local_stiffness(self._h, out)
        return out.reshape(-1, L, L)

    def csr_pattern(self):
        rp = np.zeros(self.n + 1, dtype=np.int32)
        ci = np.zeros(self.nnz, dtype=np.int32)
        self._L.orc_get_csr(self._h, rp, ci)
        return rp, ci

    def values(self, which="sysmatrix"):
        w = {"sysmatrix": ORC_SYSMATRIX, "mass": ORC_MASS, "mass_filtered": ORC_MASS_FILTERED}[which]
        out = np.zeros(self.nnz)
        self._L.orc_get_values(self._h, w, out)
        return out

    def matrix(self, which="sysmatrix"):
        import scipy.sparse as sp

        rp, ci = self.csr_pattern()
        return sp.csr_matrix((self.values(which), ci, rp), shape=(self.n, self.n))

    def spmv(self, x, which="sysmatrix"):
        w = {"sysmatrix": ORC_SYSMATRIX, "mass": ORC_MASS, "mass_filtered": ORC_MASS_FILTERED}[which]
        y = np.zeros(self.n)
        self._L.orc_spmv(self._h, w, _f64(x).reshape(-1), y)
        return y

    def local_mass(self, alpha=1.0):
        out = np.zeros(self.nt * 16)
        self._L.orc_local_mass(self._h, alpha, out)
        return out.reshape(-1, 4, 4)

    def local_laplace(self, alpha=1.0):
        out = np.zeros(self.nt * 16)
        self._L.orc_local_laplace(self._h, alpha, out)
        return out.reshape(-1, 4, 4)

    def pd_matrix_values(self):
        out = np.zeros(self.nnz)
        self._L.orc_pd_matrix_values(self._h, out.ctypes.data)
        return out

    def pcg(self, b, rtol=1e-8, max_iters=10000, precond=1, x0=None):
        x = np.zeros(self.n) if x0 is None else _f64(x0).reshape(-1).copy()
        rr = C.c_double()
        it = self._L.orc_pcg(self._h, _f64(b).reshape(-1), x, rtol, max_iters, precond, C.byref(rr))
        return x, it, rr.value

    def gather_force(self, local_force, alpha=1.0):
        f = np.zeros(self.n)
        self._L.orc_gather_force(self._h, _f64(local_force).reshape(-1), alpha, f)
        return f.reshape(-1, 3)

    def gather_hessian(self, local_K, alpha=1.0, base=None):
        v = np.zeros(self.nnz) if base is None else _f64(base).copy()
        self._L.orc_gather_hessian(self._h, _f64(local_K).reshape(-1), alpha, v)
        return v
