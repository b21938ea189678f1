"""ctypes binding of libssim_gb300.so (the C ABI declared in include/ssim_gb.h).

The library is built in-tree (``ssim_gb300/build.py``); importing this module
never falls back to anything else: if the shared object is missing the import
of the binding raises, and every compute entry point fails with a CUDA error
when no GPU is present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libssim_gb300.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "ssim_gb.h")

(OK, ERR_INVALID_ARGUMENT, ERR_NOT_CONVERGED, ERR_CUDA, ERR_NUMERICAL, ERR_STATE, ERR_OUT_OF_MEMORY,
 ERR_DEVICE_TIMEOUT) = range(8)
FP64, MIXED = 0, 1
MODELS = {"stable_neohookean": 0, "linear": 1}
STEPPER_NEWTON, STEPPER_LBFGS, STEPPER_PD, STEPPER_NONE = 0, 1, 2, 3
STEPPER_FORWARD_EULER, STEPPER_H0, STEPPER_NCG, STEPPER_NCG_EXT = 4, 5, 6, 7
FIELDS = {
    "deformation": 0,
    "prev_deform": 1,
    "inertia_deform": 2,
    "next_deform": 3,
    "velocity": 4,
    "ext_accel": 5,
    "forces": 6,
    "dbc_values": 7,
}
MATRICES = {"sysmatrix": 0, "mass": 1, "mass_filtered": 2, "sysmatrix_half": 3}
PROFILE_KERNELS = {"pcg_spmv": 0, "elem_hessian": 1, "assemble": 2, "elem_grad": 3, "pcg_update": 4, "pcg_iteration": 5}


class Params(C.Structure):
    _fields_ = [
        ("max_newton_iters", C.c_int32),
        ("armijo", C.c_double),
        ("ls_shrink", C.c_double),
        ("max_ls_iters", C.c_int32),
        ("cg_max_iters", C.c_int32),
        ("cg_rtol", C.c_double),
        ("cg_forcing", C.c_int32),
        ("cg_eta_min", C.c_double),
        ("stop_mode", C.c_int32),
        ("rel_tol", C.c_double),
        ("precond", C.c_int32),
        ("lbfgs_history", C.c_int32),
        ("lbfgs_armijo", C.c_double),
        ("max_lbfgs_iters", C.c_int32),
        ("cg_check_every", C.c_int32),
        ("ls_energy_slack", C.c_double),
        ("pd_kappa_mode", C.c_int32),
        ("pcg_persistent", C.c_int32),
        ("pcg_spin_limit", C.c_int64),
        ("pcg_barrier_extra", C.c_int32),
        ("pcg_max_blocks", C.c_int32),
        ("ncg_max_iters", C.c_int32),
        ("ncg_step0", C.c_double),
        ("ncg_eta", C.c_double),
        ("ncg_expand", C.c_int32),
        ("stop_floor", C.c_double),
        ("mixed_elem32", C.c_int32),
        ("ls_energy_slack32", C.c_double),
        ("elem32_switch", C.c_double),
        ("pcg_pipe_iters", C.c_int32),
        ("fused_assembly", C.c_int32),
        ("mixed_delta", C.c_int32),
        ("pcg_half_matrix", C.c_int32),
        ("half_matrix_min_rtol", C.c_double),
        ("half_hessian_blocks", C.c_int32),
        ("half_check_slack", C.c_double),
        ("speculative_hessian", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StepStats(C.Structure):
    _fields_ = [
        ("converged", C.c_int32),
        ("newton_iters", C.c_int32),
        ("cg_iters_total", C.c_int32),
        ("ls_steps_total", C.c_int32),
        ("grad_norm", C.c_double),
        ("grad_norm0", C.c_double),
        ("energy", C.c_double),
        ("last_change", C.c_double),
        ("elapsed_ms", C.c_double),
        ("half_solves", C.c_int32),
        ("half_check", C.c_double),
        ("spec_hits", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [
        ("elem_block", C.c_int32),
        ("hessian_block", C.c_int32),
        ("assembly_block", C.c_int32),
        ("gather_block", C.c_int32),
        ("pcg_persistent", C.c_int32),
        ("pcg_max_blocks", C.c_int32),
        ("fused_assembly", C.c_int32),
        ("from_cache", C.c_int32),
        ("elem_us", C.c_double),
        ("hessian_us", C.c_double),
        ("pcg_solve_ms", C.c_double),
        ("pcg_iterations", C.c_int32),
        ("candidates", C.c_int32),
        ("pcg_half_matrix", C.c_int32),
        ("elem_regcap", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SsimGbError(RuntimeError):
    """A CUDA, state or out-of-memory failure reported by the library."""


class NumericalError(ArithmeticError):
    """Non-finite energy / gradient / residual reported by the library."""


class DeviceTimeout(SsimGbError):
    """A bounded wait inside a kernel (a grid barrier) gave up; the CUDA context is still usable."""


_lib = None

_H = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_SIGS = {
    "ssim_gb_version": (C.c_char_p, []),
    "ssim_gb_launch_count": (C.c_uint64, []),
    "ssim_gb_struct_size": (C.c_size_t, [C.c_int32]),
    "ssim_gb_default_params": (None, [C.POINTER(Params)]),
    "ssim_gb_last_error": (C.c_char_p, [_H]),
    "ssim_gb_mesh_csr_nnz": (C.c_int, [_I, C.c_int32, C.c_int32, C.POINTER(C.c_int64)]),
    "ssim_gb_mesh_csr_pattern": (C.c_int, [_I, C.c_int32, C.c_int32, _I, _I]),
    "ssim_gb_create": (
        C.c_int,
        [_D, C.c_int32, _I, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double, C.POINTER(_H)],
    ),
    "ssim_gb_create_2d": (
        C.c_int,
        [_D, C.c_int32, _I, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double, C.POINTER(_H)],
    ),
    "ssim_gb_get_dim": (C.c_int, [_H, C.POINTER(C.c_int32)]),
    "ssim_gb_get_csr_2d": (C.c_int, [_H, C.c_int32, _I, _I, _D]),
    "ssim_gb_create_springs": (
        C.c_int,
        [_D, C.c_int32, _I, C.c_int32, C.c_double, _D, C.c_double, C.c_double, C.POINTER(_H)],
    ),
    "ssim_gb_destroy": (C.c_int, [_H]),
    "ssim_gb_sizes": (C.c_int, [_H, _I, _I, _I, C.POINTER(C.c_int64)]),
    "ssim_gb_set_stream": (C.c_int, [_H, C.c_void_p]),
    "ssim_gb_set_time_step": (C.c_int, [_H, C.c_double]),
    "ssim_gb_set_youngs": (C.c_int, [_H, C.c_double]),
    "ssim_gb_set_poisson": (C.c_int, [_H, C.c_double]),
    "ssim_gb_set_density": (C.c_int, [_H, C.c_double]),
    "ssim_gb_set_damping": (C.c_int, [_H, C.c_double]),
    "ssim_gb_set_threshold": (C.c_int, [_H, C.c_double]),
    "ssim_gb_set_precision": (C.c_int, [_H, C.c_int32]),
    "ssim_gb_set_params": (C.c_int, [_H, C.POINTER(Params)]),
    "ssim_gb_get_params": (C.c_int, [_H, C.POINTER(Params)]),
    "ssim_gb_set_material": (C.c_int, [_H, _D, _D]),
    "ssim_gb_mark_dirichlet_batched": (C.c_int, [_H, _I, C.c_int32, _D]),
    "ssim_gb_mark_general_batched": (C.c_int, [_H, _I, C.c_int32]),
    "ssim_gb_set_dof_type": (C.c_int, [_H, C.POINTER(C.c_int8)]),
    "ssim_gb_get_dof_type": (C.c_int, [_H, C.POINTER(C.c_int8)]),
    "ssim_gb_add_ext_force_dof": (C.c_int, [_H, C.c_int32, C.c_double]),
    "ssim_gb_add_gravity": (C.c_int, [_H, _D]),
    "ssim_gb_reset": (C.c_int, [_H, C.c_int32]),
    "ssim_gb_prepare_step": (C.c_int, [_H]),
    "ssim_gb_compute_step": (C.c_int, [_H, _D]),
    "ssim_gb_step_next": (C.c_int, [_H]),
    "ssim_gb_step": (C.c_int, [_H, _D]),
    "ssim_gb_restore": (C.c_int, [_H]),
    "ssim_gb_get_step_stats": (C.c_int, [_H, C.POINTER(StepStats)]),
    "ssim_gb_get_solve_log": (C.c_int, [_H, _I, C.c_int32, _I]),
    "ssim_gb_set_ncg_matrix": (C.c_int, [_H, _D]),
    "ssim_gb_set_elastic_model": (C.c_int, [_H, C.c_int32]),
    "ssim_gb_check_convergence": (C.c_int, [_H, _I]),
    "ssim_gb_threshold_abs": (C.c_int, [_H, _D]),
    "ssim_gb_update_energy_and_gradients": (C.c_int, [_H, C.c_int32, _D]),
    "ssim_gb_update_hessian": (C.c_int, [_H, C.c_int32, C.c_int32, C.c_int32]),
    "ssim_gb_energy_at": (C.c_int, [_H, _D, _D]),
    "ssim_gb_get_field": (C.c_int, [_H, C.c_int32, _D]),
    "ssim_gb_set_field": (C.c_int, [_H, C.c_int32, _D]),
    "ssim_gb_field_device_ptr": (C.c_int, [_H, C.c_int32, C.POINTER(C.c_void_p)]),
    "ssim_gb_get_csr_pattern": (C.c_int, [_H, _I, _I]),
    "ssim_gb_get_matrix_values": (C.c_int, [_H, C.c_int32, _D]),
    "ssim_gb_get_rest_volume": (C.c_int, [_H, _D]),
    "ssim_gb_get_dminv": (C.c_int, [_H, _D]),
    "ssim_gb_spmv": (C.c_int, [_H, C.c_int32, _D, _D]),
    "ssim_gb_pcg": (C.c_int, [_H, _D, _D, C.c_double, C.c_int32, _I, _D]),
    "ssim_gb_energy_noalloc": (
        C.c_int,
        [C.c_void_p] * 8 + [C.c_int32, C.c_double, C.c_double, C.c_void_p, C.c_void_p],
    ),
    "ssim_gb_set_instances": (C.c_int, [_H, _I, C.c_int32]),
    "ssim_gb_get_instance_residuals": (C.c_int, [_H, _D, _D]),
    "ssim_gb_adjoint_step": (C.c_int, [_H, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int32, _I, _I]),
    "ssim_gb_get_field_device": (C.c_int, [_H, C.c_int32, C.c_void_p]),
    "ssim_gb_set_field_device": (C.c_int, [_H, C.c_int32, C.c_void_p]),
    "ssim_gb_autotune": (C.c_int, [_H, C.POINTER(Tuning)]),
    "ssim_gb_set_tuning": (C.c_int, [_H, C.POINTER(Tuning)]),
    "ssim_gb_profile_enable": (C.c_int, [_H, C.c_int32]),
    "ssim_gb_profile_read": (C.c_int, [_H, C.c_int32, C.POINTER(C.c_int64), _D, _D]),
    "ssim_gb_synchronize": (C.c_int, [_H]),
}


def lib():
    """Load libssim_gb300.so (fails loudly if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python ssim_gb300/build.py)"
        )
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def declared_symbols() -> list[str]:
    """Every function declared in include/ssim_gb.h."""
    import re

    text = open(HEADER_PATH).read()
    return sorted(set(re.findall(r"^SSIM_GB_API [^(]*?\b(ssim_gb_\w+)\(", text, flags=re.M)))


def check(status: int, handle=None):
    if status == OK:
        return
    L = lib()
    msg = L.ssim_gb_last_error(handle)
    msg = msg.decode() if msg else ""
    if status == ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    if status == ERR_NUMERICAL:
        raise NumericalError(msg)
    if status == ERR_OUT_OF_MEMORY:
        raise MemoryError(msg)
    if status == ERR_DEVICE_TIMEOUT:
        raise DeviceTimeout(msg)
    raise SsimGbError(f"status {status}: {msg}")


def default_params(**kw) -> Params:
    p = Params()
    lib().ssim_gb_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(f"unknown solver parameter {k!r}")
        setattr(p, k, v)
    return p


def launch_count() -> int:
    return int(lib().ssim_gb_launch_count())


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_I)


def mesh_csr_pattern(cells: np.ndarray, num_vertices: int):
    """The Hessian CSR pattern of a tet mesh (global_composer.hpp:68-100), computed on the host."""
    cells = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1, 4)
    L = lib()
    nnz = C.c_int64()
    check(L.ssim_gb_mesh_csr_nnz(iptr(cells), cells.shape[0], num_vertices, C.byref(nnz)))
    rp = np.zeros(3 * num_vertices + 1, dtype=np.int32)
    ci = np.zeros(nnz.value, dtype=np.int32)
    check(L.ssim_gb_mesh_csr_pattern(iptr(cells), cells.shape[0], num_vertices, iptr(rp), iptr(ci)))
    return rp, ci
