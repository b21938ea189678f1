"""CPU-only checks of the product library: it loads, exports every symbol of include/ssim_gb.h, builds
the reference's CSR pattern bit-exactly on the host, and the mesh generators match the reference's."""
import ctypes
import os

import numpy as np
import pytest

import ssim_gb300 as g
from ssim_gb300 import _lib, mesh


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    declared = _lib.declared_symbols()
    assert len(declared) >= 50
    for name in declared:
        assert hasattr(L, name), name
    # and nothing is declared that the .so lacks, checked through dlsym directly
    so = ctypes.CDLL(_lib.LIB_PATH)
    for name in declared:
        getattr(so, name)


def test_version_and_defaults():
    L = _lib.lib()
    assert b"sm_103a" in L.ssim_gb_version()
    p = g.default_params()
    assert p.max_newton_iters == 1000  # backward_euler.hpp:21
    assert p.armijo == 0.3  # backward_euler.hpp:22
    assert p.precond == 1 and p.cg_rtol == 1e-8


def test_create_without_gpu_fails_loudly():
    """No CPU fallback: on a machine without a CUDA device creation fails with a CUDA error."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    X, T = mesh.tetra()
    with pytest.raises(_lib.SsimGbError):
        g.TimeStep(X, T, 1e-2)


@pytest.mark.parametrize("shape", [(2, 2, 2), (3, 4, 5), (7, 7, 7)])
def test_unit_box_matches_oracle(oracle, shape):
    X, T = mesh.unit_box(*shape)
    Xo, To = oracle.unit_box(*shape)
    assert np.array_equal(X, Xo) and np.array_equal(T, To)


@pytest.mark.parametrize(
    "make",
    [
        lambda: mesh.unit_box(2, 2, 2),
        lambda: mesh.unit_box(5, 4, 6),
        lambda: mesh.tetra(),
        lambda: mesh.kuhn_box((4, 3, 5)),
        lambda: (mesh.jitter_interior(mesh.kuhn_box((6, 3, 3), (2, 1, 1))[0], 0.02, 9), mesh.kuhn_box((6, 3, 3))[1]),
    ],
)
def test_csr_pattern_bit_exact(oracle, make):
    """row_ptr / col_idx of the Hessian CSR equal the oracle's (COO->CSR of global_composer.hpp:81-92)."""
    X, T = make()
    rp, ci = g.mesh_csr_pattern(T, X.shape[0])
    ts = oracle.OracleTimeStep(X, T, 1e-2, 1e6, 0.3, 1.0)
    rpo, cio = ts.csr_pattern()
    assert rp.dtype == np.int32 and ci.dtype == np.int32
    assert np.array_equal(rp, rpo)
    assert np.array_equal(ci, cio)


def test_benchmark_mesh_sizes():
    """Mesh sizes of the benchmark configs (T, V, nnz)."""
    X, T = mesh.kuhn_box((10, 10, 10))
    assert T.shape[0] == 6000 and X.shape[0] == 1331
    assert g.mesh_csr_pattern(T, X.shape[0])[1].size == 154719
    X, T = mesh.unit_box(11, 11, 11)
    assert T.shape[0] == 5000 and g.mesh_csr_pattern(T, X.shape[0])[1].size == 136719
    X, T = mesh.kuhn_box((32, 32, 32))
    assert T.shape[0] == 196608 and X.shape[0] == 35937
    assert g.mesh_csr_pattern(T, X.shape[0])[1].size == 4619817


def test_kuhn_orientation_and_volume():
    X, T = mesh.kuhn_box((3, 4, 5), (3.0, 2.0, 1.0))
    v = mesh.volumes(X, T)
    assert np.all(v > 0)
    assert abs(v.sum() - 6.0) < 1e-12


def test_bad_cells_rejected():
    X, T = mesh.tetra()
    T = T.copy()
    T[0, 2] = 7
    with pytest.raises(ValueError):
        g.mesh_csr_pattern(T, X.shape[0])


def test_splitmix64_known_values():
    # SplitMix64 seeded with 0: first outputs (reference values of the published generator)
    assert mesh.splitmix64(0, 3).tolist() == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    u = mesh.uniform(5, 10000)
    assert 0 <= u.min() and u.max() < 1 and abs(u.mean() - 0.5) < 0.01


def test_libssim_unit_box_layout():
    from ssim_gb300.libssim import fem

    v, c = fem.unit_box(4, 3, 2)
    assert v.shape == (3, 24) and c.shape == (4, 5 * 3 * 2 * 1)
    assert v.dtype == np.float64 and c.dtype == np.int32


def _header_struct_fields(name):
    """(type, field) pairs of the typedef struct ``name`` in include/ssim_gb.h."""
    import re

    text = open(_lib.HEADER_PATH).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    m = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + ";", text)
    assert m, name
    return re.findall(r"^\s*(int32_t|int64_t|double)\s+(\w+);", m.group(1), flags=re.M)


@pytest.mark.parametrize("cname, pycls, which", [("ssim_gb_params", _lib.Params, 0),
                                                 ("ssim_gb_step_stats", _lib.StepStats, 1),
                                                 ("ssim_gb_tuning", _lib.Tuning, 2)])
def test_ctypes_structs_mirror_header(cname, pycls, which):
    ctype = {"int32_t": ctypes.c_int32, "int64_t": ctypes.c_int64, "double": ctypes.c_double}
    hdr = [(f, ctype[t]) for t, f in _header_struct_fields(cname)]
    assert hdr == list(pycls._fields_)
    # the compiled library's layout (padding included) is the ctypes one
    assert _lib.lib().ssim_gb_struct_size(which) == ctypes.sizeof(pycls)
    assert _lib.lib().ssim_gb_struct_size(7) == 0
    # the library's defaults round-trip through the Python struct
    p = g.default_params()
    assert p.pcg_persistent == 3 and p.pcg_barrier_extra == 0 and p.pcg_spin_limit == 0
    assert p.pcg_pipe_iters == 80 and p.elem32_switch == 10.0 and p.mixed_elem32 == 1
