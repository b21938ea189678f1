"""The allocation-free energy entry point (ssim_gb_energy_noalloc).

It serves callers that cannot call cudaMalloc -- code whose device memory is all owned by another
allocator (a framework's caching allocator, a fixed budget taken at start-up) or a loop that must not pay an
allocation's latency or risk its failure.  It keeps the scratch of its reduction in a fixed array inside the
library, so the caller passes only inputs and the output.  This test calls it through the C ABI twice in a
row per mesh and checks each result against the existing entry point ssim_gb_energy_at on the same state
and against the FP64 oracle's energy, within the FP64 tolerance of the other parity tests.  The meshes span
the fixed scratch: one block (fewer than 128 cells), a few dozen blocks, and the 1.02M-tet beam (7,969 of
the at most 8,192 blocks).  It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10


def _mesh(name):
    from ssim_gb300 import mesh

    if name == "one_block":
        X, T = mesh.kuhn_box((3, 2, 2), (0.3, 0.2, 0.2))  # 72 tets
    elif name == "small":
        X, T = mesh.kuhn_box((12, 8, 6), (1.2, 0.8, 0.6))  # 3,456 tets
    else:
        X, T = mesh.kuhn_box((100, 50, 34), (2.0, 1.0, 0.68))  # 1,020,000 tets
    return mesh.jitter_interior(X, 0.002, 41), T


@pytest.mark.parametrize("name", ["one_block", "small", "beam1m"])
def test_energy_noalloc_matches_energy_at_and_oracle(name):
    import torch

    import ssim_gb300 as g
    from oracle import pyoracle
    from ssim_gb300 import _lib, mesh

    X, T = _mesh(name)
    nt = T.shape[0]
    E_cells = 10.0 ** mesh.uniform(42, nt, 4.0, 6.0)
    nu, rho, dt = 0.45, 1000.0, 1e-2
    ts = g.TimeStep(X, T, dt, 1e5, nu, rho)
    ts.set_material(E_cells, None)
    ts.reset("none")
    u = mesh.uniform(43, X.size, -0.003, 0.003).reshape(X.shape)
    xt = mesh.uniform(44, X.size, -0.003, 0.003).reshape(X.shape)
    ts.set("inertia_deform", xt)
    e_lib = ts.energy_at(u)
    ot = pyoracle.OracleTimeStep(X, T, dt, 1e5, nu, rho)
    ot.set_material(E_cells, None)
    ot.reset()
    ot.set("inertia_deform", xt)
    e_orc = ot.energy_at(u)

    dev = torch.device("cuda:0")
    f64 = dict(dtype=torch.float64, device=dev)
    dX = torch.tensor(X, **f64)
    du = torch.tensor(u, **f64)
    dxt = torch.tensor(xt, **f64)
    dcells = torch.tensor(T, dtype=torch.int32, device=dev)
    ddm = torch.tensor(ts.dminv(), **f64)
    dvol = torch.tensor(ts.rest_volume(), **f64)
    mu = E_cells / (2 * (1 + nu))
    lam = E_cells * nu / ((1 + nu) * (1 - 2 * nu))
    dlam = torch.tensor(lam, **f64)
    dmu = torch.tensor(mu, **f64)
    out = torch.zeros(1, **f64)
    stream = torch.cuda.current_stream().cuda_stream
    L = _lib.lib()

    def call(n=nt):
        return L.ssim_gb_energy_noalloc(
            dX.data_ptr(), du.data_ptr(), dxt.data_ptr(), dcells.data_ptr(), ddm.data_ptr(), dvol.data_ptr(),
            dlam.data_ptr(), dmu.data_ptr(), n, dt, rho, C.c_void_p(stream), out.data_ptr(),
        )

    for _ in range(2):  # the second call reuses the scratch the first one left behind
        out.zero_()
        assert call() == _lib.OK
        torch.cuda.synchronize()
        e = out.item()
        assert abs(e - e_lib) <= FP64_RTOL * abs(e_lib), (e, e_lib)
        assert abs(e - e_orc) <= FP64_RTOL * abs(e_orc), (e, e_orc)

    # beyond the fixed scratch's size: rejected with a clear error, nothing launched
    too_many = (1 << 20) + 1
    assert call(too_many) == _lib.ERR_INVALID_ARGUMENT
    assert b"num_cells" in L.ssim_gb_last_error(None)
