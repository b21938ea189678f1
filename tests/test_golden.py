"""The committed oracle fixtures (tests/golden/oracle_small.npz, made by tests/golden/make_golden.py):
the oracle must keep reproducing them (CPU), and the CUDA path must match them (GPU)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

GOLD = os.path.join(HERE, "golden", "oracle_small.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_oracle_reproduces_golden(gold):
    d = make_golden.generate()
    assert np.array_equal(d["row_ptr"], gold["row_ptr"]) and np.array_equal(d["col_idx"], gold["col_idx"])
    assert abs(d["energy"] - gold["energy"]) <= 1e-12 * abs(gold["energy"])
    for k in ("forces", "h_spsd", "h_raw", "mass"):
        assert rel(d[k], gold[k]) <= 1e-12, k
    assert rel(d["traj"], gold["traj"]) <= 1e-10


@pytest.mark.gpu
def test_gpu_matches_golden(gold):
    import ssim_gb300 as g

    s = make_golden.SETTINGS
    ts = g.TimeStep(gold["X"], gold["cells"], s["dt"], s["E"], s["nu"], s["rho"])
    ts.mark_dirichlet_batched(gold["fixed"], np.zeros((gold["fixed"].size, 3)))
    ts.add_gravity(s["gravity"])
    ts.reset("none")
    rp, ci = ts.csr_pattern()
    assert np.array_equal(rp, gold["row_ptr"]) and np.array_equal(ci, gold["col_idx"])
    ts.prepare_step()
    ts.set("inertia_deform", gold["xt"])
    ts.set("next_deform", gold["u"])
    e = ts.update_energy_and_gradients()
    assert abs(e - gold["energy"]) <= 1e-10 * abs(gold["energy"])
    assert rel(ts.get("forces"), gold["forces"]) <= 1e-10
    ts.update_hessian(False, True, True)
    assert rel(ts.values("sysmatrix"), gold["h_spsd"]) <= 1e-10
    ts.update_hessian(False, False, False)
    assert rel(ts.values("sysmatrix"), gold["h_raw"]) <= 1e-10
    assert rel(ts.values("mass"), gold["mass"]) <= 1e-15
    ts2 = g.TimeStep(gold["X"], gold["cells"], s["dt"], s["E"], s["nu"], s["rho"])
    ts2.mark_dirichlet_batched(gold["fixed"], np.zeros((gold["fixed"].size, 3)))
    ts2.add_gravity(s["gravity"])
    ts2.set_params(g.default_params(**make_golden.NEWTON))
    ts2.reset("newton")
    for k in range(3):
        ts2.step()
        assert rel(ts2.get("deformation"), gold["traj"][k]) <= 1e-10, k
