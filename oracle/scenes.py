"""The benchmark scenes on the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

A scene is the dict made by ``ssim_gb300.scenes`` (mesh, material, Dirichlet set, gravity, initial
state).  These helpers set the same scene up on the oracle; only ``tests/``, ``__graft_entry__.smoke()``
and the CPU leg of ``bench.py`` call them, as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import numpy as np

from . import pyoracle


def build_oracle(scene, rtol=None):
    """The same scene as ``ssim_gb300.scenes.build_timestep`` on the FP64 oracle."""
    if scene.get("springs"):
        ts = pyoracle.OracleTimeStep.springs(scene["X"], scene["cells"], scene["k"],
                                             vertex_mass=scene["vertex_mass"], time_step=scene["dt"])
    elif scene.get("tri2d"):
        ts = pyoracle.OracleTimeStep.tri2d(scene["X2"], scene["cells"], scene["dt"], scene["E"], scene["nu"],
                                           scene["rho"])
    else:
        ts = pyoracle.OracleTimeStep(scene["X"], scene["cells"], scene["dt"], scene["E"], scene["nu"],
                                     scene["rho"])
    if scene.get("E_cells") is not None:
        ts.set_material(scene["E_cells"], scene.get("nu_cells"))
    if len(scene["fixed"]):
        ts.mark_dirichlet(scene["fixed"])
    if any(scene["gravity"]):
        ts.add_gravity(scene["gravity"])
    if rtol is not None:
        ts.set_threshold(rtol)
    ts.reset()
    if scene.get("u0") is not None:
        ts.set("deformation", scene["u0"])
        ts.set("prev_deform", scene["u0"])
    if scene.get("velocity") is not None:
        ts.set("velocity", scene["velocity"])
    return ts


def batch_instance(batch, i):
    """Instance i of a batch made by ``ssim_gb300.scenes.batch_cubes`` as a scene dict of its own (its
    vertices, cells renumbered from 0, material, bottom face, initial velocity)."""
    a, b = int(batch["vertex_offsets"][i]), int(batch["vertex_offsets"][i + 1])
    X = batch["X"][a:b]
    cells = batch["cells"]
    sel = (cells[:, 0] >= a) & (cells[:, 0] < b)
    return dict(name=f"{batch['name']}_instance{i}", X=X, cells=(cells[sel] - a).astype(np.int32),
                dt=batch["dt"], E=float(batch["E_inst"][i]), nu=float(batch["nu_inst"][i]), rho=batch["rho"],
                fixed=np.where(X[:, 2] == 0.0)[0], gravity=batch["gravity"], u0=None, E_cells=None,
                velocity=batch["velocity"][a:b], k=int(batch["k"][i]))


def batch_instance_oracle(batch, i):
    """Instance i of the batch on the FP64 oracle, with the instance's own uniform material."""
    return build_oracle(batch_instance(batch, i))
