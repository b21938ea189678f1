"""Benchmark: backward-Euler Newton steps/s of stable Neo-Hookean tets on one GB300.

Workload (default ``beam1m``): the 1,020,000-tet beam (100x50x34 hex x 6 tets, h = 0.02), per-cell E
log-uniform in [1e4, 1e6] (SplitMix64 seed 3), nu = 0.45, rho = 1000, left face fixed, gravity, dt =
1e-2.  One step = prepare_step + Newton solve to |g| <= 1e-6 |g_0| + step_next.  ``value`` is the
mixed-precision GPU path (FP32 Hessian / assembly / PCG, FP64 energy, gradient, state, reductions);
the plain FP64 GPU path is timed in the same run on the same steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Under torchrun every rank runs an independent replica (the path does not shard); rank 0 prints one
JSON line with the whole-job value.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Newton steps/s @1M tets: mixed vs FP64 plain at 1e-6 residual; adjoint ms/step"


# Solver settings shared by the mixed and FP64 GPU arms and by the CPU arm (the oracle).  The inexact-Newton
# forcing eta = min(0.1, max(0.05, |g|/|g0|)): on the 1.02M-tet beam a floor of 0.05 took 55.3 steps/s
# against 46.1 for 0.01 with 169 against 165 Newton iterations over 20 steps.
SOLVER = dict(stop_mode=1, rel_tol=1e-6, cg_forcing=1, cg_rtol=1e-1, cg_eta_min=5e-2, cg_max_iters=5000,
              max_newton_iters=100, precond=2, max_lbfgs_iters=20000)
GPU_ONLY = dict(cg_check_every=16)  # how often the two-launch PCG reads its stop test (no effect on iterates)


def newton_params(g):
    """SOLVER as the GPU library's parameter block."""
    return g.default_params(**SOLVER, **GPU_ONLY)


def oracle_params():
    """SOLVER as the oracle's parameter block (no call into the GPU library)."""
    from oracle import pyoracle

    return pyoracle.default_params(**SOLVER)


SOLVER_TEXT = {
    "newton": "Newton, stop |g| <= 1e-6 |g0|, block-Jacobi PCG with forcing eta = min(1e-1, max(5e-2, |g|/|g0|)), "
              "backtracking Armijo 0.3",
}


def make_scene(name):
    from ssim_gb300 import scenes

    if name == "beam1m":
        return scenes.beam()
    if name == "beam_small":
        return scenes.beam(40, 20, 14, h=0.05)
    if name == "cube10":
        return scenes.cube10()
    if name == "refbox":
        return scenes.reference_box()
    if name == "bar":
        return scenes.bar()
    if name == "batch":
        return scenes.batch_cubes()
    if name == "cloth512":
        return scenes.cloth()
    if name == "sheet2d":
        return scenes.sheet2d(1001, 501)
    if name == "cloth_small":
        return scenes.cloth(128)
    raise SystemExit(f"unknown workload {name}")


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def ncu_traffic(workload, kernel):
    """DRAM bytes per launch (per iteration for the persistent PCG) of ``kernel`` from the committed ncu
    summary of this workload, if any."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("dram_bytes_per_launch:") or line.strip().startswith("dram_bytes_per_iteration:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi sampled every 100 ms while the timed region runs."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device_index=0):
        self.proc = None
        self.dev = device_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
        except FileNotFoundError:
            self.proc = None
        time.sleep(1.0)  # let nvidia-smi start sampling before the timed region
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


class _HandleFacade:
    """The calls the e2e loop makes, on a TimeStep handle (for the systems and steppers the libssim facade
    does not cover)."""

    def __init__(self, ts):
        self.step_ = ts

    def mark_dirichlet_batched(self, verts, targets):
        self.step_.mark_dirichlet_batched(verts, np.ascontiguousarray(np.asarray(targets).T))

    def step(self):
        self.step_.step()

    def deformation(self):
        return self.step_.get("deformation")


def run_gpu_arm(args, scene):
    import torch

    import ssim_gb300 as g
    from ssim_gb300 import scenes

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    params = newton_params(g)
    params.pd_kappa_mode = args.pd_kappa
    params.pcg_persistent = args.pcg_variant
    if args.pcg_half is not None:
        params.pcg_half_matrix = args.pcg_half
    if args.half_blocks is not None:
        params.half_hessian_blocks = args.half_blocks
    if args.speculate is not None:
        params.speculative_hessian = args.speculate
    result = {}
    launches0 = g.launch_count()

    if scene.get("vertex_offsets") is not None:  # batched instances: one handle over the disjoint union
        ts = scenes.build_batch_timestep(scene, precision="mixed", params=params)
    else:
        ts = scenes.build_timestep(scene, precision="mixed", params=params)
    ts.set_stream(stream.cuda_stream)
    zeros = np.zeros_like(scene["X"])
    v0 = scene.get("velocity", zeros)

    import torch.distributed as tdist

    def barrier():
        if tdist.is_available() and tdist.is_initialized():
            tdist.barrier()

    tuning = {}

    def timed_run(precision, steps, warmup, profile=False):
        # restart from the scene's initial state: the same start for every run; the state after the first
        # (untimed) step is kept for the comparison with the oracle's first step
        ts.set_precision(precision)
        ts.reset(args.stepper)
        for f in ("deformation", "prev_deform"):
            ts.set(f, zeros if scene.get("u0") is None else scene["u0"])
        ts.set("velocity", v0)
        if args.tuning is not None and precision == "mixed":  # pinned shapes: nothing swept
            ts.set_tuning(args.tuning)
            tuning[precision] = dict(args.tuning, pinned=True)
        elif args.autotune:  # launch shapes for this precision (swept once, then from the process cache)
            tuning[precision] = ts.autotune()
            if args.pcg_variant != 3:  # an explicit PCG variant outranks the sweep's choice
                ts.set_params(pcg_persistent=args.pcg_variant)
                tuning[precision]["pcg_persistent"] = args.pcg_variant
        first = None
        for i in range(warmup):
            ts.step()
            if i == 0:
                first = ts.get("deformation")
        ts.profile(profile)
        torch.cuda.synchronize()
        barrier()
        stats = []
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = g.launch_count()
        start.record(stream)
        for _ in range(steps):
            ts.step()
            stats.append(ts.stats())
        end.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = start.elapsed_time(end)
        launches = g.launch_count() - l0
        prof = {k: ts.profile_read(k) for k in ("pcg_spmv", "pcg_iteration")} if profile else None
        ts.profile(False)
        return ts, ms, stats, launches, prof, first

    # ---- headline: mixed precision, inputs resident
    with ClockSampler(dev) as clk:
        ts, ms_mixed, st_mixed, launches, _, first_mixed = timed_run("mixed", args.steps, args.warmup)
    clocks = clk.summary()
    solve_log = ts.solve_log()
    if args.arms == "mixed":
        return dict(ms_mixed=ms_mixed, ms_fp64=float("nan"), st_mixed=st_mixed, st_fp64=[], launches=launches,
                    prof=None, clocks=clocks, e2e_s=float("nan"), h2d=0, d2h=0, total_launches=0,
                    solve_log=solve_log, first={"mixed": first_mixed}, tuning=tuning)
    # ---- roofline of the dominant kernel (PCG SpMV), events around each launch, same workload
    _, _, _, _, prof, _ = timed_run("mixed", min(args.steps, 3), 1, profile=True)
    half_matrix = int(ts.params.pcg_half_matrix)  # the solves ran on the FP16 copy of the scaled matrix
    pcg_variant = int(ts.params.pcg_persistent)
    # ---- plain FP64 on the same steps
    _, ms_fp64, st_fp64, _, _, first_fp64 = timed_run("fp64", args.steps, args.warmup)
    # ---- e2e through the reference-facing API: per step h2d of the Dirichlet targets (pinned), the step,
    # d2h of the deformation (pinned)
    from ssim_gb300.libssim import fem

    fixed = np.asarray(scene["fixed"], dtype=np.int32)
    pin_targ = torch.zeros((3, fixed.size), dtype=torch.float64).pin_memory()
    facades = {"newton": fem.tet_newton_cuda, "lbfgs": fem.tet_lbfgs_cuda, "pd": fem.tet_lbfgs_pd,
               "ncg_ext": fem.tet_ncg_cuda_ext_ai}
    targ_np = pin_targ.numpy()
    if scene.get("vertex_offsets") is not None:  # batched instances: the batch handle (per-instance stopping)
        s = _HandleFacade(scenes.build_batch_timestep(scene, precision="mixed", params=params))
        s.step_.reset(args.stepper)
    elif scene.get("springs") or scene.get("tri2d") or args.stepper not in facades:
        # springs, triangles and the plain NCG have no libssim facade: the TimeStep handle itself
        s = _HandleFacade(scenes.build_timestep(scene, precision="mixed", stepper=args.stepper, params=params))
    else:
        s = facades[args.stepper](scene["X"], scene["cells"], scene["dt"], scene["E"], scene["nu"], scene["rho"],
                                  precision="mixed", params=params)
        if scene.get("E_cells") is not None:
            s.step_.set_material(scene["E_cells"], None)
        s.add_gravity(scene["gravity"])
        # the Dirichlet set before reset(): reset builds the PD matrix with its identity rows
        # (projective_dynamics.hpp:90-91); the per-step marking below only refreshes the same targets
        s.mark_dirichlet_batched(fixed, targ_np)
        s.reset()
    if args.tuning is not None:
        s.step_.set_tuning(args.tuning)
    elif args.autotune:  # the same shape as the device-timed handle: the cached choice, nothing timed
        s.step_.autotune()
    if scene.get("u0") is not None:  # the scene's initial state, as the device-timed runs start from
        for f in ("deformation", "prev_deform"):
            s.step_.set(f, scene["u0"])
    if scene.get("velocity") is not None:
        s.step_.set("velocity", scene["velocity"])
    for _ in range(args.warmup):
        s.mark_dirichlet_batched(fixed, targ_np)
        s.step()
        _ = s.deformation()
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.mark_dirichlet_batched(fixed, targ_np)
        s.step()
        d = s.deformation()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    barrier()
    result.update(
        ms_mixed=ms_mixed, ms_fp64=ms_fp64, st_mixed=st_mixed, st_fp64=st_fp64, launches=launches, prof=prof,
        clocks=clocks, e2e_s=e2e_s, h2d=fixed.size * 3 * 8 + fixed.size * 4, d2h=d.size * 8,
        total_launches=g.launch_count() - launches0, nnz=ts.nnz, solve_log=solve_log, half_matrix=half_matrix, pcg_variant=pcg_variant,
        first={"mixed": first_mixed, "fp64": first_fp64}, tuning=tuning,
    )
    if args.adjoint:
        mixed, g_mixed = run_adjoint("mixed")
        fp64, g_fp64 = run_adjoint("fp64")
        # the mixed gradients against the FP64 ones (both arms at the same 1e-6 tolerances)
        for k, (a, b) in enumerate(zip(g_mixed, g_fp64)):
            mixed[("grad_E_rel_err_vs_fp64", "grad_v0_rel_err_vs_fp64")[k]] = float(
                ((a - b).norm() / b.norm()).item())
        result["adjoint"] = [mixed, fp64]
    return result


def run_adjoint(precision, n=32, steps=40, checkpoint_every=8):
    """Differentiable rollout (32^3 hex x 6 = 196,608 tets, 40 steps, checkpoints every 8): wall time of the
    forward rollout and of the backward pass (segment recomputation + one adjoint solve per step), per
    step, with the headline Newton settings and the adjoint PCG at the same 1e-6 relative tolerance."""
    import torch

    import ssim_gb300 as g
    from ssim_gb300 import adjoint, scenes

    sc = scenes.rollout_cube(n)
    eng = adjoint.RolloutEngine(sc["X"], sc["cells"], sc["fixed"], dt=sc["dt"], nu=sc["nu"], rho=sc["rho"],
                                precision=precision, params=newton_params(g), adjoint_rtol=1e-6)
    E = torch.tensor(sc["E_cells"], dtype=torch.float64, device="cuda", requires_grad=True)
    v0 = torch.tensor(sc["v0"], dtype=torch.float64, device="cuda", requires_grad=True)
    Xt = torch.tensor(sc["X"], dtype=torch.float64, device="cuda")
    target = torch.tensor(sc["target"], dtype=torch.float64, device="cuda")
    # one untimed short rollout with its loss and backward pass (allocations and first-use costs: the first
    # torch kernel launch of a process loads torch's kernel modules, seconds on a fresh box)
    u = adjoint.rollout(E, v0, eng, 2, checkpoint_every)
    ((Xt + u - target) ** 2).sum().backward()
    E.grad, v0.grad = None, None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u = adjoint.rollout(E, v0, eng, steps, checkpoint_every)
    loss = ((Xt + u - target) ** 2).sum()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    it0 = eng.cg_iters
    loss.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return {"precision": precision, "workload": sc["name"], "steps": steps, "checkpoint_every": checkpoint_every,
            "forward_ms_per_step": round((t1 - t0) * 1e3 / steps, 3),
            "adjoint_ms_per_step": round((t2 - t1) * 1e3 / steps, 3),
            "adjoint_cg_iters_per_step": round((eng.cg_iters - it0) / steps, 1),
            "grad_finite": bool(torch.isfinite(E.grad).all().item() and torch.isfinite(v0.grad).all().item())}, \
        (E.grad.detach().clone(), v0.grad.detach().clone())


def cpu_baseline_inproc(scene, max_seconds, max_steps, warmup=0, method="newton", dump=None):
    """The FP64 oracle on this host's cores over the GPU arm's step window: ``warmup`` untimed steps of the
    same workload from its initial state, then whole timed steps (``method``: newton, lbfgs or pd) as many
    as fit in ``max_seconds`` (at least one, at most ``max_steps``).  ``dump``: a path where the state after
    the first step is saved (float64 [V, 3]) for the comparison with the GPU arms."""
    from oracle import pyoracle
    from oracle import scenes as oscenes

    op = oracle_params()
    ot = oscenes.build_oracle(scene)
    done = 0

    def one_step():
        nonlocal done
        ot.prepare_step()
        ot.compute_step(method, op)
        ot.step_next()
        done += 1
        if done == 1 and dump:
            np.save(dump, ot.get("deformation"))

    t0 = time.perf_counter()
    for _ in range(warmup):
        one_step()
    t_warm = time.perf_counter() - t0
    timed, spent = 0, 0.0
    while True:
        t1 = time.perf_counter()
        one_step()
        spent += time.perf_counter() - t1  # excludes the one-off state dump after the first step
        timed += 1
        if timed >= max_steps or spent >= max_seconds:
            break
    return {"value": timed / spent, "unit": "steps/s", "cores": pyoracle.num_threads(), "kind": "port",
            "sample": f"steps {warmup + 1}-{warmup + timed} of the same workload from its initial state "
                      f"({warmup} untimed warm-up step(s), {t_warm:.1f} s), {method}, FP64 oracle (C++/OpenMP "
                      f"restatement of the reference path), {spent:.1f} s timed on the host CPU"}


def cpu_baseline(workload, max_seconds, max_steps, warmup, stepper="newton", dump=None):
    """Runs the CPU baseline in a fresh process so its OpenMP pool does not share the process with torch."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--workload", workload,
           "--cpu-seconds", str(max_seconds), "--steps", str(max_steps), "--warmup", str(warmup),
           "--stepper", stepper, "--precond", str(SOLVER["precond"])]
    if dump:
        cmd += ["--dump-first-state", dump]
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    for line in r.stdout.splitlines()[::-1]:
        if line.startswith("{"):
            return json.loads(line)["cpu_baseline"]
    return {"value": None, "unavailable": (r.stderr or "no output")[-300:]}


def rel_err(a, b):
    """max |a - b| / max |b| over all entries."""
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def bench_config(scene, stepper, world):
    """The ``config`` object of both arms' lines (identical, so the two lines describe the same run)."""
    T, V = scene["cells"].shape[0], scene["X"].shape[0]
    cells_key = "springs" if scene.get("springs") else ("triangles" if scene.get("tri2d") else "tets")
    return {
        "workload": scene["name"], cells_key: T, "vertices": V, "dofs": 3 * V, "stepper": stepper,
        "solver": SOLVER_TEXT.get(stepper, f"{stepper}, stop |g| <= 1e-6 |g0| (per instance for batches)"),
        "precision": "GPU value: FP32 arithmetic for the Hessian, assembly and PCG (the Newton solves on an FP16 "
                     "copy of the Jacobi-scaled matrix, each checked on the FP32 values; FP16 element blocks for "
                     "their assemblies) with FP64 energy/gradient/state/dots; fp64_plain and the CPU reference: "
                     "FP64 throughout",
        "parallelism": "replicas" if world > 1 else "1 GPU",
        "l2": "working set per step ~1 GB > L2 (no explicit flush)",
    }


def max_over_ranks(values):
    """Element-wise maximum of ``values`` over the ranks of the process group (the values themselves when
    there is no group): every replica's timings reduced to the job's (slowest rank) before rank 0 reports."""
    import torch
    import torch.distributed as tdist

    if not (tdist.is_available() and tdist.is_initialized()):
        return list(values)
    t = torch.tensor(list(values), dtype=torch.float64)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return t.tolist()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="beam1m",
                    help="beam1m (default), beam_small, cube10, refbox, bar, batch, cloth512, cloth_small, sheet2d")
    ap.add_argument("--stepper", default="newton", choices=["newton", "lbfgs", "pd", "ncg", "ncg_ext"],
                    help="stepper of the timed GPU runs (and of the CPU baseline, Newton for ncg / ncg_ext)")
    ap.add_argument("--pd-kappa", type=int, default=0, choices=[0, 1, 2],
                    help="PD diffusivity: 0 the reference's (E, nu) slots, 1 Lame, 2 per element")
    ap.add_argument("--pcg-variant", type=int, default=3, choices=[0, 1, 2, 3, 4],
                    help="ssim_gb_params.pcg_persistent of the GPU arms (3: automatic; 4: pipelined PCG)")
    ap.add_argument("--pcg-half", type=int, default=None, choices=[0, 1],
                    help="FP16 copy of the scaled system matrix for the loose PCG solves (default: the library's)")
    ap.add_argument("--half-blocks", type=int, default=None, choices=[0, 1],
                    help="FP16 element Hessian blocks for the assemblies of those solves (default: the library's)")
    ap.add_argument("--speculate", type=int, default=None, choices=[0, 1],
                    help="assemble the next Newton matrix during the line search (default: the library's)")
    ap.add_argument("--precond", type=int, default=None, choices=[1, 2],
                    help="PCG preconditioner of every arm (1 Jacobi, 2 block-Jacobi); default: the bench's")
    ap.add_argument("--cpu-seconds", type=float, default=30.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--dump-first-state", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--arms", default="all", choices=["all", "mixed"], help="mixed: only the headline timed run")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the kernels' default launch shapes (no ssim_gb_autotune sweep before the timed runs)")
    ap.add_argument("--tuning", type=json.loads, default=None,
                    help="apply this launch-shape tuning (a JSON object as the bench line's 'tuning' reports for the "
                         "mixed arm) to the mixed runs instead of sweeping; for profiling runs, whose tools distort "
                         "the sweep's timings")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false",
                    help="skip the differentiable-rollout timing (32^3 cube, 40 steps)")
    args = ap.parse_args()
    if args.precond is not None:
        SOLVER["precond"] = args.precond
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")

    scene = make_scene(args.workload)
    T = scene["cells"].shape[0]
    config = bench_config(scene, args.stepper, world)
    cells_key = next(k for k in ("tets", "springs", "triangles") if k in config)
    cpu_method = args.stepper if args.stepper in ("newton", "lbfgs", "pd") else "newton"

    if args.impl == "reference":
        # the reference's CPU path (its restatement: the reference itself does not build here) over the GPU
        # arm's step window; nothing of the GPU library is loaded
        if rank == 0:
            cb = cpu_baseline_inproc(scene, args.cpu_seconds, max(1, args.steps), args.warmup, cpu_method,
                                     args.dump_first_state)
            line = {
                "metric": METRIC, "impl": "reference", "value": cb["value"], "unit": "steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SplitMix64)", "config": config,
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            }
            print(json.dumps(line), flush=True)
        if dist:
            dist.destroy_process_group()
        return

    r = run_gpu_arm(args, scene)
    # the job's times are the slowest replica's
    t_mixed, ms_fp64, e2e_s = max_over_ranks([r["ms_mixed"], r["ms_fp64"], r["e2e_s"]])
    steps_total = args.steps * world
    value = steps_total / (t_mixed / 1e3)
    fp64_value = steps_total / (ms_fp64 / 1e3)
    peak, peak_kind = load_peaks()
    prof = r["prof"]
    roofline = None
    # algorithmic bytes of one SpMV of the system matrix as a scalar CSR in FP32 (the reference's format):
    # nnz (value + column) + row pointers + x read + y written; one PCG iteration adds 7 n-vectors
    s_b, n = 4, 3 * scene["X"].shape[0]
    spmv_algo = r.get("nnz", 0) * (s_b + 4) + 4 * (n + 1) + 2 * s_b * n
    if prof and prof["pcg_iteration"]["launches"] > 0:
        p = prof["pcg_iteration"]
        avg_s = p["total_ms"] / p["launches"] / 1e3
        algo = spmv_algo + 7 * s_b * n
        variant = r.get("pcg_variant", args.pcg_variant)
        half = r.get("half_matrix", 0) == 1 and sum(s.get("half_solves", 0) for s in r["st_mixed"]) > 0
        pipe = variant == 4 or (half and variant == 3)
        kname = ("pipe_half" if pipe else "cgcg_half") if half else ("pipe_persistent" if pipe else "cgcg_persistent")
        roofline = {"kernel": {
            "pipe_half": "pipe_half_kernel (whole pipelined PCG solve in one cooperative launch on the FP16 copy of "
                         "the Jacobi-scaled matrix, full block SELL-32; unit = one PCG iteration: SpMV of m = M w "
                         "fused with the vector recurrences and dots, one reducing grid barrier)",
            "cgcg_half": "cgcg_half_kernel (whole Chronopoulos-Gear PCG solve in one cooperative launch on the FP16 "
                         "copy of the Jacobi-scaled matrix, full block SELL-32; unit = one PCG iteration: SpMV + "
                         "dots, grid reduction, vector update, grid barrier)",
            "pipe_persistent": "pipe_persistent_kernel<float> (whole pipelined PCG solve in one cooperative launch; "
                               "unit = one PCG iteration: symmetric SELL-32 SpMV of m = M w fused with the vector "
                               "recurrences and dots, one reducing grid barrier)",
            "cgcg_persistent": "cgcg_persistent_kernel<float> (whole Chronopoulos-Gear PCG solve in one cooperative "
                               "launch; unit = one PCG iteration: symmetric SELL-32 SpMV + dots, grid reduction, "
                               "vector update, grid barrier)"}[kname],
                    "bound": "hbm", "achieved": round(algo / avg_s / 1e9, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(algo / avg_s / 1e9 / peak, 4), "peak_source": peak_kind,
                    "algorithmic_bytes_per_iteration": algo, "avg_iteration_us": round(avg_s * 1e6, 2),
                    "iterations_timed": p["launches"],
                    "traffic": ncu_traffic(args.workload, kname),
                    "format_bytes_per_iteration": round(p["bytes_per_launch"]),
                    "format_frac": round(p["bytes_per_launch"] / avg_s / 1e9 / peak, 4)}
    elif prof and prof["pcg_spmv"]["launches"] > 0:
        p = prof["pcg_spmv"]
        avg_s = p["total_ms"] / p["launches"] / 1e3
        roofline = {"kernel": "pcg_spmv_kernel<float> (SELL-32 3x3-block symmetric SpMV + fused p update + p.q)",
                    "bound": "hbm", "achieved": round(spmv_algo / avg_s / 1e9, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(spmv_algo / avg_s / 1e9 / peak, 4), "peak_source": peak_kind,
                    "algorithmic_bytes_per_launch": spmv_algo, "avg_launch_us": round(avg_s * 1e6, 2),
                    "launches_timed": p["launches"], "traffic": ncu_traffic(args.workload, "pcg_spmv"),
                    "format_bytes_per_launch": round(p["bytes_per_launch"]),
                    "format_frac": round(p["bytes_per_launch"] / avg_s / 1e9 / peak, 4)}
    st = r["st_mixed"]
    stf = r["st_fp64"]
    if rank == 0:
        cb, err = None, None
        if not args.no_cpu_baseline:
            import tempfile

            with tempfile.TemporaryDirectory() as tmp:
                dump = os.path.join(tmp, "oracle_first_state.npy")
                cb = cpu_baseline(args.workload, args.cpu_seconds, args.steps, args.warmup, cpu_method, dump)
                if os.path.exists(dump):
                    uo = np.load(dump)
                    err = {k: rel_err(v, uo) for k, v in r.get("first", {}).items() if v is not None}
                    err.update(after_steps=1, measure="max|u_gpu - u_oracle| / max|u_oracle| after the first step "
                               "from the scene's initial state, every arm (and the oracle) at the bench's solver "
                               "settings (Newton stop 1e-6 relative)")
        rel_res = [s["grad_norm"] / s["grad_norm0"] if s["grad_norm0"] > 0 else 0.0 for s in st]
        line = {
            "metric": METRIC,
            "value": round(value, 4),
            "unit": "steps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(t_mixed / args.steps, 3),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32+f64",
            "data": "synthetic (seeded SplitMix64 material)",
            "config": config,
            "fp64_plain": {"value": round(fp64_value, 4), "unit": "steps/s", "ms_per_step": round(ms_fp64 / args.steps, 3),
                           "newton_iters": sum(s["newton_iters"] for s in stf),
                           "cg_iters": sum(s["cg_iters_total"] for s in stf)},
            "mixed_over_fp64": round(value / fp64_value, 3),
            "newton_iters": sum(s["newton_iters"] for s in st),
            "cg_iters": sum(s["cg_iters_total"] for s in st),
            "half_solves": sum(s.get("half_solves", 0) for s in st),
            "max_rel_residual": max(rel_res) if rel_res else None,
            "err_vs_oracle": err,
            f"{cells_key}_per_s": round(T * value, 1),
            "e2e": {"value": round(steps_total / e2e_s, 4), "unit": "steps/s", "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"]},
            "gpu_launches": r["launches"],
            "roofline": roofline,
            "cpu_baseline": cb,
            "clocks": r["clocks"],
            "tuning": {k: {f: v.get(f, 0) for f in ("elem_block", "hessian_block", "assembly_block", "gather_block",
                                                    "pcg_persistent", "pcg_max_blocks", "fused_assembly",
                                                    "pcg_half_matrix", "elem_regcap", "candidates", "pinned")}
                       for k, v in r.get("tuning", {}).items()} or None,
            "adjoint_ms_per_step": r["adjoint"][0]["adjoint_ms_per_step"] if r.get("adjoint") else None,
            "adjoint": r.get("adjoint"),
        }
        # per-step detail (Newton / PCG iteration counts, residuals, PCG length of every solve) on stderr
        print(json.dumps({"detail": {"newton_iters": [s["newton_iters"] for s in st],
                                     "cg_iters": [s["cg_iters_total"] for s in st], "rel_residual": rel_res,
                                     "half_solves": [s.get("half_solves", 0) for s in st],
                                     "half_check": [round(s.get("half_check", 0.0), 3) for s in st],
                                     "fp64_newton_iters": [s["newton_iters"] for s in stf],
                                     "fp64_cg_iters": [s["cg_iters_total"] for s in stf],
                                     "pcg_iters_per_solve_from_reset": r.get("solve_log")}}),
              file=sys.stderr, flush=True)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
