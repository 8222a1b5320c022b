"""Benchmark: Mcell-updates/s per RK stage of the explicit Navier-Stokes step.

Workload (default): the tetrahedral scaling case - a periodic [0,2pi]^3 box
of 64^3 hexes each split into 6 tets (1,572,864 cells, 3,145,728 faces),
Rusanov flux, Green-Gauss gradients + Barth-Jespersen, Re=1600, Pr=0.71,
Taylor-Green vortex at Mach 0.8, Williamson RK3, CFL 0.5, the whole step
replayed as a CUDA graph.  Synthetic mesh and initial state (no dataset).

value  = cells * stages * steps / device time  (state resident in HBM)
e2e    = the same metric through the public C ABI with host buffers: every
         step uploads the conserved state from pinned host memory, runs one
         step and reads the state back
roofline: the dominant kernel's algorithmic bytes (the fixed byte model in
         byte_model below) / its average CUDA-event duration, against the
         measured HBM copy bandwidth
cpu_baseline: the FP64 CPU oracle on the host cores, bounded sample
error_vs_fp64: the mixed path against the FP64 GPU path over the first steps
implicit: the implicit steady channel (96 x 48 x 48): seconds to a 1e-8
         relative residual with each preconditioner, end to end through the
         C ABI, the reference's implicit step on the GPU and on the host

--impl reference times the CPU implementation of the path (the reference's
own sources when they were built here, else the C restatement) on the host
cores, as independent single-threaded replicas (the reference has no
threading), and prints the same metric.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

STAGES = {"euler": 1, "rk33": 3, "rk45": 5, "ssprk3": 3}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--case", default="tgv_tet", choices=["tgv_tet", "tgv_hex", "tgv_mixed", "euler16", "channel"])
    p.add_argument("--pcs", default="coupled,none,block_jacobi",
                   help="implicit channel: the preconditioners to time (comma-separated; coupled first)")
    p.add_argument("--harvest-newton", type=int, default=200,
                   help="implicit channel: Newton steps of the harvesting solve (200: the configuration's)")
    p.add_argument("--no-learned", action="store_true",
                   help="implicit channel: skip harvesting, training and evaluating the learned preconditioner")
    p.add_argument("--n", type=int, default=64)
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--cpu-sample-stages", type=int, default=15)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--max-newton", type=int, default=400,
                   help="channel: Newton step limit per solve (a small value for profiling runs)")
    p.add_argument("--no-implicit", action="store_true",
                   help="skip the implicit channel solve the default run adds to its line")
    p.add_argument("--fp64-check-steps", type=int, default=200,
                   help="explicit steps of the mixed-vs-FP64 error check the default run adds")
    return p.parse_args()


def make_case(args):
    from fv3d_gb300 import cases
    if args.case == "tgv_tet":
        return cases.tgv_tet(args.n)
    if args.case == "tgv_hex":
        return cases.tgv_hex(args.n)
    if args.case == "tgv_mixed":
        return cases.tgv_mixed(args.n)
    return cases.euler16(args.n)


# ---------------------------------------------------------------------------
# algorithmic byte model (per kernel launch): reads of every array a pass
# semantically needs once, writes once; neighbour re-reads, padding and
# face-flux buffers not counted
# ---------------------------------------------------------------------------
def byte_model(case, precision):
    """Two passes per stage (gradient pass, flux + update pass)."""
    nc, nf = case.mesh.n_cells, case.mesh.n_faces
    r = 4 if precision == "mixed" else 8
    ng, nr = 9, 8                      # gradient / limited variables
    lsq = case.params.get("gradient", 0) == 1
    state, kreg, vol = 40, 80, 8       # U (FP64), RK register r+w (FP64), 1/V
    grad, mm = 3 * ng * r, 2 * nr * r
    face_ids = 8
    geo_grad = (6 * r) if lsq else (3 * r + r)   # LSQ weights | n*A + lambda
    geo_flux = 3 * r + 3 * r + 3 * r            # n*A, r1, r2
    grad_pass = nc * (state + vol + grad + mm) + nf * (face_ids + geo_grad)
    flux_pass = nc * (grad + mm + state + state + kreg + vol) + nf * (face_ids + geo_flux)
    return {"gradient_pass": grad_pass, "flux_update_pass": flux_pass,
            "stage": grad_pass + flux_pass}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU leg (oracle): bounded sample of residual evaluations + stage updates
# ---------------------------------------------------------------------------
def cpu_sample(case_args, n_stages, which):
    from oracle import oracle as orc
    from fv3d_gb300 import cases
    c = {"tgv_tet": cases.tgv_tet, "tgv_hex": cases.tgv_hex, "tgv_mixed": cases.tgv_mixed,
         "euler16": cases.euler16}[case_args[0]](case_args[1])
    o = orc.Oracle(which)
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(c.u0)
    dt = o.timestep_convective(0.5)
    t0 = time.perf_counter()
    o.step_lserkw2(0, 0, 0.0, dt)           # warm-up stage (forward Euler = 1 stage)
    t1 = time.perf_counter()
    for k in range(n_stages):
        o.step_lserkw2(0, k, 0.0, dt)
    t2 = time.perf_counter()
    return c.mesh.n_cells * n_stages / (t2 - t1) / 1e6, t2 - t1, t1 - t0


def cpu_baseline(args, replicas=1):
    from oracle import oracle as orc
    which = "reference" if orc.available("reference") else "restated"
    if which == "restated" and not orc.available("restated"):
        orc.build("restated")
    case_args = (args.case, args.n)
    if replicas == 1:
        v, secs, _ = cpu_sample(case_args, args.cpu_sample_stages, which)
        vals = [v]
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(replicas) as pool:
            res = pool.starmap(cpu_sample, [(case_args, args.cpu_sample_stages, which)] * replicas)
        vals = [r[0] for r in res]
        secs = max(r[1] for r in res)
    kind = "reference" if which == "reference" else "port"
    return {"value": float(sum(vals)), "unit": "Mcell-updates/s per RK stage", "cores": replicas,
            "kind": kind,
            "sample": f"{args.cpu_sample_stages} explicit stages (FP64 residual + update) on the full "
                      f"{args.case} n={args.n} mesh after 1 warm-up stage, {replicas} single-threaded "
                      f"replica(s), {secs:.1f} s"}


def workload_config(args, case):
    return {"workload": f"{args.case}_{args.n}: {case.mesh.n_cells} cells, {case.mesh.n_faces} faces, "
                        f"{'Rusanov' if case.params['flux_scheme'] == 1 else 'AUSM'}, "
                        f"{'LSQ' if case.params.get('gradient', 0) else 'Green-Gauss'}+Barth-Jespersen, "
                        f"viscous Re=1600, TGV, RK3 CFL 0.5, CUDA graph per step",
            "cells": case.mesh.n_cells, "faces": case.mesh.n_faces, "precision": args.precision,
            "l2": "working set > 129 MB L2 (records + fluxes + state ~1.3 GB); no flush needed",
            "parallelism": "replicas only (1 GPU per process, no collectives)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from fv3d_gb300 import cases  # noqa: F401
    case = make_case(args)
    replicas = max(1, min(len(os.sched_getaffinity(0)), 16))
    cb = cpu_baseline(args, replicas)
    metric = "Mcell-updates/s per RK stage"
    line = {"impl": "reference", "metric": metric, "value": cb["value"], "unit": metric,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(args, case), "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": metric, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


CHANNEL_KEYS = ("converged", "newton_steps", "gmres_iterations", "jv_evaluations", "rel_res", "wall_ms",
                "fallbacks")


def implicit_cpu_baseline(c, steps=2):
    """The reference's implicit time step (timestep_newton, implicit.c:224-351:
    one Newton iteration with the lumped Jacobian of calc_jacobian_numerical,
    ten residuals, and the block-diagonal solve; steady, so the step ends
    after its first iteration, within max_iter_inner = 2) on the host:
    seconds per step over `steps` steps after one warm-up step, one core."""
    from oracle import oracle as orc
    which = "reference" if orc.available("reference") else "restated"
    o = orc.Oracle(which)
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(c.u0)
    dt = o.timestep_convective(1.0)
    o.step_newton(0, 0.0, dt, scheme=0, solver=1, max_iter_inner=2, is_transient=False)
    t0 = time.perf_counter()
    for k in range(steps):
        o.step_newton(k + 1, 0.0, dt, scheme=0, solver=1, max_iter_inner=2, is_transient=False)
    secs = time.perf_counter() - t0
    return {"value": round(secs / steps, 4), "unit": "s per Newton step (timestep_newton)", "cores": 1,
            "kind": "reference" if which == "reference" else "port",
            "sample": f"{steps} steady backward-Euler steps of timestep_newton on the full channel (one Newton "
                      f"iteration each: 10 FP64 residuals for the lumped Jacobian + the block-diagonal solve) "
                      f"after 1 warm-up step, 1 core, {secs:.1f} s"}


def implicit_channel(args, with_cpu=True):
    """Implicit steady channel (96 x 48 x 48 stretched hexes, AUSM, second
    order, Re=1000): wall time of the pseudo-transient Newton-Krylov solve to
    a 1e-8 relative FP64 residual through the C ABI, with each
    preconditioner: the cell-coupling one (the fastest), none (FGMRES(30),
    3 restarts), block Jacobi (FGMRES(30), the configuration as written),
    and the learned one (falling back to the coupled one).  Also the
    reference's own implicit step
    (timestep_newton) on the GPU and on the host cores."""
    from fv3d_gb300 import api, cases
    c = cases.channel()
    runs = {}
    plans = [("coupled", dict(inner_dim=10, inner_sweeps=2, inner_omega=0.7, sync_every=3, pc_refresh=3,
                              max_newton=args.max_newton)),
             ("none", dict(max_restarts=3, max_newton=args.max_newton)),
             ("block_jacobi", dict(max_newton=min(args.max_newton, 100)))]
    wanted = args.pcs.split(",")
    plans = [p_ for p_ in plans if p_[0] in wanted or p_[0] == "coupled"]
    with api.Solver(c.mesh, c.params, c.region_type, c.region_prim, "fp64", "morton") as s:
        for pc, kw in plans:
            s.set_state(c.u0)
            st = s.solve_implicit(preconditioner=pc, check=False, **kw)
            runs[pc] = {k: st[k] for k in CHANNEL_KEYS}
            runs[pc]["settings"] = kw
        # end to end through the C ABI: the initial state from pinned host
        # rows, the solve, the converged state back into them
        try:
            import torch
            hb = torch.empty((c.mesh.n_cells, 5), dtype=torch.float64, pin_memory=True).numpy()
        except Exception:
            hb = np.empty((c.mesh.n_cells, 5))
        hb[:] = c.u0
        t0 = time.perf_counter()
        s.set_state(hb)
        s.solve_implicit(preconditioner="coupled", check=False, **plans[0][1])
        s.get_conserved(out=hb)
        e2e_s = time.perf_counter() - t0
        # the reference's own implicit step (lumped blocks) on the GPU, per step
        s.set_state(c.u0)
        dt = s.timestep(1.0)
        s.step_newton(0, 0.0, dt, "euler", max_iter_inner=2, is_transient=False, check=False)
        t1 = time.perf_counter()
        for k in range(5):
            s.step_newton(k + 1, 0.0, dt, "euler", max_iter_inner=2, is_transient=False, check=False)
        gpu_step = (time.perf_counter() - t1) / 5
        if not args.no_learned:
            # training pairs from plain Newton-Krylov steps (a separate,
            # untimed solve harvesting 100,000 cells per Newton step, up to
            # 2e7 pairs), a few epochs of Adam, then the learned solve, whose
            # stagnating cycles are redone with the coupled preconditioner
            s.mlp_init(5)
            s.mlp_harvest(100000, 20000000)
            s.set_state(c.u0)
            hv = s.solve_implicit(preconditioner="none", max_newton=args.harvest_newton, max_restarts=3,
                                  check=False)
            s.mlp_harvest(0, 20000000)
            tr = s.mlp_train(epochs=4, batch=16384, lr=2e-3)
            tr["harvest_newton_steps"] = hv["newton_steps"]
            s.set_state(c.u0)
            kw = dict(plans[0][1])
            st = s.solve_implicit(preconditioner="learned", fallback="coupled", check=False, **kw)
            runs["learned"] = {k: st[k] for k in CHANNEL_KEYS}
            runs["learned"]["settings"] = dict(kw, fallback="coupled")
            runs["learned"]["train"] = tr
            # one application of the network to a field on the mesh: the
            # tcgen05 kernels (used) and the warp-level mma.sync ones
            peaks = {}
            pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
            if os.path.exists(pk):
                with open(pk) as f:
                    peaks = json.load(f)
            flop = 21632.0 * c.mesh.n_cells
            app = {}
            for kind in ("mma_sync", "tcgen05"):
                s.mlp_set_kernel(kind)
                ms = s.profile_mlp(50)
                app[kind] = {"ms": round(ms, 5), "tflops": round(flop / (ms * 1e-3) / 1e12, 2)}
            app["flop_per_application"] = flop
            app["bf16_peak_tflops"] = peaks.get("bf16_tflops")
            app["frac_tcgen05"] = (round(app["tcgen05"]["tflops"] / peaks["bf16_tflops"], 4)
                                   if peaks.get("bf16_tflops") else None)
            runs["learned"]["mlp_apply"] = app
    conv = {k: v for k, v in runs.items() if v["converged"]}
    best = min(conv, key=lambda k: conv[k]["wall_ms"]) if conv else "coupled"
    out = {"metric": "seconds to 1e-8 relative steady residual", "value": round(runs[best]["wall_ms"] / 1e3, 4),
           "unit": "s", "higher_is_better": False, "preconditioner": best,
           "workload": f"channel 96x48x48: {c.mesh.n_cells} cells, {c.mesh.n_faces} faces, AUSM, Green-Gauss "
                       "linear, no limiter, Re=1000, adiabatic walls, inflow, pressure outlet, periodic z; "
                       "pseudo-transient Newton, SER CFL 100 -> 1e4, FGMRES(30) to eta 0.01, FD Jv in FP32, "
                       "FP64 residual and update",
           "e2e": {"value": round(e2e_s, 4), "unit": "s",
                   "h2d_bytes_per_step": int(hb.nbytes), "d2h_bytes_per_step": int(hb.nbytes),
                   "note": "wall clock around fv3d_set_state (pinned host rows) + fv3d_solve_implicit "
                           "(coupled) + fv3d_get_conserved (pinned host rows); one 'step' = one solve"},
           "reference_step_on_gpu_s": round(gpu_step, 5),
           "runs": runs}
    if with_cpu:
        out["cpu_baseline"] = implicit_cpu_baseline(c)
    return out


def run_channel(args):
    """The implicit channel alone, as its own JSON line."""
    imp = implicit_channel(args, with_cpu=not args.no_cpu_baseline)
    line = {"metric": imp["metric"], "value": imp["value"], "unit": "s", "n_gpus": 1, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 (Jv f32)", "data": "synthetic",
            "config": {"workload": imp["workload"], "preconditioner": imp["preconditioner"]},
            "implicit": imp}
    print(json.dumps(line))


def max_over_ranks(ms, dist):
    """The slowest rank's timed-region length (the job's time)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(cells, stages, ms, world):
    """Mcell-updates/s per RK stage of all ranks together (each rank a
    replica of the same workload)."""
    return cells * stages / (ms * 1e-3) / 1e6 * world


def main():
    args = parse()
    if args.case == "channel":
        run_channel(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # barrier + max over ranks only
        dist.init_process_group("gloo")
    from fv3d_gb300 import api
    case = make_case(args)
    scheme = "rk33"
    nst = STAGES[scheme]
    s = api.Solver(case.mesh, case.params, case.region_type, case.region_prim, args.precision,
                   "morton", device=local)
    s.set_state(case.u0)
    # warm-up (includes graph capture)
    s.step_explicit(scheme, max(3, args.warmup), cfl=0.5)
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        st = s.step_explicit(scheme, args.steps, cfl=0.5)   # CUDA events around the graph replays
    if dist:
        dist.barrier()
    ms = max_over_ranks(st["elapsed_ms"], dist)
    n_stages = args.steps * nst
    value = whole_job_value(case.mesh.n_cells, n_stages, ms, world)
    # per-kernel durations: CUDA events around each launch of real steps
    # (the launches the timed graph replays, the same coefficients and the
    # device dt), averaged over every stage of 20 steps after the timed region
    prof = [float(x) for x in s.profile_step(scheme, 20, 0.5)]
    kms = prof[:2]
    model = byte_model(case, args.precision)
    if args.precision == "mixed":
        # two launches per stage: k_mx_sides (gradient pass), k_mx_flux_update
        names = ["gradient_pass", "flux_update_pass"]
        kernels = ["k_mx_sides", "k_mx_flux_update"]
        kt = [float(kms[0]), float(kms[1])]
        kbytes = [model["gradient_pass"], model["flux_update_pass"]]
    else:
        # FP64: gradients (gradient pass), face flux + gather/update (flux pass)
        names = ["gradient_pass", "flux_update_pass"]
        kernels = ["k_gradients", "k_face_flux+k_gather_update"]
        kt = [float(kms[0]), float(kms[1])]
        kbytes = [model["gradient_pass"], model["flux_update_pass"]]
    dom = int(np.argmax(kt))
    peak, peak_kind = measured_peaks()
    achieved = kbytes[dom] / (kt[dom] * 1e-3) / 1e9
    stage_ms = ms / n_stages
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            traffic = json.load(f).get(f"{args.case}_{args.n}_{args.precision}", {}).get(kernels[dom])
    roofline = {"bound": "hbm", "kernel": kernels[dom], "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_kind": peak_kind, "algorithmic_bytes": kbytes[dom],
                "kernel_ms": {k: round(t, 5) for k, t in zip(kernels, kt)},
                "flux_ms_last_stage": round(prof[2], 5),
                "stage_ms": round(stage_ms, 5),
                "stage_frac": round(model["stage"] / (stage_ms * 1e-3) / 1e9 / peak, 4),
                "stage_bytes": model["stage"]}
    # end to end through the public API with pinned host buffers
    e2e = None
    try:
        import torch
        hb = torch.empty((case.mesh.n_cells, 5), dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        hb = np.empty((case.mesh.n_cells, 5))
    s.get_conserved(out=hb)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        # the state from page-locked host rows, one step, the state back into
        # them (fv3d_step_explicit_io: one call, one synchronisation)
        s.step_explicit_io(scheme, 1, cfl=0.5, u_in=hb, u_out=hb)
    t1 = time.perf_counter()
    e2e = {"value": case.mesh.n_cells * nst * args.e2e_steps / (t1 - t0) / 1e6,
           "unit": "Mcell-updates/s per RK stage", "h2d_bytes_per_step": int(hb.nbytes),
           "d2h_bytes_per_step": int(hb.nbytes), "steps": args.e2e_steps,
           "note": "wall clock around fv3d_step_explicit_io: pinned host state in (H2D), 1 graph step, "
                   "host state out (D2H), every step"}
    s.close()
    # error of the mixed path against the FP64 GPU path over the first
    # fp64_check_steps steps of the same run (from the initial state)
    err64 = None
    if args.precision == "mixed" and args.fp64_check_steps > 0:
        outs = {}
        for prec in ("mixed", "fp64"):
            with api.Solver(case.mesh, case.params, case.region_type, case.region_prim, prec, "morton",
                            device=local) as s2:
                s2.set_state(case.u0)
                s2.step_explicit(scheme, args.fp64_check_steps, cfl=0.5)
                outs[prec] = s2.get_conserved()
        d = np.linalg.norm(outs["mixed"] - outs["fp64"], axis=0)
        ref = np.linalg.norm(outs["fp64"], axis=0)
        err64 = {"steps": args.fp64_check_steps,
                 "rel_l2": [float(x) for x in d / np.maximum(ref, ref[0])],
                 "note": "mixed FP32/FP64 against the FP64 GPU path (itself within 1e-15 of the reference's "
                         "own CPU solution after 500 steps, tests/test_gpu_fullrun.py), relative L2 per "
                         "conserved variable"}
    if rank != 0:
        return
    cb = None
    if not args.no_cpu_baseline and world == 1:
        cb = cpu_baseline(args, 1)
    imp = None
    if world == 1 and not args.no_implicit:
        imp = implicit_channel(args, with_cpu=not args.no_cpu_baseline)
    line = {"metric": "Mcell-updates/s per RK stage", "value": round(value, 2),
            "unit": "Mcell-updates/s per RK stage", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": workload_config(args, case), "roofline": roofline, "cpu_baseline": cb,
            "e2e": e2e, "gpu_launches": args.steps * ((2 if args.precision == "mixed" else 3) * nst + 1),
            "clocks": clk.summary(), "error_vs_fp64": err64, "implicit": imp}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
