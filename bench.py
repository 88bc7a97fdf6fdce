#!/usr/bin/env python
"""Throughput benchmark: IMPES cell-steps/s on the 1024 x 1024 parallel quarter-five-spot.

Workload (one "step" = one IMPES step: pressure solve, Darcy velocities, CFL dt, TR source,
Crank-Nicolson Peaceman dispersion, symmetric-parallel MUSCL transport, TR source, CN):
  1024^2 cells on [0, sqrt 2]^2, four corner one-cell wells (two injectors, two producers),
  M = 41 quarter-power mobility, harmonic averaging, nu = 1 (5-point), porosity 1, CFL 0.5,
  MUSCL/van Leer, alpha_l = 1e-3, alpha_t = 1e-4 (cell units), molecular diffusion 1e-6,
  V-cycle preconditioned CG to relative residual 1e-10 (FP64 unless --precision mixed;
  V(1,2) for the five-point operator, V(1,1) for the nine-point one),
  c0 = 0 plus a seeded U[0, 1e-3) perturbation in a 4-cell band next to each injector.
Synthetic inputs (no dataset).  The working set (~150 MB) is close to L2 (129 MB), so L2 is
flushed (a 256 MB write) between timed steps; each step is timed with CUDA events.

--impl reference times the reference's CPU implementation on the host cores: the reference
itself cannot be built (Blitz++, libconfig++, HYPRE, MPI are unavailable), so its FP64 C++
restatement (oracle/) runs instead, multi-threaded, on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 1024
METRIC = "cell-steps/s @1024^2 (IMPES step: FP64 MG to 1e-10 + MUSCL + CN dispersion)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--n", type=int, default=None, help="grid side (default 1024; 4096 for --study pressure)")
    ap.add_argument("--nu", type=float, default=1.0,
                    help="stencil weight: 1 = five-point (the default workload), 2/3 = the reference examples' "
                         "weighted nine-point operator")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--later-after", type=int, default=1000,
                    help="time a second window of --steps steps after this many IMPES steps (0: skip)")
    ap.add_argument("--no-large-roofline", action="store_true",
                    help="skip the 4096^2 roofline probe of the fine-level sweep")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the in-run training of the warm-start network for the pressure-solve line")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch each kernel on the stream instead of replaying the step graph (for ncu)")
    ap.add_argument("--study", default=None, choices=["pressure", "warmstart", "ensemble", "learned", "network", "sweep"],
                    help="pressure: FP64 vs mixed-precision solves on re-seeded heterogeneous fields; "
                         "warmstart: V-cycles and ms per solve along the IMPES run for zero and previous-step "
                         "initial guesses")
    ap.add_argument("--solves", type=int, default=20, help="re-seeded solves of the pressure study")
    ap.add_argument("--members-per-size", type=int, default=64,
                    help="ensemble study: realisations at each of 128^2, 256^2, 384^2, 512^2")
    ap.add_argument("--no-autotune", action="store_true", help="ensemble study: keep the default schedules")
    ap.add_argument("--quick", action="store_true", help="network study: two shapes, few repetitions (profiling)")
    ap.add_argument("--members", type=int, default=100, help="learned study: 256^2 realisations for training pairs")
    ap.add_argument("--pairs-per-member", type=int, default=200, help="learned study: pairs per realisation")
    ap.add_argument("--epochs", type=float, default=2.0, help="learned study: training epochs")
    ap.add_argument("--seed", type=int, default=7, help="learned study: network initialisation seed")
    ap.add_argument("--net-in", default=None, help="learned study: load trained weights (.npy) instead of training")
    ap.add_argument("--net-out", default=None, help="learned study: save the trained weights (.npy)")
    ap.add_argument("--eval-sizes", default="512,1024", help="learned study: evaluation grid sides")
    ap.add_argument("--eval-seeds", type=int, default=4, help="learned study: held-out realisations per size")
    ap.add_argument("--eval-samples", type=int, default=8, help="learned study: timed solves per realisation")
    ap.add_argument("--eval-skip", type=int, default=20, help="learned study: IMPES steps before the first solve")
    ap.add_argument("--eval-every", type=int, default=10, help="learned study: IMPES steps between solves")
    ap.add_argument("--eval-factor", type=int, default=0,
                    help="learned study: feature averaging factor (default N / 256, the training grid)")
    ap.add_argument("--eval-ell", type=float, default=0.0,
                    help="learned study: permeability correlation length in cells (default 16 N / 256, the "
                         "training fields' length relative to the domain)")
    return ap.parse_args()


def dist_info():
    from impec2d_gb300.replicas import dist_info as _d
    return _d()


def initial_state(N, seed=1234):
    """c0 and q (device layout, numpy) of the workload."""
    import numpy as np
    rng = np.random.default_rng(seed)
    c = np.zeros((N, N))
    for (ci, cj) in ((0, 0), (N - 1, N - 1)):  # injectors of the parallel configuration
        for i in range(5):
            for j in range(5):
                if i + j < 4 or (i + j == 4):
                    ii = i if ci == 0 else N - 1 - i
                    jj = j if cj == 0 else N - 1 - j
                    c[ii, jj] = rng.uniform(0.0, 1e-3)
    L = math.sqrt(2.0)
    dx = L / N
    q = np.zeros(N * N)
    val = 1.0 / (dx * dx)  # InitOneCellParallel (src/Util.cpp:565-573)
    q[0] = val
    q[N * N - 1] = val
    q[N - 1] = -val
    q[(N - 1) * N] = -val
    return c, q


def bench_config(N, precision="fp64", nu=1.0):
    """The `config` object of both arms' JSON lines: the same workload, named the same way."""
    return {"workload": f"parallel quarter-five-spot {N}x{N}, MUSCL + CN Peaceman (alpha_l 1e-3, alpha_t 1e-4, "
                        f"Dm 1e-6), pressure by multigrid to relative residual 1e-10"
                        + (f", nu = {nu:.4g} (weighted nine-point)" if nu != 1.0 else ""),
            "precision": precision, "l2": "flushed (256 MB write) between timed steps",
            "parallelism": "one replica per process"}


def workload_params(E, N, precision, nu=1.0):
    L = math.sqrt(2.0)
    return E.default_params(N, N, x_ub=L, y_ub=L, stype=E.PARALLEL, hmtype=E.MUSCL, nu=nu, diffusion=1,
                            alpha_l=1e-3, alpha_t=1e-4, Dm=1e-6, cfl=0.5, porosity=1.0, eps=1e-10, para_eps=1e-10,
                            precision=E.PREC_MIXED if precision == "mixed" else E.PREC_FP64, max_cycles=200)


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    def __init__(self, gpu):
        self.gpu, self.p, self.path = gpu, None, None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        self.path = f"/tmp/impec_clocks_{os.getpid()}.csv"
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}", "--format=csv,noheader",
                                       "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1].split()[0]))
                mx = float(f[2].split()[0])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(N, steps, threads=None, warmup=0, budget_s=None):
    """Oracle (FP64 C++ restatement, OpenMP) on the host cores: cell-steps/s of `steps` steps
    after `warmup` untimed ones.  With budget_s, the timed steps stop once they have taken
    that long (at least one).  Returns (cell-steps/s, threads, seconds, steps timed)."""
    import ctypes as C

    import numpy as np

    import oracle as O
    O.build()
    L = O.lib()
    prev_threads = L.or_set_num_threads(threads) if threads else None
    P = O.make_params(N1=N, N2=N, x_ub=math.sqrt(2.0), y_ub=math.sqrt(2.0), stype=O.PARALLEL, hmtype=O.MUSCL, nu=1.0,
                      diffusion=1, alpha_l=1e-3, alpha_t=1e-4, Dm=1e-6, cfl=0.5, eps=1e-10, para_eps=1e-10)
    c0, q = initial_state(N)
    c = O.with_ghosts(P, c0)
    p, v = np.zeros(O.scalar_shape(P)), np.zeros(O.vel_shape(P))
    S = O.State()
    S.prev_first_sweep = 1
    tidx = C.c_int(0)
    def step():
        L.or_impes_step(C.byref(P), C.byref(S), O.ptr(c), O.ptr(p), O.ptr(v), O.ptr(q), None, 0, C.byref(tidx), 1,
                        1e-10)
    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        step()
        done += 1
        if budget_s and time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    used = L.or_num_threads()
    if prev_threads:
        L.or_set_num_threads(prev_threads)
    return N * N * done / dt, used, dt, done


def pressure_solves(E, ctx, N, q, args, flush):
    """ms per pressure solve to 1e-10 on the run's current state: the concentration now and the
    pressure of the step before it.  Modes: plain FP64 multigrid from a zero guess (the
    reference's method, src/MGSolver.cpp:575-577) and mixed precision from zero; both from the
    previous step's pressure; and mixed precision with the learned warm start (the previous
    pressure moved along the network's prediction), the network trained here first on pairs
    the solver writes from 256^2 heterogeneous realisations (a short in-run training).  Each
    timed solve starts from the same c and previous p; CUDA events bracket the captured solve."""
    import torch

    from impec2d_gb300.workloads import device_view
    cd, pd = [device_view(x, (N, N)) for x in ctx.state_ptrs()[:2]]
    c_now, p_prev = cd.clone(), pd.clone()
    out = {}
    net = None
    if not args.no_learned:
        from impec2d_gb300 import learned as LW
        net = E.Net(seed=args.seed)
        X, T, t_gen = LW.generate_pairs(E, 20, 100, N=256, every=2, skip=2)
        hist, t_train = LW.train(net, X, T, epochs=4, batch=64, lr=3e-4, weight_decay=1e-4)
        out["learned_training"] = {"pairs": int(X.shape[0]), "grid": "256x256 heterogeneous realisations",
                                   "epochs": 4, "steps": hist[-1][0], "final_batch_loss": hist[-1][1],
                                   "generation_s": t_gen, "train_s": t_train}
        del X, T
        torch.cuda.empty_cache()
    modes = [("fp64", "zero"), ("mixed", "zero"), ("fp64", "previous"), ("mixed", "previous")]
    if net:
        modes.append(("mixed", "learned"))
    for prec, guess in modes:
        Pp = workload_params(E, N, prec, args.nu)
        Pp.warm_start = 0 if guess == "zero" else 1
        cp = E.Context(Pp)
        cp.upload(None, q, ghost=2)
        if guess == "learned":
            net.attach(cp, factor=max(1, N // 256), mode=1)
        cc, pc = [device_view(x, (N, N)) for x in cp.state_ptrs()[:2]]

        def reset():
            cc.copy_(c_now)
            pc.copy_(p_prev)
        reset()
        cp.pressure_solve_resident()  # capture and warm-up
        ts, cyc = [], []
        for _ in range(5):
            reset()
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            cp.pressure_solve_resident(sync=False)
            e1.record()
            e1.synchronize()
            c_, rr, rr0 = cp.last_solve()
            cyc.append(c_)
            ts.append(e0.elapsed_time(e1))
        key = prec if guess == "zero" else f"{prec}_{guess}"
        out[key] = {"ms_per_solve": statistics.median(ts), "cycles": statistics.median(cyc), "relres": rr,
                    "initial_relres": rr0, "guess": guess}
        if guess == "learned":
            out[key]["alpha"] = E.Net.last_alpha(cp)
            E.Net.detach(cp)
        cp.close()
    if net:
        net.close()
    if "mixed_learned" in out:
        out["mixed_learned_vs_fp64_speedup"] = out["fp64"]["ms_per_solve"] / out["mixed_learned"]["ms_per_solve"]
    return out


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    n = args.n or N_DEFAULT
    # the W warm-up and K timed IMPES steps of the GPU arm, on all host cores; the timed part
    # stops early (stated in "sample") if it would run past four minutes
    cps, cores, secs, done = cpu_baseline(n, args.steps, warmup=args.warmup, budget_s=240.0)
    sample = f"{done} timed IMPES steps at {n}^2 after {args.warmup} warm-up steps from t=0 ({secs:.1f} s)"
    if done < args.steps:
        sample += f"; stopped after {done} of {args.steps} steps at the four-minute budget"
    line = {"impl": "reference", "metric": METRIC, "value": cps, "unit": "cell-steps/s", "n_gpus": args.gpus,
            "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * secs / done,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(n), "solver": {"schedule": "oracle multigrid V-cycles (stationary)",
                                                   "threads": cores},
            "cpu_baseline": {"value": cps, "unit": "cell-steps/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": cps, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def grf(N, ell, seed):
    from impec2d_gb300.workloads import grf as _grf
    return _grf(N, ell, seed)


def study_pressure(args):
    """FP64 vs mixed-precision pressure solves to 1e-10 on re-seeded heterogeneous fields:
    N^2 diagonal quarter-five-spot on the unit square, c = logistic(4 g_c) with g_c a GRF of
    correlation length 32 cells, ln K = GRF(sigma 1, correlation length 16), M = 41
    quarter-power mobility.  Reports ms per solve, V-cycles, and the mixed-precision solution's
    deviation from the FP64 one."""
    import torch

    import impec2d_gb300 as E
    from impec2d_gb300 import build as B
    B.build()
    N = args.n or 4096
    ctxs = {}
    for prec in ("fp64", "mixed"):
        P = E.default_params(N, N, stype=E.DIAGONAL, hmtype=E.MUSCL, nu=1.0, eps=1e-10, max_cycles=200,
                             precision=E.PREC_MIXED if prec == "mixed" else E.PREC_FP64)
        ctxs[prec] = E.Context(P)
    dx = 1.0 / N
    q = torch.zeros(N * N, dtype=torch.float64, device="cuda")
    q[0], q[-1] = 1.0 / (dx * dx), -1.0 / (dx * dx)
    for cx in ctxs.values():
        cx.set_source(q)
    res = {k: {"ms": [], "cycles": [], "relres": []} for k in ctxs}
    errs = []
    p = {k: torch.zeros((N, N), dtype=torch.float64, device="cuda") for k in ctxs}
    for s in range(args.solves):
        c = torch.sigmoid(4.0 * grf(N, 32.0, 1000 + 2 * s)).contiguous()
        K = torch.exp(grf(N, 16.0, 1001 + 2 * s)).contiguous()
        for k, cx in ctxs.items():
            cx.set_permeability(K, K)
            p[k].zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            cyc, rr, _ = cx.pressure_solve(c, p[k], 1e-10)
            e1.record()
            torch.cuda.synchronize()
            res[k]["ms"].append(e0.elapsed_time(e1))
            res[k]["cycles"].append(cyc)
            res[k]["relres"].append(rr)
        errs.append(float(torch.linalg.vector_norm(p["mixed"] - p["fp64"]) / torch.linalg.vector_norm(p["fp64"])))
    out = {"study": "pressure", "workload": f"{N}x{N} diagonal quarter-five-spot, c = logistic(4 GRF(l=32)), "
                                            f"ln K = GRF(sigma=1, l=16), M=41, tol 1e-10",
           "solves": args.solves, "data": "synthetic (seeded GRFs on the GPU)"}
    for k, r in res.items():
        out[k] = {"ms_per_solve_median": statistics.median(r["ms"]), "ms_per_solve_mean": statistics.mean(r["ms"]),
                  "cycles_mean": statistics.mean(r["cycles"]), "relres_max": max(r["relres"])}
    out["mixed_vs_fp64"] = {"speedup": out["fp64"]["ms_per_solve_median"] / out["mixed"]["ms_per_solve_median"],
                            "rel_l2_diff_max": max(errs)}
    print(json.dumps(out))
    for cx in ctxs.values():
        cx.close()


def study_sweep(args):
    """The fine-level red-black sweep of the bench workload at --n (default 4096): one pressure
    solve on the workload's initial state (kernel by kernel, so profilers see each launch), then
    the cold roofline probe of the sweep, for the one-launch and the two-launch variants."""
    import numpy as np
    import torch

    import impec2d_gb300 as E
    from impec2d_gb300 import build as B
    B.build()
    N = args.n or 4096
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = {"study": "sweep", "grid": f"{N}x{N}", "precision": args.precision}
    for name, tile in (("default", None), ("two_launch", 0)):
        P = workload_params(E, N, args.precision, args.nu)
        ctx = E.Context(P)
        if tile is not None:
            ctx.set_tuning("tile_cells", tile)
        c0, q = initial_state(N)
        ctx.set_source(torch.from_numpy(q).cuda())
        p = torch.zeros((N, N), dtype=torch.float64, device="cuda")
        cyc, rr, _ = ctx.pressure_solve(torch.from_numpy(np.ascontiguousarray(c0)).cuda(), p, 1e-10)
        out[name] = {"solve_cycles": cyc, "relres": rr,
                     "roofline": E.roofline_probe(ctx, P, args.precision, flush=flush, reps=args.steps)}
        ctx.close()
    print(json.dumps(out))


def study_warmstart(args):
    """V-cycles and ms per pressure solve along the 1024^2 IMPES run, zero initial guess (the
    reference's choice) against the previous step's pressure."""
    import numpy as np
    import torch

    import impec2d_gb300 as E
    from impec2d_gb300 import build as B
    B.build()
    N = args.n or N_DEFAULT
    out = {"study": "warmstart", "workload": f"parallel quarter-five-spot {N}x{N} (IMPES steps as in the bench)",
           "steps": args.steps}
    for warm in (0, 1):
        P = workload_params(E, N, args.precision, args.nu)
        P.warm_start = warm
        ctx = E.Context(P)
        c0, q = initial_state(N)
        g = 2
        cg = np.zeros((N + 2 * g, N + 2 * g))
        cg[g:g + N, g:g + N] = c0
        ctx.upload(cg, q, ghost=g)
        ctx.set_time(0.0)
        cyc, ms = [], []
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            info = ctx.step()
            e1.record()
            torch.cuda.synchronize()
            cyc.append(info.its)
            ms.append(e0.elapsed_time(e1))
        out["previous_step" if warm else "zero"] = {"cycles_mean": statistics.mean(cyc[1:] or cyc),
                                                    "ms_per_step_median": statistics.median(ms[1:] or ms)}
        ctx.close()
    print(json.dumps(out))


def ensemble_member(E, N, seed, precision="mixed"):
    """One realisation of the batched-ensemble workload (lognormal K with sigma 0.5 and
    correlation 16 cells, M from {5, 20, 41, 100}, diagonal or parallel by seed, MUSCL +
    Peaceman, FP64 transport, pressure in the given precision)."""
    from impec2d_gb300.workloads import realisation
    return realisation(E, N, seed, precision=precision)


def study_ensemble(args):
    """Batched ensemble: members of four sizes advanced by one graph launch per IMPES step,
    against the same members stepped one after another."""
    import torch

    import impec2d_gb300 as E
    from impec2d_gb300 import build as B
    B.build()
    sizes = (128, 256, 384, 512)
    k = args.members_per_size
    tuned = {}
    if not args.no_autotune:  # one probe per size, on its own state after a few steps
        for N in sizes:
            probe = ensemble_member(E, N, 0)
            probe.run_steps(3)
            probe.step()
            rep = probe.autotune(reps=3)
            tuned[N] = {n: probe.get_tuning(n) for n in ("mg_pre", "mg_post", "cluster")}
            tuned[N]["report"] = rep.strip().splitlines()[-1]
            probe.close()
    from impec2d_gb300.replicas import dist_info, max_over_ranks, shard
    rank, world, local = dist_info()
    if world > 1:  # members dealt to ranks by index; no exchange between ranks
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    listing = [(N, i) for N in sizes for i in range(k)]
    members = []
    for j in shard(len(listing), rank, world):
        N, i = listing[j]
        ctx = ensemble_member(E, N, i)
        for name, v in tuned.get(N, {}).items():
            if name != "report":
                ctx.set_tuning(name, v)
        members.append((N, ctx))
    cells = sum(N * N for N, _ in listing)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    t0 = time.perf_counter()
    ens = E.Ensemble([c for _, c in members])
    t_capture = time.perf_counter() - t0
    ens.step(args.warmup)
    barrier()
    t0 = time.perf_counter()
    ens.step(args.steps)
    barrier()
    t_ens = max_over_ranks(time.perf_counter() - t0, device="cuda")
    # the same members one after another (each its own graph launch per step)
    for _, c in members:
        c.run_steps(1)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for _, c in members:
            c.run_steps(1)
    barrier()
    t_seq = max_over_ranks(time.perf_counter() - t0, device="cuda")
    out = {"study": "ensemble",
           "workload": f"{len(members)} realisations, {k} each at 128^2, 256^2, 384^2, 512^2; lognormal K "
                       f"(sigma 0.5), M in {{5,20,41,100}}, diagonal/parallel by seed; MUSCL + Peaceman; "
                       f"mixed-precision pressure",
           "cells": cells, "steps": args.steps, "warmup": args.warmup,
           "ensemble": {"cell_steps_per_s": cells * args.steps / t_ens, "ms_per_step": 1e3 * t_ens / args.steps,
                        "capture_s": t_capture},
           "one_after_another": {"cell_steps_per_s": cells * args.steps / t_seq, "ms_per_step": 1e3 * t_seq / args.steps},
           "speedup": t_seq / t_ens, "autotune": tuned or None, "data": "synthetic (seeded GRF permeability)",
           "n_gpus": world, "scaling": "strong (members dealt to ranks)"}
    if rank == 0:
        print(json.dumps(out))
    ens.close()
    for _, c in members:
        c.close()


NET_LAYERS = [(8, 32, 0), (32, 32, 0), (32, 64, 1), (64, 64, 1), (64, 128, 2), (128, 128, 2), (128, 256, 3),
              (256, 256, 3), (256, 128, 2), (128, 128, 2), (128, 64, 1), (64, 64, 1), (64, 32, 0), (32, 32, 0),
              (32, 8, 0)]  # (cin, cout, level) of the warm-start network


def net_flops(B, H, W):
    """Dense 3x3-convolution FLOPs of one forward pass (2 * 9 * cin * cout per output pixel)."""
    return sum(2 * 9 * ci * co * B * (H >> lv) * (W >> lv) for ci, co, lv in NET_LAYERS)


def study_network(args):
    """Tensor-core throughput of the warm-start network's own kernels: forward passes at the
    inference shapes (one 256^2 / 512^2 map) and the training batch (64 x 256^2), and AdamW
    training steps (forward + input and weight gradients = 3x the forward FLOPs), against the
    measured dense BF16 peak.  CUDA events around `reps` back-to-back calls."""
    import torch

    import impec2d_gb300 as E
    from impec2d_gb300 import build as B
    B.build()
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    net = E.Net(seed=1)
    out = {"study": "network", "peak_bf16_tflops": peak,
           "peak_source": "measured" if "bf16_tflops" in peaks else "fallback", "data": "synthetic (random maps)"}
    reps = 3 if args.quick else 20
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    shapes = [(1, 256), (64, 256)] if args.quick else [(1, 128), (1, 256), (1, 512), (8, 256), (64, 256)]
    for Bn, H in shapes:
        X = torch.randn((Bn, H, H, 8), generator=g, device="cuda").to(torch.bfloat16)
        for _ in range(2):
            net.forward(X)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            net.forward(X)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / reps
        tf = net_flops(Bn, H, H) / ms / 1e9
        out[f"forward_{Bn}x{H}x{H}"] = {"ms": ms, "tflops": tf, "frac": tf / peak}
    for Bn, H in [(64, 256)]:
        X = torch.randn((Bn, H, H, 8), generator=g, device="cuda").to(torch.bfloat16)
        T = torch.randn((Bn, H, H), generator=g, device="cuda")
        net.train_batch(X, T, lr=1e-6)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(max(2, reps // 4)):
            net.train_batch(X, T, lr=1e-6)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / max(2, reps // 4)
        tf = 3 * net_flops(Bn, H, H) / ms / 1e9
        out[f"train_step_{Bn}x{H}x{H}"] = {"ms": ms, "tflops": tf, "frac": tf / peak}
    print(json.dumps(out))
    net.close()


def study_learned(args):
    """Learned warm start (the heterogeneous batched-ensemble family): training pairs written
    by the solver from 256^2 realisations, AdamW training (lr 3e-4, batch 64) with the
    engine's tensor-core kernels, then pressure solves to 1e-10 along held-out 512^2 and
    1024^2 runs, started from zero, from the previous pressure, and from the previous pressure
    moved by the network's prediction, in FP64 and mixed precision.  Reports V-cycles and ms per
    solve (CUDA events around the captured solve)."""
    import numpy as np
    import torch

    import impec2d_gb300 as E
    from impec2d_gb300 import build as B
    from impec2d_gb300 import learned as LW
    from impec2d_gb300.workloads import device_view, realisation
    B.build()

    def log(m):
        print(m, file=sys.stderr, flush=True)
    out = {"study": "learned", "data": "synthetic (seeded lognormal-K realisations; pairs written by the GPU solver)"}
    net = E.Net(seed=args.seed)
    if args.net_in:
        net.set_parameters(np.load(args.net_in))
        out["net"] = {"loaded": os.path.basename(args.net_in)}
    else:
        X, T, t_gen = LW.generate_pairs(E, args.members, args.pairs_per_member, N=256, every=2, skip=2, log=log)
        nval = args.pairs_per_member * max(1, args.members // 20)  # whole realisations held out
        Xva, Tva, Xtr, Ttr = X[:nval], T[:nval], X[nval:], T[nval:]
        v0 = LW.validation_mse(net, Xva, Tva)
        hist, t_train = LW.train(net, Xtr, Ttr, epochs=args.epochs, batch=64, lr=3e-4, weight_decay=1e-4,
                                 Xval=Xva, Tval=Tva, log=log)
        out["training"] = {"pairs": int(X.shape[0]), "train_pairs": int(Xtr.shape[0]), "validation_pairs": nval,
                           "grid": "256x256", "generation_s": t_gen, "epochs": args.epochs, "batch": 64, "lr": 3e-4,
                           "steps": hist[-1][0], "train_s": t_train, "ms_per_train_step": 1e3 * t_train / hist[-1][0],
                           "validation_mse_untrained": v0, "history": hist}
        if args.net_out:
            np.save(args.net_out, net.parameters())
        del X, T, Xva, Tva, Xtr, Ttr
        torch.cuda.empty_cache()
    modes = [("fp64", "zero"), ("fp64", "previous"), ("mixed", "zero"), ("mixed", "previous"), ("mixed", "learned"),
             ("fp64", "learned")]
    evals = {}
    for N in [int(x) for x in args.eval_sizes.split(",")]:
        factor = args.eval_factor or max(1, N // 256)
        ell = args.eval_ell or 16.0 * N / 256
        res = {f"{p}/{g}": {"cycles": [], "ms": [], "alpha": [], "relres0": []} for p, g in modes}
        for si in range(args.eval_seeds):
            seed = 10000 + si
            drv = realisation(E, N, seed, "mixed", ell=ell, warm_start=1)
            ctxs = {}
            for p, g in modes:
                cx = realisation(E, N, seed, p, ell=ell, warm_start=0 if g == "zero" else 1)
                if g == "learned":
                    net.attach(cx, factor=factor, mode=1)
                ctxs[f"{p}/{g}"] = cx
            drv.run_steps(args.eval_skip)
            cd, pd = [device_view(x, (N, N)) for x in drv.state_ptrs()[:2]]
            for k in range(args.eval_samples + 1):
                drv.run_steps(args.eval_every)
                torch.cuda.synchronize()
                for name, cx in ctxs.items():
                    cc, pc = [device_view(x, (N, N)) for x in cx.state_ptrs()[:2]]
                    cc.copy_(cd)
                    pc.copy_(pd)
                    torch.cuda.synchronize()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    cx.pressure_solve_resident(sync=False)
                    e1.record()
                    e1.synchronize()
                    cyc, rr, rr0 = cx.last_solve()
                    assert rr <= 1e-10, (name, rr)
                    if k == 0:
                        continue  # the first solve captures the graph
                    res[name]["cycles"].append(cyc)
                    res[name]["relres0"].append(rr0)
                    res[name]["ms"].append(e0.elapsed_time(e1))
                    if name.endswith("learned"):
                        res[name]["alpha"].append(E.Net.last_alpha(cx))
            for name, cx in ctxs.items():
                if name.endswith("learned"):
                    E.Net.detach(cx)
                cx.close()
            drv.close()
        ev = {"net_grid": f"{N // factor}x{N // factor}", "feature_factor": factor, "seeds": args.eval_seeds,
              "solves_per_seed": args.eval_samples, "permeability_correlation_cells": ell}
        for name, r in res.items():
            ev[name] = {"cycles_mean": statistics.mean(r["cycles"]), "ms_per_solve_median": statistics.median(r["ms"]),
                        "ms_per_solve_mean": statistics.mean(r["ms"]),
                        "initial_relres_median": statistics.median(r["relres0"])}
            if r["alpha"]:
                ev[name]["alpha_median"] = statistics.median(r["alpha"])
        for p in ("fp64", "mixed"):
            L_, Pv, Z = ev[f"{p}/learned"], ev[f"{p}/previous"], ev[f"{p}/zero"]
            ev[f"{p}_learned_saves"] = {
                "cycles_vs_previous": Pv["cycles_mean"] - L_["cycles_mean"],
                "cycles_vs_zero": Z["cycles_mean"] - L_["cycles_mean"],
                "ms_vs_previous": Pv["ms_per_solve_median"] - L_["ms_per_solve_median"],
                "ms_vs_zero": Z["ms_per_solve_median"] - L_["ms_per_solve_median"]}
        ev["mixed_learned_vs_fp64_zero_speedup"] = (ev["fp64/zero"]["ms_per_solve_median"]
                                                    / ev["mixed/learned"]["ms_per_solve_median"])
        evals[f"{N}x{N}"] = ev
        log(json.dumps({f"{N}x{N}": ev}))
    out["evaluation"] = evals
    print(json.dumps(out))
    net.close()


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.study == "pressure":
        return study_pressure(args)
    if args.study == "warmstart":
        return study_warmstart(args)
    if args.study == "sweep":
        return study_sweep(args)
    if args.study == "ensemble":
        return study_ensemble(args)
    if args.study == "learned":
        return study_learned(args)
    if args.study == "network":
        return study_network(args)
    if args.no_graph:
        os.environ["IMPEC_NO_GRAPH"] = "1"  # read by the engine at each step
    import numpy as np
    import torch

    import impec2d_gb300 as E
    from impec2d_gb300 import build as B

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    B.build()
    N = args.n or N_DEFAULT
    P = workload_params(E, N, args.precision, args.nu)
    ctx = E.Context(P)
    c0, q = initial_state(N)
    g = 2
    cg = np.zeros((N + 2 * g, N + 2 * g))
    cg[g:g + N, g:g + N] = c0
    ctx.upload(cg, q, ghost=g)
    ctx.set_time(0.0)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    clocks = Clocks(local)
    clocks.start()
    for _ in range(args.warmup):
        ctx.run_steps(1)
    launches0 = E.launch_count(ctx)
    barrier()
    t_wall = time.perf_counter()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ctx.run_steps(1)
        e1.record()
        times.append((e0, e1))
    barrier()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in times]
    launches = E.launch_count(ctx) - launches0
    info = ctx.step()  # one more (untimed) step for the solver statistics
    from impec2d_gb300.replicas import max_over_ranks, whole_job_rate
    total_ms = max_over_ranks(sum(step_ms), device="cuda")
    ms = total_ms / args.steps
    value = whole_job_rate(N * N * args.steps, total_ms * 1e-3, world)

    # end to end through the host-buffer C ABI: pinned host c in, c and p out, every step
    e2e = None
    if not args.no_e2e:
        import ctypes as C
        hc = torch.empty((N + 2 * g) * (N + 2 * g), dtype=torch.float64).pin_memory().numpy()
        hp = torch.empty_like(torch.from_numpy(hc)).pin_memory().numpy()
        ctx.download(hc, None, None, ghost=g)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.upload(hc, None, ghost=g)
            ctx.run_steps(1)
            ctx.download(hc, hp, None, ghost=g)
        barrier()
        te = max_over_ranks(time.perf_counter() - t0, device="cuda")
        e2e = {"value": whole_job_rate(N * N * args.steps, te, world), "unit": "cell-steps/s",
               "h2d_bytes_per_step": N * N * 8, "d2h_bytes_per_step": 2 * N * N * 8}

    # a later window of the same run: the fingers have formed and the solves are harder
    later = None
    if args.later_after > 0:
        done = args.warmup + args.steps + 1
        if done < args.later_after:
            ctx.run_steps(args.later_after - done)
        barrier()
        lt = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            ctx.run_steps(1)
            e1.record()
            lt.append((e0, e1))
        barrier()
        lms = max_over_ranks(sum(a.elapsed_time(b) for a, b in lt), device="cuda") / args.steps
        linfo = ctx.step()
        later = {"after_step": max(done, args.later_after), "t": linfo.t, "steps": args.steps, "ms_per_step": lms,
                 "value": whole_job_rate(N * N * args.steps, lms * args.steps * 1e-3, world),
                 "mg_cycles": linfo.its, "cn_sweeps": linfo.para_its}

    pressure = pressure_solves(E, ctx, N, q, args, flush)

    roof_small = E.roofline_probe(ctx, P, args.precision, flush=flush)
    # The dominant kernel's HBM roofline: the fine-level FP64 sweep where its data cannot stay
    # in L2, at 4096^2 (the mixed-precision case's grid).  Inside the 1024^2 step the same sweep runs from
    # L2 (the whole hierarchy, ~150 MB, is about L2's size); its cold figure is kept beside it.
    roof_large = None
    if not args.no_large_roofline and args.nu == 1.0:
        NL = 4096
        PL = workload_params(E, NL, args.precision, args.nu)
        cl = E.Context(PL)
        cL, qL = initial_state(NL)
        cgL = np.zeros((NL + 2 * g, NL + 2 * g))
        cgL[g:g + NL, g:g + NL] = cL
        cl.upload(cgL, qL, ghost=g)
        cl.pressure_solve_resident()  # builds the operator hierarchy of this state
        roof_large = E.roofline_probe(cl, PL, args.precision, flush=flush)
        cl.close()
        del cgL
    sched = f"V({ctx.get_tuning('mg_pre')},{ctx.get_tuning('mg_post')})"
    line = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(N, args.precision, args.nu),
            "solver": {"schedule": f"{sched}-preconditioned CG", "mg_cycles": info.its, "relres": info.relres,
                       "cn_sweeps": info.para_its, "dt": info.dt, "wall_s": t_wall, "replicas": world},
            "pressure_solve_1e-10": pressure, "gpu_launches": int(launches), "clocks": clk,
            "roofline": roof_large or roof_small}
    if roof_large:
        roof_large["why_this_grid"] = ("HBM bounds this sweep only where its level does not fit L2; inside the "
                                       f"{N}^2 step the level is L2-resident (roofline_{N} holds its cold figure)")
        line[f"roofline_{N}"] = roof_small
    if e2e:
        line["e2e"] = e2e
    if later:
        line["later_window"] = later
    if rank == 0 and not args.no_cpu_baseline:
        cps, cores, secs, _ = cpu_baseline(N, 3)
        line["cpu_baseline"] = {"value": cps, "unit": "cell-steps/s", "cores": cores, "kind": "port",
                                "sample": f"3 IMPES steps at {N}^2 from t=0, oracle FP64 C++ with OpenMP ({secs:.1f} s)"}
        cps1, _, secs1, done1 = cpu_baseline(N, 1, threads=1)
        line["cpu_baseline"]["one_thread"] = {"value": cps1, "unit": "cell-steps/s", "cores": 1,
                                              "sample": f"{done1} IMPES step at {N}^2 from t=0 ({secs1:.1f} s)"}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
