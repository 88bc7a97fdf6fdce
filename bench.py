#!/usr/bin/env python
"""Throughput benchmark: IMPES cell-steps/s on the 1024 x 1024 parallel quarter-five-spot.

Workload (one "step" = one IMPES step: pressure solve, Darcy velocities, CFL dt, TR source,
Crank-Nicolson Peaceman dispersion, symmetric-parallel MUSCL transport, TR source, CN):
  1024^2 cells on [0, sqrt 2]^2, four corner one-cell wells (two injectors, two producers),
  M = 41 quarter-power mobility, harmonic averaging, nu = 1 (5-point), porosity 1, CFL 0.5,
  MUSCL/van Leer, alpha_l = 1e-3, alpha_t = 1e-4 (cell units), molecular diffusion 1e-6,
  multigrid V(2,2) to relative residual 1e-10 (FP64 unless --precision mixed),
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
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch each kernel on the stream instead of replaying the step graph (for ncu)")
    ap.add_argument("--study", default=None, choices=["pressure", "warmstart", "ensemble"],
                    help="pressure: FP64 vs mixed-precision solves on re-seeded heterogeneous fields; "
                         "warmstart: V-cycles and ms per solve along the IMPES run for zero and previous-step "
                         "initial guesses")
    ap.add_argument("--solves", type=int, default=20, help="re-seeded solves of the pressure study")
    ap.add_argument("--members-per-size", type=int, default=64,
                    help="ensemble study: realisations at each of 128^2, 256^2, 384^2, 512^2")
    ap.add_argument("--no-autotune", action="store_true", help="ensemble study: keep the default schedules")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


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


def workload_params(E, N, precision):
    L = math.sqrt(2.0)
    return E.default_params(N, N, x_ub=L, y_ub=L, stype=E.PARALLEL, hmtype=E.MUSCL, nu=1.0, diffusion=1,
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


def cpu_baseline(N, steps, threads=None):
    """Oracle (FP64 C++ restatement, OpenMP) on the host cores: cell-steps/s of `steps` steps."""
    import ctypes as C

    import numpy as np

    import oracle as O
    O.build()
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    L = O.lib()
    P = O.make_params(N1=N, N2=N, x_ub=math.sqrt(2.0), y_ub=math.sqrt(2.0), stype=O.PARALLEL, hmtype=O.MUSCL, nu=1.0,
                      diffusion=1, alpha_l=1e-3, alpha_t=1e-4, Dm=1e-6, cfl=0.5, eps=1e-10, para_eps=1e-10)
    c0, q = initial_state(N)
    c = O.with_ghosts(P, c0)
    p, v = np.zeros(O.scalar_shape(P)), np.zeros(O.vel_shape(P))
    S = O.State()
    S.prev_first_sweep = 1
    tidx = C.c_int(0)
    t0 = time.perf_counter()
    for _ in range(steps):
        L.or_impes_step(C.byref(P), C.byref(S), O.ptr(c), O.ptr(p), O.ptr(v), O.ptr(q), None, 0, C.byref(tidx), 1,
                        1e-10)
    dt = time.perf_counter() - t0
    return N * N * steps / dt, L.or_num_threads(), dt


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    n = args.n or N_DEFAULT
    cps, cores, secs = cpu_baseline(n, max(1, args.steps // 4) + 1)
    line = {"impl": "reference", "metric": METRIC, "value": cps, "unit": "cell-steps/s", "n_gpus": args.gpus,
            "steps": max(1, args.steps // 4) + 1, "warmup": 0, "ms_per_step": 1e3 / cps * n * n,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"parallel quarter-five-spot {n}x{n}, MUSCL + CN Peaceman, FP64 MG 1e-10"},
            "cpu_baseline": {"value": cps, "unit": "cell-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{max(1, args.steps // 4) + 1} IMPES steps at {n}^2 from t=0 ({secs:.1f} s)"},
            "e2e": {"value": cps, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def grf(N, ell, seed):
    """Seeded Gaussian random field on the GPU: white noise (Philox, seeded) filtered in Fourier
    space to the covariance exp(-r^2 / ell^2) (ell in cells, periodic), zero mean, unit variance."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    w = torch.randn((N, N), generator=g, device="cuda", dtype=torch.float64)
    f = torch.fft.fftfreq(N, device="cuda", dtype=torch.float64)
    H = torch.exp(-(math.pi * ell) ** 2 * (f[:, None] ** 2 + f[None, :] ** 2) / 2)
    x = torch.fft.ifft2(torch.fft.fft2(w) * H).real
    return ((x - x.mean()) / x.std()).contiguous()


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
        P = workload_params(E, N, args.precision)
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
    """One realisation of the batched-ensemble workload: lognormal K (sigma 0.5, correlation
    16 cells), M from {5, 20, 41, 100} and diagonal or parallel orientation chosen by the seed,
    MUSCL + Peaceman dispersion (alpha_l 1e-3, alpha_t 1e-4), FP64 transport and
    mixed-precision pressure."""
    import numpy as np
    import torch
    M = (5.0, 20.0, 41.0, 100.0)[seed % 4]
    parallel = (seed // 4) % 2 == 1
    L = math.sqrt(2.0) if parallel else 1.0
    P = E.default_params(N, N, x_ub=L, y_ub=L, stype=E.PARALLEL if parallel else E.DIAGONAL, hmtype=E.MUSCL,
                         nu=1.0, diffusion=1, alpha_l=1e-3, alpha_t=1e-4, cfl=0.5, porosity=1.0, eps=1e-10,
                         para_eps=1e-10, mu_res=M, mu_inj=1.0, max_cycles=200,
                         precision=E.PREC_MIXED if precision == "mixed" else E.PREC_FP64)
    ctx = E.Context(P)
    dx = L / N
    qv = 1.0 / (dx * dx)
    q = np.zeros(N * N)
    q[0] = qv
    if parallel:
        q[-1], q[N - 1], q[(N - 1) * N] = qv, -qv, -qv
    else:
        q[-1] = -qv
    K = torch.exp(0.5 * grf(N, 16.0, 5000 + seed)).contiguous()
    ctx.upload(np.zeros((N + 4, N + 4)), q, ghost=2)
    ctx.set_permeability(K, K)
    ctx.set_time(0.0)
    return ctx


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
    members = []
    for N in sizes:
        for i in range(k):
            ctx = ensemble_member(E, N, i)
            for name, v in tuned.get(N, {}).items():
                if name != "report":
                    ctx.set_tuning(name, v)
            members.append((N, ctx))
    cells = sum(N * N for N, _ in members)
    t0 = time.perf_counter()
    ens = E.Ensemble([c for _, c in members])
    t_capture = time.perf_counter() - t0
    ens.step(args.warmup)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ens.step(args.steps)
    t_ens = time.perf_counter() - t0
    # the same members one after another (each its own graph launch per step)
    for _, c in members:
        c.run_steps(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for _, c in members:
            c.run_steps(1)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    out = {"study": "ensemble",
           "workload": f"{len(members)} realisations, {k} each at 128^2, 256^2, 384^2, 512^2; lognormal K "
                       f"(sigma 0.5), M in {{5,20,41,100}}, diagonal/parallel by seed; MUSCL + Peaceman; "
                       f"mixed-precision pressure",
           "cells": cells, "steps": args.steps, "warmup": args.warmup,
           "ensemble": {"cell_steps_per_s": cells * args.steps / t_ens, "ms_per_step": 1e3 * t_ens / args.steps,
                        "capture_s": t_capture},
           "one_after_another": {"cell_steps_per_s": cells * args.steps / t_seq, "ms_per_step": 1e3 * t_seq / args.steps},
           "speedup": t_seq / t_ens, "autotune": tuned or None, "data": "synthetic (seeded GRF permeability)"}
    print(json.dumps(out))
    ens.close()
    for _, c in members:
        c.close()


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.study == "pressure":
        return study_pressure(args)
    if args.study == "warmstart":
        return study_warmstart(args)
    if args.study == "ensemble":
        return study_ensemble(args)
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
    P = workload_params(E, N, args.precision)
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
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms = total_ms / args.steps
    value = N * N * args.steps * world / (total_ms * 1e-3)

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
        te = time.perf_counter() - t0
        e2e = {"value": N * N * args.steps * world / te, "unit": "cell-steps/s", "h2d_bytes_per_step": N * N * 8,
               "d2h_bytes_per_step": 2 * N * N * 8}

    # ms per pressure solve to 1e-10 on the current state: plain FP64 MG vs mixed precision
    pressure = {}
    hc = np.zeros((N + 2 * g, N + 2 * g))
    ctx.download(hc, None, None, ghost=g)
    for prec in ("fp64", "mixed"):
        Pp = workload_params(E, N, prec)
        cp = E.Context(Pp)
        cp.upload(hc, q, ghost=g)
        cyc, rr = cp.pressure_solve_resident()  # capture + warm-up
        ts = []
        for _ in range(5):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            cp.pressure_solve_resident(sync=False)
            e1.record()
            ts.append((e0, e1))
        torch.cuda.synchronize()
        cyc, rr = cp.pressure_solve_resident()
        pressure[prec] = {"ms_per_solve": statistics.median(a.elapsed_time(b) for a, b in ts), "cycles": cyc,
                          "relres": rr}
        cp.close()

    roof = E.roofline_probe(ctx, P, args.precision)
    line = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"parallel quarter-five-spot {N}x{N}, MUSCL + CN Peaceman (alpha_l 1e-3, alpha_t 1e-4,"
                                   f" Dm 1e-6), MG V(2,2) to 1e-10",
                       "precision": args.precision, "l2": "flushed (256 MB write) between timed steps",
                       "parallelism": f"replicas x{world}"},
            "solver": {"mg_cycles": info.its, "relres": info.relres, "cn_sweeps": info.para_its, "dt": info.dt,
                       "wall_s": t_wall},
            "pressure_solve_1e-10": pressure, "gpu_launches": int(launches), "clocks": clk, "roofline": roof}
    if e2e:
        line["e2e"] = e2e
    if rank == 0 and not args.no_cpu_baseline:
        cps, cores, secs = cpu_baseline(N, 3)
        line["cpu_baseline"] = {"value": cps, "unit": "cell-steps/s", "cores": cores, "kind": "port",
                                "sample": f"3 IMPES steps at {N}^2 from t=0, oracle FP64 C++ with OpenMP ({secs:.1f} s)"}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
