"""Writes the golden fixtures of the reference Impec2D, produced by the reference itself.

Run where a reference checkout is at hand (IMPEC2D_REFERENCE names it, or the default of
oracle/Makefile.ref):  python tests/golden/make_ref_golden.py
It builds oracle/_ref (the reference's own src/*.cpp compiled unchanged against the stand-ins
in oracle/refshim) and records, on seeded inputs:

  ref_ops.npz       per-operation inputs and outputs of three small cases (diagonal MUSCL with
                    circle wells and Crank-Nicolson dispersion; parallel, nu = 2/3, mean
                    concentration; horizontal front with pulsing injection): the assembled
                    pressure and CN systems, face mobilities, the direct pressure solve, Darcy
                    velocities, the CFL step, TR source, MUSCL and upwind fluxes, the split
                    advection and the whole HyperbolicSplitSolver::Solve, sources, diagnostics;
  ref_runs/<case>/  whole runs of Impec2DSolver::Solve on a .cfg (results_dir "."), with every
                    file the reference wrote: diagnostics.dat, concentration.dat, pressure.dat
                    and, on diagonal grids, velocity_u.dat / velocity_v.dat;
  ref_advection.npz log(dx), log(L1 error) of the reference's advection convergence case, and
  muscl_sine_convergence.cfg, the same case as a .cfg (its output directory is the token @DIR@).

The reference's pressure and CN systems are solved directly here (its HYPRE is absent), so
solve outputs carry the rounding of a direct solve rather than HYPRE's stopping tolerance.
"""
import ctypes as C
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from oracle import ref as R  # noqa: E402


def fields(P, seed):
    rng = np.random.default_rng(seed)
    c = np.zeros(O.scalar_shape(P))
    c[P.g:P.g + P.N1, P.g:P.g + P.N2] = rng.uniform(0.0, 1.0, (P.N1, P.N2))
    O.lib().or_fill_scalar_neumann(C.byref(P), O.ptr(c))
    v = rng.uniform(-1.0, 1.0, O.vel_shape(P))
    v[np.abs(v) < 1e-3] = 1e-3
    O.lib().or_fill_velocity_neumann(C.byref(P), O.ptr(v))
    return c, v


OPS_CASES = {
    "diag": dict(N1=24, N2=20, stype=O.DIAGONAL, hmtype=O.MUSCL, porosity=0.7, nu=1.0, avgproc=O.HARMONIC,
                 well_profile=O.CIRCULAR, well_rc=0.2, diffusion=1, alpha_l=0.3, alpha_t=0.03),
    "par": dict(N1=22, N2=22, x_ub=1.4142135623730951, y_ub=1.4142135623730951, stype=O.PARALLEL,
                hmtype=O.MUSCL, porosity=1.0, nu=2.0 / 3.0, avgproc=O.MEANCONC, well_profile=O.ONECELL,
                diffusion=1, alpha_l=0.2, alpha_t=0.02),
    "horiz": dict(N1=24, N2=20, stype=O.HORIZONTAL, hmtype=O.MUSCL, porosity=0.5, nu=1.0, inj_mode=0,
                  q_freq=20.0, q_high_multiple=50.0, well_width=0.1, diffusion=1, alpha_l=0.2, alpha_t=0.02),
}

RUN_CASES = {
    # the reference's loop always advects with MUSCL (src/Impec2DSolver.cpp:132)
    "diag32_muscl": dict(N1=32, N2=32, stype=O.DIAGONAL, hmtype=O.MUSCL, porosity=1.0, nu=1.0,
                         well_profile=O.ONECELL, tfinal=0.05, eps=1e-12),
    "par32_muscl_cn": dict(N1=32, N2=32, x_ub=1.4142135623730951, y_ub=1.4142135623730951, stype=O.PARALLEL,
                           hmtype=O.MUSCL, porosity=1.0, nu=1.0, well_profile=O.ONECELL, diffusion=1,
                           alpha_l=0.05, alpha_t=0.005, tfinal=0.03, eps=1e-12, para_eps=1e-12),
    "diag30_circle_nu23": dict(N1=30, N2=30, stype=O.DIAGONAL, hmtype=O.MUSCL, porosity=1.0, nu=2.0 / 3.0,
                               well_profile=O.CIRCULAR, well_rc=0.1, tfinal=0.04, eps=1e-12),
}


def ops(out):
    for name, kw in OPS_CASES.items():
        P = O.make_params(**kw)
        c, v = fields(P, {"diag": 11, "par": 12, "horiz": 13}[name])
        n = P.N1 * P.N2
        rec = {"c": c, "v": v}
        with R.Case(P) as h:
            q = h.source()
            if P.stype == O.HORIZONTAL:
                h.horizontal_source(q, 0.013)
                rec["q_t"] = np.array(0.013)
            rec["q"] = q
            A = np.zeros(n * 9)
            h.pressure_matrix(c, A)
            rec["A9"] = A
            b = np.zeros(n)
            h.pressure_rhs(q, b)
            rec["b"] = b
            lx, ly = np.zeros((P.N1 + 1) * P.N2), np.zeros(P.N1 * (P.N2 + 1))
            h.face_mobility(c, lx, ly)
            rec["lamx"], rec["lamy"] = lx, ly
            p = np.zeros(O.scalar_shape(P))
            assert h.pressure_solve(c.copy(), q, p) == 0
            rec["p"] = p
            vp = np.zeros(O.vel_shape(P))
            h.calc_velocities(p.copy(), vp, c)
            rec["v_of_p"] = vp
            rec["dt"] = np.array(h.max_stable_dt(c, vp))
            dt = 0.5 * float(rec["dt"])
            rec["dt_used"] = np.array(dt)
            ct = c.copy()
            rec["tr_outflux"] = np.array(h.tr_integrate(ct, q, dt))
            rec["tr_c"] = ct
            g = P.g
            for scheme, tag in ((O.MUSCL, "muscl"), (O.UPWINDSPLIT, "upwind")):
                F, G = np.zeros((P.N1 + 1) * (P.N2 + 2 * g)), np.zeros((P.N1 + 2 * g) * (P.N2 + 1))
                h.flux_F(scheme, F, c, v, dt)
                h.flux_G(scheme, G, c, v, dt)
                rec[f"F_{tag}"], rec[f"G_{tag}"] = F, G
                ca = c.copy()
                s = C.c_int(1)
                h.advect_split(scheme, ca, vp, dt, C.byref(s))
                rec[f"advect_{tag}"] = ca
            An = np.zeros(n * 9)
            h.cn_matrix(vp, 0.5 * dt, An)
            rec["cn_A9"] = An
            bn = np.zeros(n)
            h.cn_rhs(c, vp, 0.5 * dt, bn)
            rec["cn_b"] = bn
            cc = c.copy()
            assert h.cn_solve(cc, vp, 0.5 * dt) == 0
            rec["cn_c"] = cc
            ch = c.copy()
            s, o = C.c_int(1), C.c_double(0.0)
            assert h.hyperbolic_solve(O.MUSCL, ch, vp, q, dt, C.byref(s), C.byref(o)) == 0
            rec["hyp_c"], rec["hyp_outflux"] = ch, np.array(o.value)
            rec["total_mass"] = np.array(h.total_mass(c))
            rec["mass_error"] = np.array(h.mass_error(c, 0.37, 0.11))
            rec["div_error"] = np.array(h.divergence_error(vp))
            rec["vel_error"] = np.array(h.velocity_boundary_error(vp))
        for k, a in rec.items():
            out[f"{name}/{k}"] = np.asarray(a)
        out[f"{name}/params"] = np.array(repr(kw))


def runs(dest):
    if os.path.isdir(dest):
        shutil.rmtree(dest)
    os.makedirs(dest)
    for name, kw in RUN_CASES.items():
        P = O.make_params(**kw)
        d = tempfile.mkdtemp(prefix="impec_ref_run_")
        cfg = R.write_cfg(os.path.join(d, "case.cfg"), P, results_dir=d)
        h = R.lib().ref_open(cfg.encode())
        steps = C.c_int(0)
        assert R.lib().ref_run(h, None, None, None, None, C.byref(steps)) == 0
        R.lib().ref_close(h)
        cd = os.path.join(dest, name)
        os.makedirs(cd)
        with open(cfg) as f:
            text = f.read().replace(d, ".")
        with open(os.path.join(cd, "case.cfg"), "w") as f:
            f.write(text)
        for fn in sorted(os.listdir(d)):
            if fn.endswith(".dat"):
                shutil.copy(os.path.join(d, fn), os.path.join(cd, fn))
        shutil.rmtree(d)


def advection(path, cfg_out):
    d = tempfile.mkdtemp(prefix="impec_ref_adv_")
    P = O.make_params(N1=50, N2=50, stype=O.DIAGONAL, hmtype=O.MUSCL, porosity=1.0, cfl=0.95, is_test=1,
                      tstart=0.0, tfinal=1.0, dim_splitting=O.SYMMETRIC_PARALLEL)
    cfg = R.write_cfg(os.path.join(d, "t.cfg"), P, results_dir=d, test=dict(levels=4))
    # the same case as a .cfg for the engine's TestComponent, output directory left as @DIR@
    R.write_cfg(cfg_out, P, results_dir="@DIR@", test=dict(levels=4, norm_file="@DIR@/norm.out"))
    lx, ln = np.zeros(4), np.zeros(4)
    assert R.lib().ref_advection_test(cfg.encode(), -1.0, 1.0, O.ptr(lx), O.ptr(ln)) == 0
    np.savez(path, logdx=lx, lognorm=ln, cells=np.array([50, 100, 200, 400]))
    shutil.rmtree(d)


def main():
    O.build()
    if R.build() is None:
        raise SystemExit("no reference checkout: set IMPEC2D_REFERENCE")
    out = {}
    ops(out)
    np.savez_compressed(os.path.join(HERE, "ref_ops.npz"), **out)
    runs(os.path.join(HERE, "ref_runs"))
    advection(os.path.join(HERE, "ref_advection.npz"), os.path.join(HERE, "muscl_sine_convergence.cfg"))
    print("wrote", os.path.join(HERE, "ref_ops.npz"), os.path.join(HERE, "ref_runs"),
          os.path.join(HERE, "ref_advection.npz"))


if __name__ == "__main__":
    main()
