"""The CUDA engine against outputs written by the reference itself.

The fixtures under tests/golden (ref_ops.npz, ref_runs/, ref_advection.npz) were produced by
the reference's own code -- src/*.cpp of pw359/Impec2D compiled unchanged in oracle/_ref -- by
tests/golden/make_ref_golden.py.  Nothing here needs the reference checkout, so these tests run
where the GPU is.

Tolerances, relative to the field's largest magnitude unless stated:
  * face mobilities: bit for bit;
  * single operators (operator apply, velocities, the CFL step, TR, one sweep, the split
    advection): 1e-13;
  * pressure solve to 1e-12: relative residual under the reference's own assembled matrix
    <= 2e-12, and within 1e-9 of the reference's direct solution;
  * Crank-Nicolson solve and the whole HyperbolicSplitSolver::Solve: 1e-12;
  * whole .cfg runs through the engine's drop-in Impec2DSolver: every file the reference wrote
    is written, with the same lines and columns; values agree to the 6 significant digits both
    print (relative 2e-5, absolute 1e-9 for the round-off-sized error columns);
  * the advection convergence case: each level's L1 error within 1e-9 relative.
"""
import ast
import ctypes as C
import os
import shutil

import numpy as np
import pytest

import oracle as O
from helpers import dev, host, vel_split

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
ENGINE_KEYS = {"N1", "N2", "x_lb", "x_ub", "y_lb", "y_ub", "mu_res", "mu_inj", "avgproc", "nu", "porosity", "cfl",
               "diffusion", "alpha_l", "alpha_t", "stype", "hmtype", "dim_splitting", "eps", "para_eps", "is_test"}


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLD, "ref_ops.npz"))


def _case(E, gold, name, **over):
    kw = ast.literal_eval(str(gold[f"{name}/params"]))
    OP = O.make_params(**kw)
    ekw = {k: v for k, v in kw.items() if k in ENGINE_KEYS and k not in ("N1", "N2")}
    ekw.update(over)
    P = E.default_params(OP.N1, OP.N2, **ekw)
    g = lambda k: gold[f"{name}/{k}"]  # noqa: E731
    return P, OP, g


def _interior(OP, a):
    return np.ascontiguousarray(O.interior(OP, a))


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


CASES = ["diag", "par", "horiz"]


@pytest.mark.parametrize("name", CASES)
def test_assembly_and_velocities(engine, gold, name):
    import torch
    E = engine
    P, OP, g = _case(E, gold, name)
    ctx = E.Context(P)
    c = dev(_interior(OP, g("c")))
    N1, N2 = P.N1, P.N2
    lx = torch.zeros((N1 + 1) * N2, dtype=torch.float64, device="cuda")
    ly = torch.zeros(N1 * (N2 + 1), dtype=torch.float64, device="cuda")
    ctx.face_mobility(c, lx, ly)
    assert np.array_equal(host(lx), g("lamx")) and np.array_equal(host(ly), g("lamy"))
    # the operator against the reference's assembled matrix (Dirichlet rows as assembled)
    x = np.random.default_rng(5).normal(size=(N1, N2))
    A = g("A9").reshape(N1 * N2, 9)
    y = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
    ctx.pressure_apply(c, dev(x), y)
    xr = x.ravel()
    offs = [(0, 0), (-1, 0), (-1, -1), (0, -1), (1, -1), (1, 0), (1, 1), (0, 1), (-1, 1)]
    yr = np.zeros(N1 * N2)
    for i in range(N1):
        for j in range(N2):
            s = 0.0
            for e, (di, dj) in enumerate(offs):
                ii, jj = i + di, j + dj
                if 0 <= ii < N1 and 0 <= jj < N2:
                    s += A[i * N2 + j, e] * xr[ii * N2 + jj]
            yr[i * N2 + j] = s
    assert np.abs(host(y).ravel() - yr).max() <= 1e-13 * np.abs(A).sum(1).max() * np.abs(x).max()
    # Darcy velocities of the reference's pressure
    p = dev(_interior(OP, g("p")))
    u = torch.zeros((N1 + 1, N2), dtype=torch.float64, device="cuda")
    v = torch.zeros((N1, N2 + 1), dtype=torch.float64, device="cuda")
    ctx.velocity(p, c, u, v)
    ur, vr = vel_split(OP, g("v_of_p"))
    assert _rel(host(u), ur) <= 1e-13 and _rel(host(v), vr) <= 1e-13
    assert abs(ctx.max_stable_dt(dev(ur), dev(vr)) - float(g("dt"))) <= 1e-14 * float(g("dt"))
    ctx.close()


@pytest.mark.parametrize("name", CASES)
def test_pressure_solve_against_reference_system(engine, gold, name):
    import torch
    E = engine
    P, OP, g = _case(E, gold, name, max_cycles=300)
    ctx = E.Context(P)
    ctx.set_source(dev(g("q")))
    c = dev(_interior(OP, g("c")))
    p = torch.zeros((P.N1, P.N2), dtype=torch.float64, device="cuda")
    cyc, rr, _ = ctx.pressure_solve(c, p, 1e-12)
    assert rr <= 1e-12
    ph = host(p).ravel()
    A, b = g("A9"), g("b")
    rr_ref = O.lib().or_relres9(C.byref(OP), O.ptr(A), O.ptr(ph.copy()), O.ptr(b))
    assert rr_ref <= 2e-12, rr_ref
    assert _rel(host(p), _interior(OP, g("p"))) <= 1e-9
    ctx.close()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("scheme", ["muscl", "upwind"])
def test_transport_against_reference(engine, gold, name, scheme):
    import torch
    E = engine
    hm = E.MUSCL if scheme == "muscl" else E.UPWINDSPLIT
    P, OP, g = _case(E, gold, name, hmtype=hm, dim_splitting=E.SYMMETRIC_PARALLEL)
    ctx = E.Context(P)
    ctx.set_source(dev(g("q")))
    c0 = _interior(OP, g("c"))
    dt = float(g("dt_used"))
    # one x sweep and one y sweep from the reference's intercell fluxes (random velocities)
    uq, vq = vel_split(OP, g("v"))
    gg = OP.g
    F = g(f"F_{scheme}").reshape(P.N1 + 1, P.N2 + 2 * gg)[:, gg:gg + P.N2]
    G = g(f"G_{scheme}").reshape(P.N1 + 2 * gg, P.N2 + 1)[gg:gg + P.N1, :]
    dx, dy = (P.x_ub - P.x_lb) / P.N1, (P.y_ub - P.y_lb) / P.N2
    cx = dev(c0)
    ctx.advect_x(cx, dev(uq), dt)
    assert _rel(host(cx), c0 + dt / dx * (F[:-1] - F[1:])) <= 1e-13
    cy = dev(c0)
    ctx.advect_y(cy, dev(vq), dt)
    assert _rel(host(cy), c0 + dt / dy * (G[:, :-1] - G[:, 1:])) <= 1e-13
    # the symmetric-parallel split with the velocities of the reference's pressure
    ur, vr = vel_split(OP, g("v_of_p"))
    cs = dev(c0)
    ctx.advect_split(cs, dev(ur), dev(vr), dt, 1)
    assert _rel(host(cs), _interior(OP, g(f"advect_{scheme}"))) <= 1e-13
    if scheme == "muscl":
        ct = dev(c0)
        tmo = ctx.tr_integrate(ct, dt)
        assert _rel(host(ct), _interior(OP, g("tr_c"))) <= 1e-13
        assert abs(tmo - float(g("tr_outflux"))) <= 1e-13 * abs(float(g("tr_outflux")))
    ctx.close()


@pytest.mark.parametrize("name", CASES)
def test_dispersion_and_split_solve_against_reference(engine, gold, name):
    E = engine
    P, OP, g = _case(E, gold, name, para_eps=1e-13, dim_splitting=E.SYMMETRIC_PARALLEL)
    ctx = E.Context(P)
    ctx.set_source(dev(g("q")))
    c0 = _interior(OP, g("c"))
    dt = float(g("dt_used"))
    ur, vr = vel_split(OP, g("v_of_p"))
    cc = dev(c0)
    its, rr = ctx.dispersion_cn(cc, dev(ur), dev(vr), 0.5 * dt, 1e-13)
    assert _rel(host(cc), _interior(OP, g("cn_c"))) <= 1e-12, (its, rr)
    ch = dev(c0)
    _, outflux = ctx.hyperbolic_solve(ch, dev(ur), dev(vr), dt, 1, 0.0)
    assert _rel(host(ch), _interior(OP, g("hyp_c"))) <= 1e-12
    assert abs(outflux - float(g("hyp_outflux"))) <= 1e-12 * abs(float(g("hyp_outflux")))
    ctx.close()


@pytest.mark.parametrize("name", ["diag", "par"])
def test_diagnostics_against_reference(engine, gold, name):
    E = engine
    P, OP, g = _case(E, gold, name)
    ctx = E.Context(P)
    ctx.set_source(dev(g("q")))
    ur, vr = vel_split(OP, g("v_of_p"))
    mass, div_err, vel_err, cmax, cmin = ctx.diagnostics(dev(_interior(OP, g("c"))), dev(ur), dev(vr))
    assert abs(mass - float(g("total_mass"))) <= 1e-13 * float(g("total_mass"))
    assert abs(div_err - float(g("div_error"))) <= 1e-11
    assert abs(vel_err - float(g("vel_error"))) <= 1e-11
    ctx.close()


def _read_columns(path):
    rows = []
    with open(path) as f:
        for line in f:
            rows.append(line.split())
    return rows


@pytest.mark.parametrize("case", sorted(os.listdir(os.path.join(GOLD, "ref_runs"))))
def test_whole_cfg_run_writes_the_reference_files(engine, tmp_path, case):
    """Impec2DSolver(cfg).Run() through the engine (impec_run_cfg) on the same .cfg the reference
    ran: the same output files (diagnostics.dat, the x y value dumps), line for line."""
    E = engine
    src = os.path.join(GOLD, "ref_runs", case)
    cfg = tmp_path / "case.cfg"
    cfg.write_text(open(os.path.join(src, "case.cfg")).read().replace('"."', f'"{tmp_path}"'))
    assert E.lib().impec_run_cfg(str(cfg).encode(), 1) == 0, E.last_error()
    ref_files = sorted(f for f in os.listdir(src) if f.endswith(".dat"))
    got_files = sorted(f for f in os.listdir(tmp_path) if f.endswith(".dat"))
    assert got_files == ref_files
    for fn in ref_files:
        ref, got = _read_columns(os.path.join(src, fn)), _read_columns(tmp_path / fn)
        assert len(ref) == len(got), fn
        for k, (a, b) in enumerate(zip(ref, got)):
            assert len(a) == len(b), (fn, k, a, b)
            if fn == "diagnostics.dat":
                assert a[0] == b[0]  # step counter
                cols = [2, 3, 4]  # t, dt, cells per dt; column 1 is the solver's iteration count
                for m in cols:
                    assert abs(float(a[m]) - float(b[m])) <= 2e-5 * abs(float(a[m])), (fn, k, m, a, b)
                for m in range(5, len(a)):  # mass, no-flow and divergence errors: round-off sized
                    assert abs(float(a[m]) - float(b[m])) <= 1e-9, (fn, k, m, a, b)
            else:
                if not a:
                    continue
                assert a[:2] == b[:2], (fn, k, a, b)  # the x y columns print identically
                va, vb = float(a[2]), float(b[2])
                assert abs(va - vb) <= 2e-5 * abs(va) + 1e-9, (fn, k, a, b)


def test_advection_convergence_case_against_reference(engine, tmp_path):
    """The reference's advection convergence case (examples/hyperbolic_test.cfg settings: MUSCL,
    sine profile, L1, CFL 0.95, periodic, 50^2 doubled over 4 levels) through the engine's
    TestComponent: each level's error within 1e-9 of the reference's, order 1.86712."""
    E = engine
    gold = np.load(os.path.join(GOLD, "ref_advection.npz"))
    cfg = tmp_path / "adv.cfg"
    text = open(os.path.join(GOLD, "muscl_sine_convergence.cfg")).read().replace("@DIR@", str(tmp_path))
    cfg.write_text(text)
    assert E.lib().impec_run_cfg(str(cfg).encode(), 1) == 0, E.last_error()
    rows = np.loadtxt(tmp_path / "norm.out")
    assert rows.shape == (4, 2)
    assert np.abs(rows[:, 0] - gold["logdx"]).max() <= 1e-12
    assert np.abs(np.exp(rows[:, 1]) / np.exp(gold["lognorm"]) - 1).max() <= 1e-9
    order = np.polyfit(rows[:, 0], rows[:, 1], 1)[0]
    assert abs(order - 1.86712) < 5e-5, order
    shutil.rmtree(tmp_path, ignore_errors=True)
