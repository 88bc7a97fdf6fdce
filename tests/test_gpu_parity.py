"""Per-operation parity of the CUDA engine (through the C ABI) against the CPU oracle.

Tolerances (relative to the field's max magnitude): 1e-13 for single operators
(mobility, operator apply, velocity, one transport sweep, TR); for linear solves the
relative residual under the oracle's own matrix must reach the requested tolerance and
the solution must agree with the oracle's banded-LU solve to within a condition-number
allowance stated per test.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from helpers import cell_ghost, dev, host, oparams, rel_err, smooth_field, source, vel_ghost, vel_split

pytestmark = pytest.mark.gpu

GRIDS = [(32, 32), (37, 29), (48, 64)]


def _ctx(E, N1, N2, **kw):
    P = E.default_params(N1, N2, **kw)
    return P, E.Context(P)


def _rand_c(N1, N2, seed):
    return smooth_field(N1, N2, seed)


@pytest.mark.parametrize("N1,N2", GRIDS)
@pytest.mark.parametrize("avg", [1, 0])
def test_face_mobility_bitexact(engine, oracle_lib, N1, N2, avg):
    E = engine
    P, ctx = _ctx(E, N1, N2, avgproc=avg)
    OP = oparams(P)
    c = _rand_c(N1, N2, 1)
    lx, ly = np.zeros((N1 + 1) * N2), np.zeros(N1 * (N2 + 1))
    oracle_lib.or_face_mobility(C.byref(OP), O.ptr(cell_ghost(OP, c)), O.ptr(lx), O.ptr(ly))
    import torch
    dlx = torch.zeros((N1 + 1) * N2, dtype=torch.float64, device="cuda")
    dly = torch.zeros(N1 * (N2 + 1), dtype=torch.float64, device="cuda")
    ctx.face_mobility(dev(c), dlx, dly)
    # same operations in the same order: bit-identical
    assert np.array_equal(host(dlx), lx)
    assert np.array_equal(host(dly), ly)


@pytest.mark.parametrize("N1,N2", GRIDS)
@pytest.mark.parametrize("nu", [1.0, 2.0 / 3.0])
@pytest.mark.parametrize("stype", [1, 0])
def test_pressure_apply(engine, oracle_lib, N1, N2, nu, stype):
    E = engine
    if stype == 0 and N1 != N2:
        pytest.skip("parallel configuration requires a square grid (src/SimParams.cpp:459-462)")
    P, ctx = _ctx(E, N1, N2, nu=nu, stype=stype)
    OP = oparams(P)
    c = _rand_c(N1, N2, 2)
    x = np.random.default_rng(3).normal(size=(N1, N2))
    A = np.zeros(N1 * N2 * 9)
    oracle_lib.or_pressure_matrix(C.byref(OP), O.ptr(cell_ghost(OP, c)), O.ptr(A))
    y_or = np.zeros(N1 * N2)
    oracle_lib.or_matvec9(C.byref(OP), O.ptr(A), O.ptr(x.ravel().copy()), O.ptr(y_or))
    import torch
    y = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
    ctx.pressure_apply(dev(c), dev(x), y)
    scale = np.abs(A.reshape(-1, 9)).sum(1).max() * np.abs(x).max()
    assert np.abs(host(y).ravel() - y_or).max() <= 1e-13 * scale


def _oracle_pressure(oracle_lib, OP, c, q):
    p = np.zeros(O.scalar_shape(OP))
    its, rr = C.c_int(), C.c_double()
    rc = oracle_lib.or_pressure_solve(C.byref(OP), O.ptr(cell_ghost(OP, c)), O.ptr(q), O.ptr(p), 0, 1e-14,
                                      C.byref(its), C.byref(rr))
    assert rc == 0
    return O.interior(OP, p).copy()


@pytest.mark.parametrize("N1,N2", GRIDS + [(141, 141), (100, 50)])
@pytest.mark.parametrize("nu", [1.0, 2.0 / 3.0])
@pytest.mark.parametrize("prec", [0, 1])
def test_pressure_solve(engine, oracle_lib, N1, N2, nu, prec):
    E = engine
    stype = 0 if N1 == N2 == 141 else 1
    P, ctx = _ctx(E, N1, N2, nu=nu, stype=stype, precision=prec, max_cycles=200)
    OP = oparams(P)
    c = _rand_c(N1, N2, 4)
    q = source(OP)
    ctx.set_source(dev(q))
    import torch
    p = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
    tol = 1e-12
    cyc, rr, _ = ctx.pressure_solve(dev(c), p, tol)
    assert rr <= tol and cyc < 200
    # relative residual of the device solution under the oracle's (reference) pinned matrix
    A = np.zeros(N1 * N2 * 9)
    b = np.zeros(N1 * N2)
    oracle_lib.or_pressure_matrix(C.byref(OP), O.ptr(cell_ghost(OP, c)), O.ptr(A))
    oracle_lib.or_pressure_rhs(C.byref(OP), O.ptr(q), O.ptr(b))
    ph = host(p).ravel().copy()
    rr_or = oracle_lib.or_relres9(C.byref(OP), O.ptr(A), O.ptr(ph), O.ptr(b))
    assert rr_or <= 2 * tol
    # agreement with the direct solve: kappa(A) ~ 1e5 at these sizes
    p_or = _oracle_pressure(oracle_lib, OP, c, q)
    assert rel_err(host(p), p_or) <= 1e-6


@pytest.mark.parametrize("N1,N2", [(37, 29), (141, 141), (100, 50), (300, 130)])
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("ctas", ["16", "8"])
@pytest.mark.parametrize("nu", [1.0, 2.0 / 3.0])
def test_cluster_vcycle_matches_per_level_kernels(engine, monkeypatch, N1, N2, prec, ctas, nu):
    """The coarse levels of a V-cycle in one cluster launch (row bands in shared memory,
    neighbour rows over distributed shared memory) reproduce the per-level launches bit for bit:
    same cycles, same residual, same pressure, with fewer launches.  nu = 2/3 gives nine-point
    operators, smoothed by four-colour Gauss-Seidel."""
    E = engine
    import torch
    monkeypatch.setenv("IMPEC_MG_CL_CTAS", ctas)
    out = []
    for cluster in ("0", "1"):
        monkeypatch.setenv("IMPEC_MG_CLUSTER", cluster)
        P, ctx = _ctx(E, N1, N2, nu=nu, stype=1, precision=prec, max_cycles=200)
        OP = oparams(P)
        ctx.set_source(dev(source(OP)))
        p = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
        n0 = E.launch_count(ctx)
        cyc, rr, _ = ctx.pressure_solve(dev(_rand_c(N1, N2, 9)), p, 1e-11)
        out.append((cyc, rr, host(p), E.launch_count(ctx) - n0))
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])
    if prec == 1 and nu < 1.0:  # FP32 nine-point cycles do not use the cluster kernel
        assert out[1][3] == out[0][3]
    else:
        assert out[1][3] < out[0][3]  # the cluster kernel replaced per-level launches


@pytest.mark.parametrize("N1,N2,stype", [(37, 29, 1), (300, 130, 1), (1024, 1024, 1), (97, 70, 2)])
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("krylov", ["1", "0"])
def test_red_black_shortcuts_match_full_kernels(engine, monkeypatch, N1, N2, stype, prec, krylov):
    """Pre-smoothing that starts from an implicit zero (no zero fill; the first colour is
    x = b / diag) and a red-only prolongation ahead of a sweep that overwrites the black cells
    change nothing. The cycles, residual and pressure are the same bit for bit as with the full
    kernels, for the CG and the stationary iteration, and with a Dirichlet row (stype 2)."""
    E = engine
    import torch
    monkeypatch.setenv("IMPEC_MG_KRYLOV", krylov)
    out = []
    for skip in ("0", "1"):
        monkeypatch.setenv("IMPEC_MG_RB_SKIP", skip)
        P, ctx = _ctx(E, N1, N2, nu=1.0, stype=stype, precision=prec, max_cycles=200)
        OP = oparams(P)
        ctx.set_source(dev(source(OP)))
        p = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
        cyc, rr, _ = ctx.pressure_solve(dev(_rand_c(N1, N2, 9)), p, 1e-11)
        out.append((cyc, rr, host(p)))
        ctx.close()
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])
    assert out[1][1] <= 1e-11


@pytest.mark.parametrize("N1,N2,stype", [(37, 29, 1), (300, 130, 1), (1024, 1024, 1), (97, 70, 2)])
@pytest.mark.parametrize("prec", [0, 1])
def test_red_only_restriction(engine, monkeypatch, N1, N2, stype, prec):
    """Restriction that sums only the red residuals: after the pre-smoothing's black pass the
    black residuals are zero up to one rounding, so dropping them moves the coarse right-hand
    side by about machine epsilon.  The solve needs the same CG iterations, meets the
    tolerance, and lands within it of the full restriction's solution."""
    E = engine
    import torch
    tol = 1e-11
    out = []
    for red_only in ("0", "1"):
        monkeypatch.setenv("IMPEC_MG_RB_RESID", red_only)
        P, ctx = _ctx(E, N1, N2, nu=1.0, stype=stype, precision=prec, max_cycles=200)
        OP = oparams(P)
        ctx.set_source(dev(source(OP)))
        p = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
        cyc, rr, _ = ctx.pressure_solve(dev(_rand_c(N1, N2, 9)), p, tol)
        out.append((cyc, rr, host(p)))
        ctx.close()
    assert out[0][0] == out[1][0], (out[0][:2], out[1][:2])
    assert out[0][1] <= tol and out[1][1] <= tol
    # both solve to 1e-11 in relative residual; kappa ~ 1e5 at these sizes
    assert rel_err(out[1][2], out[0][2]) <= 1e-6


@pytest.mark.parametrize("N1,N2", GRIDS)
@pytest.mark.parametrize("nu", [1.0, 2.0 / 3.0])
def test_velocity(engine, oracle_lib, N1, N2, nu):
    E = engine
    P, ctx = _ctx(E, N1, N2, nu=nu)
    OP = oparams(P)
    c = _rand_c(N1, N2, 5)
    p = smooth_field(N1, N2, 6, -3.0, 2.0)
    pg = cell_ghost(OP, p)
    v = np.zeros(O.vel_shape(OP))
    oracle_lib.or_calc_velocities(C.byref(OP), O.ptr(pg), O.ptr(v), O.ptr(cell_ghost(OP, c)))
    u_or, v_or = vel_split(OP, v)
    import torch
    du = torch.zeros((N1 + 1, N2), dtype=torch.float64, device="cuda")
    dv = torch.zeros((N1, N2 + 1), dtype=torch.float64, device="cuda")
    ctx.velocity(dev(p), dev(c), du, dv)
    scale = max(np.abs(u_or).max(), np.abs(v_or).max())
    assert np.abs(host(du) - u_or).max() <= 1e-13 * scale
    assert np.abs(host(dv) - v_or).max() <= 1e-13 * scale
    dt_or = oracle_lib.or_max_stable_dt(C.byref(OP), O.ptr(v))
    dt = ctx.max_stable_dt(dev(u_or), dev(v_or))
    assert dt == pytest.approx(dt_or, rel=1e-14)


def _vel_field(OP, seed):
    """A consistent velocity field: oracle Darcy velocities of a smooth pressure."""
    c = _rand_c(OP.N1, OP.N2, seed)
    p = smooth_field(OP.N1, OP.N2, seed + 1, -1.0, 1.0) * 0.05
    v = np.zeros(O.vel_shape(OP))
    O.lib().or_calc_velocities(C.byref(OP), O.ptr(cell_ghost(OP, p)), O.ptr(v), O.ptr(cell_ghost(OP, c)))
    return v


@pytest.mark.parametrize("N1,N2", GRIDS)
@pytest.mark.parametrize("scheme", [4, 0, 1, 2, 3])  # MUSCL, upwind, WAF split, WAF, CTU (unsplit)
@pytest.mark.parametrize("mode", [4, 0, 1, 2, 3])
def test_advect_split(engine, oracle_lib, N1, N2, scheme, mode):
    E = engine
    P, ctx = _ctx(E, N1, N2, hmtype=scheme, dim_splitting=mode, porosity=0.7)
    OP = oparams(P)
    vg = _vel_field(OP, 7)
    u, v = vel_split(OP, vg)
    c = _rand_c(N1, N2, 8)
    cg = cell_ghost(OP, c)
    dt = 0.9 * oracle_lib.or_max_stable_advection_dt(C.byref(OP), O.ptr(vg)) * OP.porosity
    for pfs0 in (0, 1):
        cg2 = cg.copy()
        pfs = C.c_int(pfs0)
        oracle_lib.or_advect_split(C.byref(OP), O.ptr(cg2), O.ptr(vg), dt, C.byref(pfs))
        dc = dev(c)
        pfs_dev = ctx.advect_split(dc, dev(u), dev(v), dt, pfs0)
        assert pfs_dev == pfs.value
        assert rel_err(host(dc), O.interior(OP, cg2)) <= 1e-13


@pytest.mark.parametrize("scheme", [4, 0, 1, 3])
def test_advect_periodic(engine, oracle_lib, scheme):
    """Periodic advection test setup of src/Impec2DSolver.cpp:848-1015 (constant velocity)."""
    E = engine
    N = 40
    P, ctx = _ctx(E, N, N, hmtype=scheme, bc=1, is_test=1, cfl=0.95)
    OP = oparams(P)
    vg = np.zeros(O.vel_shape(OP))
    vg[..., 0], vg[..., 1] = -1.0, 1.0
    u, v = vel_split(OP, vg)
    c = np.array([[oracle_lib.or_profile(C.byref(OP), 0, (i + .5) / N, (j + .5) / N) for j in range(N)]
                  for i in range(N)])
    cg = cell_ghost(OP, c, periodic=True)
    dt = oracle_lib.or_max_stable_advection_dt(C.byref(OP), O.ptr(vg))
    pfs = C.c_int(1)
    oracle_lib.or_advect_split(C.byref(OP), O.ptr(cg), O.ptr(vg), dt, C.byref(pfs))
    dc = dev(c)
    ctx.advect_split(dc, dev(u), dev(v), dt, 1)
    assert rel_err(host(dc), O.interior(OP, cg)) <= 1e-13


@pytest.mark.parametrize("N1,N2", GRIDS)
@pytest.mark.parametrize("stype", [1, 0])
def test_tr_integrate(engine, oracle_lib, N1, N2, stype):
    E = engine
    if stype == 0 and N1 != N2:
        pytest.skip("parallel configuration requires a square grid")
    P, ctx = _ctx(E, N1, N2, stype=stype)
    OP = oparams(P)
    q = source(OP)
    ctx.set_source(dev(q))
    c = _rand_c(N1, N2, 9)
    cg = cell_ghost(OP, c)
    dt = 1e-4
    tmo_or = oracle_lib.or_tr_integrate(C.byref(OP), O.ptr(cg), O.ptr(q), dt)
    dc = dev(c)
    tmo = ctx.tr_integrate(dc, dt)
    assert rel_err(host(dc), O.interior(OP, cg)) <= 1e-15
    assert tmo == pytest.approx(tmo_or, rel=1e-13, abs=1e-300)


@pytest.mark.parametrize("N1,N2", GRIDS)
@pytest.mark.parametrize("alpha", [(1e-3, 1e-4), (1.0, 0.1)])
def test_dispersion_cn(engine, oracle_lib, N1, N2, alpha):
    E = engine
    P, ctx = _ctx(E, N1, N2, diffusion=1, alpha_l=alpha[0], alpha_t=alpha[1], para_eps=1e-13, max_cycles=400)
    OP = oparams(P)
    vg = _vel_field(OP, 10)
    u, v = vel_split(OP, vg)
    c = _rand_c(N1, N2, 11)
    cg = cell_ghost(OP, c)
    dt = 0.5 * oracle_lib.or_max_stable_dt(C.byref(OP), O.ptr(vg))
    its, rr = C.c_int(), C.c_double()
    assert oracle_lib.or_cn_solve(C.byref(OP), O.ptr(cg), O.ptr(vg), dt, 0, 1e-14, C.byref(its), C.byref(rr)) == 0
    dc = dev(c)
    its_d, rr_d = ctx.dispersion_cn(dc, dev(u), dev(v), dt, 1e-13)
    assert rr_d <= 1e-13
    assert rel_err(host(dc), O.interior(OP, cg)) <= 1e-11


@pytest.mark.parametrize("cfg", ["diag_upwind", "par_muscl_disp", "diag_muscl_disp_nu"])
def test_impes_steps_short_horizon(engine, oracle_lib, cfg):
    """Whole IMPES steps (pressure, velocity, dt, split transport) against the oracle over a
    short horizon, before the physical instability amplifies differences."""
    E = engine
    N = 48
    kw = dict(diag_upwind=dict(stype=1, hmtype=0, nu=1.0),
              par_muscl_disp=dict(stype=0, hmtype=4, nu=1.0, diffusion=1, alpha_l=1e-3, alpha_t=1e-4),
              diag_muscl_disp_nu=dict(stype=1, hmtype=4, nu=2.0 / 3.0, diffusion=1, alpha_l=1.0, alpha_t=0.1))[cfg]
    P, ctx = _ctx(E, N, N, eps=1e-13, para_eps=1e-13, max_cycles=200, **kw)
    OP = oparams(P)
    q = source(OP)
    c0 = np.zeros((N, N))
    cptr, pptr, uptr, vptr, qptr = ctx.state_ptrs()
    ctx.upload(cell_ghost(OP, c0), q, ghost=2)
    c = cell_ghost(OP, c0)
    p = np.zeros(O.scalar_shape(OP))
    vv = np.zeros(O.vel_shape(OP))
    S = O.State()
    S.prev_first_sweep = 1
    tidx = C.c_int(0)
    for k in range(10):
        oracle_lib.or_impes_step(C.byref(OP), C.byref(S), O.ptr(c), O.ptr(p), O.ptr(vv), O.ptr(q), None, 0,
                                 C.byref(tidx), 0, 1e-14)
        info = ctx.step()
        assert info.dt == pytest.approx(S.dt, rel=1e-9)
    ch, ph, vh = np.zeros_like(c), np.zeros_like(p), np.zeros_like(vv)
    ctx.download(ch, ph, vh, ghost=2)
    assert rel_err(O.interior(OP, ch), O.interior(OP, c)) <= 1e-9
    assert rel_err(O.interior(OP, ph), O.interior(OP, p)) <= 1e-8
    assert info.mass_err < 1e-12


def test_large_grid_properties(engine, oracle_lib):
    """1024^2 parallel configuration: size-independent invariants (mass balance, no-flow,
    div u = q) and solver convergence to 1e-10 in both precisions."""
    E = engine
    N = 1024
    for prec in (0, 1):
        P = E.default_params(N, N, stype=0, x_ub=2 ** 0.5, y_ub=2 ** 0.5, hmtype=4, diffusion=1, alpha_l=1e-3,
                             alpha_t=1e-4, Dm=1e-6, eps=1e-10, para_eps=1e-10, precision=prec)
        ctx = E.Context(P)
        OP = oparams(P)
        q = source(OP)
        ctx.upload(cell_ghost(OP, np.zeros((N, N))), q, ghost=2)
        for k in range(3):
            info = ctx.step()
            assert info.relres <= 1e-10
        cptr, pptr, uptr, vptr, _ = ctx.state_ptrs()
        import torch
        c = torch.empty((N, N), dtype=torch.float64, device="cuda")
        u = torch.empty((N + 1, N), dtype=torch.float64, device="cuda")
        v = torch.empty((N, N + 1), dtype=torch.float64, device="cuda")
        ch = np.zeros(O.scalar_shape(OP))
        vh = np.zeros(O.vel_shape(OP))
        ctx.download(ch, None, vh, ghost=2)
        uh, vvh = vel_split(OP, vh)
        c.copy_(dev(O.interior(OP, ch)))
        u.copy_(dev(uh))
        v.copy_(dev(vvh))
        mass, div_err, vel_err, cmax, cmin = ctx.diagnostics(c, u, v)
        assert info.mass_err < 1e-11
        assert vel_err < 1e-9 * np.abs(uh).max()
        assert div_err < 1e-6
        ctx.close()


@pytest.mark.parametrize("N1,N2", [(64, 64), (101, 101), (90, 70)])
def test_parallel_projection_bitexact(engine, oracle_lib, N1, N2):
    """Output projection of a parallel run onto the diagonal grid
    (ParallelProjector::FillDiagonal, src/ParallelProjector.cpp:178-199) equals the oracle's
    restatement bit for bit, for c and p, on device and host buffers."""
    E = engine
    import torch
    r2 = np.sqrt(2.0)
    P, ctx = _ctx(E, N1, N2, x_ub=r2, y_ub=r2, stype=0)
    OP = oparams(P)
    g = OP.g
    c = smooth_field(N1, N2, 21)
    p = smooth_field(N1, N2, 22, -3.0, 2.0)
    ctx.upload(np.ascontiguousarray(cell_ghost(OP, c)), None, ghost=g)
    ph = np.ascontiguousarray(cell_ghost(OP, p))
    assert E.lib().impec_pressure_upload(ctx.h, ph.ctypes.data_as(C.POINTER(C.c_double)), g) == 0
    dN1, dN2 = int(round(N1 / r2)), int(round(N2 / r2))
    for field, interior in ((0, c), (1, p)):
        ref = np.zeros(dN1 * dN2)
        oracle_lib.or_project_diagonal(C.byref(OP), O.ptr(cell_ghost(OP, interior)), dN1, dN2, O.ptr(ref))
        out = torch.zeros(dN1 * dN2, dtype=torch.float64, device="cuda")
        ctx.project_diagonal(field, out, dN1, dN2)
        torch.cuda.synchronize()
        assert np.array_equal(host(out), ref)
        hb = np.zeros(dN1 * dN2)
        s = E.lib().impec_project_diagonal_download(ctx.h, field, hb.ctypes.data_as(C.POINTER(C.c_double)), dN1, dN2)
        assert s == 0 and np.array_equal(hb, ref)


@pytest.mark.parametrize("prec", [0, 1])
def test_cg_and_stationary_cycles_agree_on_heterogeneous_coefficients(engine, oracle_lib, monkeypatch, prec):
    """V-cycle preconditioned CG (the default) and stationary V-cycles both reach the
    tolerance under the oracle's own matrix on a lognormal permeability field, agree with
    each other, and CG needs fewer cycles."""
    E = engine
    import torch
    N1, N2 = 129, 97
    rng = np.random.default_rng(7)
    K = np.exp(2.0 * (smooth_field(N1, N2, 31) - 0.5) + 0.3 * rng.standard_normal((N1, N2)))
    c = _rand_c(N1, N2, 32)
    out = {}
    for kry in ("0", "1"):
        monkeypatch.setenv("IMPEC_MG_KRYLOV", kry)
        P, ctx = _ctx(E, N1, N2, nu=1.0, stype=1, precision=prec, max_cycles=400)
        OP = oparams(P)
        q = source(OP)
        ctx.set_source(dev(q))
        ctx.set_permeability(dev(K), dev(K))
        p = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
        cyc, rr, _ = ctx.pressure_solve(dev(c), p, 1e-11)
        assert rr <= 1e-11
        out[kry] = (cyc, host(p))
    assert out["1"][0] < out["0"][0]
    assert rel_err(out["1"][1], out["0"][1]) <= 1e-7


# ---------------------------------------------------------------- horizontal-front source
# source_type "horizontal": injection over the first and production over the last well_width
# rows (InitHorizontalFront, src/Util.cpp:607-639), a Dirichlet row (1, j) in the pressure
# system (src/MGSolver.cpp:119-140, 518-567) and (N1-2, j) in the CN system (:1295-1317).

@pytest.mark.parametrize("nu", [1.0, 2.0 / 3.0])
def test_horizontal_pressure_apply(engine, oracle_lib, nu):
    E = engine
    N1, N2 = 40, 32
    P, ctx = _ctx(E, N1, N2, nu=nu, stype=2)
    OP = oparams(P)
    ctx.set_source(dev(source(OP)))
    c = _rand_c(N1, N2, 2)
    x = np.random.default_rng(3).normal(size=(N1, N2))
    A = np.zeros(N1 * N2 * 9)
    oracle_lib.or_pressure_matrix(C.byref(OP), O.ptr(cell_ghost(OP, c)), O.ptr(A))
    y_or = np.zeros(N1 * N2)
    oracle_lib.or_matvec9(C.byref(OP), O.ptr(A), O.ptr(x.ravel().copy()), O.ptr(y_or))
    import torch
    y = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
    ctx.pressure_apply(dev(c), dev(x), y)
    scale = np.abs(A.reshape(-1, 9)).sum(1).max() * np.abs(x).max()
    assert np.abs(host(y).ravel() - y_or).max() <= 1e-13 * scale


@pytest.mark.parametrize("N1,N2", [(64, 48), (97, 70)])
@pytest.mark.parametrize("nu", [1.0, 2.0 / 3.0])
@pytest.mark.parametrize("prec", [0, 1])
def test_horizontal_pressure_solve(engine, oracle_lib, N1, N2, nu, prec):
    """The Dirichlet-row system (known cells eliminated, SPD) solved by V-cycle CG reaches the
    tolerance under the oracle's matrix and matches the oracle's banded LU solve."""
    E = engine
    import torch
    P, ctx = _ctx(E, N1, N2, nu=nu, stype=2, precision=prec, max_cycles=200)
    OP = oparams(P)
    c = _rand_c(N1, N2, 4)
    q = source(OP)
    ctx.set_source(dev(q))
    p = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
    tol = 1e-12
    cyc, rr, _ = ctx.pressure_solve(dev(c), p, tol)
    assert rr <= tol and cyc < 200
    A = np.zeros(N1 * N2 * 9)
    b = np.zeros(N1 * N2)
    oracle_lib.or_pressure_matrix(C.byref(OP), O.ptr(cell_ghost(OP, c)), O.ptr(A))
    oracle_lib.or_pressure_rhs(C.byref(OP), O.ptr(q), O.ptr(b))
    ph = host(p).ravel().copy()
    assert oracle_lib.or_relres9(C.byref(OP), O.ptr(A), O.ptr(ph), O.ptr(b)) <= 2 * tol
    p_or = _oracle_pressure(oracle_lib, OP, c, q)
    assert rel_err(host(p), p_or) <= 1e-8


@pytest.mark.parametrize("prec", [0, 1])
def test_true_residual_loop_host_and_graph(engine, oracle_lib, prec):
    """CG's recurrence residual drifts from the true one by rounding, so each stop is verified
    on the true residual and CG continues from it until ||b - A p|| / ||b|| itself meets tol.
    This Dirichlet-row system at 1e-12 needs that: the recurrence stop alone left a true
    residual of 1.1e-12.  The host-driven solve and the resident graph (WHILE node) give the
    same cycles, residual and pressure bits, and the oracle's matrix confirms the residual."""
    E = engine
    import torch
    N1, N2, tol = 97, 70, 1e-12
    out = []
    for resident in (False, True):
        P, ctx = _ctx(E, N1, N2, nu=1.0, stype=2, precision=prec, max_cycles=200, eps=tol)
        OP = oparams(P)
        c = _rand_c(N1, N2, 4)
        q = source(OP)
        if resident:
            ctx.upload(cell_ghost(OP, c), q, ghost=2)
            cyc, rr = ctx.pressure_solve_resident()
            pg = np.zeros((N1 + 4, N2 + 4))
            ctx.download(None, pg, None, ghost=2)
            p = pg[2:-2, 2:-2].copy()
        else:
            ctx.set_source(dev(q))
            pd = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
            cyc, rr, _ = ctx.pressure_solve(dev(c), pd, tol)
            p = host(pd)
        out.append((cyc, rr, p))
        ctx.close()
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1], (out[0][:2], out[1][:2])
    assert np.array_equal(out[0][2], out[1][2])
    assert out[0][1] <= tol
    A = np.zeros(N1 * N2 * 9)
    b = np.zeros(N1 * N2)
    oracle_lib.or_pressure_matrix(C.byref(OP), O.ptr(cell_ghost(OP, c)), O.ptr(A))
    oracle_lib.or_pressure_rhs(C.byref(OP), O.ptr(q), O.ptr(b))
    ph = out[0][2].ravel().copy()
    assert oracle_lib.or_relres9(C.byref(OP), O.ptr(A), O.ptr(ph), O.ptr(b)) <= 2 * tol


def test_horizontal_dispersion_cn(engine, oracle_lib):
    """CN with the Dirichlet row c = 0 at i = N1-2."""
    E = engine
    N1, N2 = 48, 40
    P, ctx = _ctx(E, N1, N2, stype=2, diffusion=1, alpha_l=1.0, alpha_t=0.1, para_eps=1e-13, max_cycles=400)
    OP = oparams(P)
    vg = _vel_field(OP, 10)
    u, v = vel_split(OP, vg)
    c = _rand_c(N1, N2, 11)
    cg = cell_ghost(OP, c)
    dt = 0.5 * oracle_lib.or_max_stable_dt(C.byref(OP), O.ptr(vg))
    its, rr = C.c_int(), C.c_double()
    assert oracle_lib.or_cn_solve(C.byref(OP), O.ptr(cg), O.ptr(vg), dt, 0, 1e-14, C.byref(its), C.byref(rr)) == 0
    dc = dev(c)
    its_d, rr_d = ctx.dispersion_cn(dc, dev(u), dev(v), dt, 1e-13)
    assert rr_d <= 1e-13
    out = host(dc)
    assert np.all(out[N1 - 2] == 0.0)
    assert rel_err(out, O.interior(OP, cg)) <= 1e-11


@pytest.mark.parametrize("nu,disp,pulsing", [(1.0, 0, False), (2.0 / 3.0, 1, False), (2.0 / 3.0, 1, True)])
def test_horizontal_impes_steps_short_horizon(engine, oracle_lib, nu, disp, pulsing):
    """Whole IMPES steps with the horizontal front against the oracle; with pulsing injection
    (InitHorizontalFront at the current time before every step, src/Impec2DSolver.cpp:437-439)
    the rates change in place between steps."""
    E = engine
    N1, N2 = 48, 40
    kw = dict(stype=2, hmtype=4, nu=nu, diffusion=disp, alpha_l=1e-2, alpha_t=1e-3)
    P, ctx = _ctx(E, N1, N2, eps=1e-13, para_eps=1e-13, max_cycles=200, **kw)
    OP = oparams(P, inj_mode=0, q_freq=400.0) if pulsing else oparams(P)
    q = source(OP)
    rates = set()
    c0 = np.zeros((N1, N2))
    ctx.upload(cell_ghost(OP, c0), q, ghost=2)
    c = cell_ghost(OP, c0)
    p = np.zeros(O.scalar_shape(OP))
    vv = np.zeros(O.vel_shape(OP))
    S = O.State()
    S.prev_first_sweep = 1
    tidx = C.c_int(0)
    for k in range(8):
        if pulsing:
            oracle_lib.or_init_source(C.byref(OP), O.ptr(q), S.t)
            ctx.set_source(dev(q))
            rates.add(float(q[0]))
        oracle_lib.or_impes_step(C.byref(OP), C.byref(S), O.ptr(c), O.ptr(p), O.ptr(vv), O.ptr(q), None, 0,
                                 C.byref(tidx), 0, 1e-14)
        info = ctx.step()
        assert info.dt == pytest.approx(S.dt, rel=1e-9)
    if pulsing:
        assert len(rates) == 2  # both phases of the pulse were used
    ch, ph, vh = np.zeros_like(c), np.zeros_like(p), np.zeros_like(vv)
    ctx.download(ch, ph, vh, ghost=2)
    assert rel_err(O.interior(OP, ch), O.interior(OP, c)) <= 1e-9
    assert rel_err(O.interior(OP, ph), O.interior(OP, p)) <= 1e-8


def test_horizontal_source_rate_update_in_place(engine):
    """A source with the same well cells and new rates (the pulsing / linear front,
    src/Impec2DSolver.cpp:437-439) updates the rates in place; the next steps equal those of a
    context built with the new rates from the start."""
    E = engine
    N1, N2 = 40, 32
    P, ctx = _ctx(E, N1, N2, stype=2)
    q = source(oparams(P))
    z = np.zeros((N1 + 4, N2 + 4))
    P2, ref = _ctx(E, N1, N2, stype=2)
    for cx in (ctx, ref):
        cx.upload(z, q, ghost=2)
        cx.step()  # captures the step graph
    ctx.set_source(dev(q * 50.0))  # same cells: rates updated under the existing graph
    ref.set_source(dev(np.zeros_like(q)))  # different cells: well list rebuilt, graph captured again
    ref.set_source(dev(q * 50.0))
    for _ in range(3):
        a, b = ctx.step(), ref.step()
        assert a.dt == b.dt
    ca, cb = np.zeros_like(z), np.zeros_like(z)
    ctx.download(ca, None, None, ghost=2)
    ref.download(cb, None, None, ghost=2)
    assert np.array_equal(ca, cb)


@pytest.mark.parametrize("cfg", ["diag_upwind", "par_muscl_disp", "diag_muscl_disp_nu", "diag_upwind_mixed"])
def test_quarter_five_spot_integrated_quantities(engine, oracle_lib, cfg):
    """A whole displacement at 32 x 32, M = 41, porosity 1, to 1 pore volume injected, engine
    and oracle in lockstep: the reference's CPU case (diagonal grid, first-order upwind) and
    the benchmark's method (parallel grid with four corner wells, MUSCL, Crank-Nicolson
    Peaceman dispersion).  Past breakthrough the unstable displacement lets round-off grow,
    so the comparison is by integrated quantities: the time step of every step, the
    breakthrough step and time (produced volume above 1e-3), the produced volume at the end,
    and mass balance."""
    E = engine
    N = 32
    kw = dict(diag_upwind=dict(stype=1, hmtype=0, nu=1.0),
              par_muscl_disp=dict(stype=0, hmtype=4, nu=1.0, diffusion=1, alpha_l=1e-3, alpha_t=1e-4),
              # the reference examples' weighted nine-point operator
              diag_muscl_disp_nu=dict(stype=1, hmtype=4, nu=2.0 / 3.0, diffusion=1, alpha_l=1.0, alpha_t=0.1),
              # mixed-precision pressure against the FP64 oracle
              diag_upwind_mixed=dict(stype=1, hmtype=0, nu=1.0, precision=1))[cfg]
    P, ctx = _ctx(E, N, N, cfl=0.5, mu_res=41.0, mu_inj=1.0, eps=1e-10, para_eps=1e-10, **kw)
    OP = oparams(P)
    q = source(OP)
    ctx.upload(cell_ghost(OP, np.zeros((N, N))), q, ghost=2)
    ctx.set_time(0.0)
    c = cell_ghost(OP, np.zeros((N, N)))
    p, vv = np.zeros(O.scalar_shape(OP)), np.zeros(O.vel_shape(OP))
    S = O.State()
    S.prev_first_sweep = 1
    tidx = C.c_int(0)
    bt_e = bt_o = None
    worst_dt = mass_e = mass_o = 0.0
    n = 0
    t_end = 1.0 * (P.x_ub - P.x_lb) * (P.y_ub - P.y_lb) / (2.0 if P.stype == 0 else 1.0)  # 1 PV
    while S.t < t_end:
        oracle_lib.or_impes_step(C.byref(OP), C.byref(S), O.ptr(c), O.ptr(p), O.ptr(vv), O.ptr(q), None, 0,
                                 C.byref(tidx), 0, 1e-13)
        info = ctx.step()
        n += 1
        worst_dt = max(worst_dt, abs(info.dt - S.dt) / S.dt)
        if bt_o is None and S.total_outflux > 1e-3:
            bt_o = (n, S.t)
        if bt_e is None and info.total_outflux > 1e-3:
            bt_e = (n, info.t)
        mass_e, mass_o = max(mass_e, info.mass_err), max(mass_o, S.mass_err)
    rel_out = abs(info.total_outflux - S.total_outflux) / S.total_outflux
    print(f"{n} steps to t = {S.t:.4f}: worst dt deviation {worst_dt:.2e}; breakthrough engine {bt_e}, "
          f"oracle {bt_o}; produced {info.total_outflux:.6f} vs {S.total_outflux:.6f} (rel {rel_out:.2e}); "
          f"max mass error engine {mass_e:.1e}, oracle {mass_o:.1e}")
    # mass balance: the engine's CN solves stop at the 1e-10 relative residual asked for, which is
    # not exactly conservative (measured up to 1.8e-9 with strong nine-point dispersion)
    assert mass_e <= 1e-8 and mass_o <= 1e-8
    assert worst_dt <= 1e-8
    assert bt_e is not None and bt_o is not None and abs(bt_e[0] - bt_o[0]) <= 1
    assert abs(bt_e[1] - bt_o[1]) <= 1e-9 * bt_o[1]
    assert rel_out <= 1e-8  # measured: 3e-12 (upwind, FP64 or mixed) to 3.6e-9 (nine-point dispersion)
    ctx.close()


@pytest.mark.parametrize("N1,N2,stype,eps", [(64, 64, 0, 1e-10), (97, 70, 2, 1e-12)])
def test_graph_replay_counts_the_launches_of_the_stream_path(engine, monkeypatch, N1, N2, stype, eps):
    """The step graph's launch accounting (fixed nodes plus loop bodies times their trip
    counts, the basis of the bench's gpu_launches) equals the kernels the stream path launches
    one by one for the same steps, and both give the same state.  The second case is a
    Dirichlet-row system at a tolerance where the true-residual verification can continue CG."""
    E = engine
    counts, states = [], []
    for graph in (True, False):
        if graph:
            monkeypatch.delenv("IMPEC_NO_GRAPH", raising=False)
        else:
            monkeypatch.setenv("IMPEC_NO_GRAPH", "1")
        P, ctx = _ctx(E, N1, N2, stype=stype, hmtype=4, nu=1.0, diffusion=1, alpha_l=1e-3, alpha_t=1e-4, eps=eps,
                      para_eps=1e-10)
        OP = oparams(P)
        ctx.upload(cell_ghost(OP, np.zeros((N1, N2))), source(OP), ghost=2)
        ctx.set_time(0.0)
        ctx.step()  # graph mode: capture and first replay
        n0 = E.launch_count(ctx)
        for _ in range(3):
            ctx.step()
        counts.append(E.launch_count(ctx) - n0)
        ch, ph = np.zeros((N1 + 4, N2 + 4)), np.zeros((N1 + 4, N2 + 4))
        ctx.download(ch, ph, None, ghost=2)
        states.append((ch, ph))
        ctx.close()
    assert counts[0] == counts[1] and counts[0] > 0, counts
    assert np.array_equal(states[0][0], states[1][0]) and np.array_equal(states[0][1], states[1][1])


@pytest.mark.parametrize("nu", [1.0, 2.0 / 3.0])
def test_pinned_solve_anisotropic_permeability(engine, oracle_lib, nu):
    """K11 != K22 (an engine extension; the reference has K = 1): the consistent-singular solve
    plus shift still satisfies the reference's pinned system, because the folded operator stays
    symmetric with zero column sums (tests/test_oracle.py); checked against the oracle's banded
    LU of the pinned matrix."""
    import torch
    E = engine
    N1, N2 = 40, 36
    rng = np.random.default_rng(21)
    K11, K22 = np.exp(0.5 * rng.normal(size=(N1, N2))), np.exp(0.5 * rng.normal(size=(N1, N2)))
    P, ctx = _ctx(E, N1, N2, nu=nu, stype=1, max_cycles=300)
    OP = oparams(P, K11=K11, K22=K22)
    c = _rand_c(N1, N2, 22)
    q = source(OP)
    ctx.set_source(dev(q))
    ctx.set_permeability(dev(K11), dev(K22))
    p = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
    cyc, rr, _ = ctx.pressure_solve(dev(c), p, 1e-12)
    A, b = np.zeros(N1 * N2 * 9), np.zeros(N1 * N2)
    oracle_lib.or_pressure_matrix(C.byref(OP), O.ptr(cell_ghost(OP, c)), O.ptr(A))
    oracle_lib.or_pressure_rhs(C.byref(OP), O.ptr(q), O.ptr(b))
    rr_or = oracle_lib.or_relres9(C.byref(OP), O.ptr(A), O.ptr(host(p).ravel().copy()), O.ptr(b))
    assert rr <= 1e-12 and rr_or <= 2e-12, (rr, rr_or)
    assert rel_err(host(p), _oracle_pressure(oracle_lib, OP, c, q)) <= 1e-8
    ctx.close()


@pytest.mark.parametrize("method,order", [("waf", 1.99349), ("waf_split", 1.99349), ("ctu", 2.01571)])
def test_waf_ctu_convergence_through_the_cfg_surface(engine, oracle_lib, tmp_path, method, order):
    """The advection convergence case of examples/hyperbolic_test.cfg (sine, L1, CFL 0.95,
    periodic, 50^2 doubled over 4 levels) with hyper_method waf / waf_split / ctu, run like
    the reference executable (impec_run_cfg -> TestComponent): the engine's errors equal the
    oracle's to 1e-9 on the two cheap levels, and the order is the oracle's (recorded upstream:
    WAF 2.00924, CTU 2.00125; no reference source exists for either scheme)."""
    import os
    from test_oracle import _advection_error
    E = engine
    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "muscl_sine_convergence.cfg")
    text = open(gold).read().replace("@DIR@", str(tmp_path)).replace('hyper_method = "muscl"',
                                                                     f'hyper_method = "{method}"')
    cfg = tmp_path / "adv.cfg"
    cfg.write_text(text)
    assert E.lib().impec_run_cfg(str(cfg).encode(), 1) == 0, E.last_error()
    rows = np.loadtxt(tmp_path / "norm.out")
    hm = {"waf": O.WAF, "waf_split": O.WAFSPLIT, "ctu": O.CTU}[method]
    for k, N in enumerate([50, 100]):
        e_or = _advection_error(oracle_lib, N, (-1.0, 1.0), hmtype=hm)
        assert abs(np.exp(rows[k, 1]) / e_or - 1) <= 1e-9, (N, np.exp(rows[k, 1]), e_or)
    fit = np.polyfit(rows[:, 0], rows[:, 1], 1)[0]
    assert abs(fit - order) < 1e-3, fit


@pytest.mark.parametrize("N1,N2,stype", [(300, 130, 1), (1024, 1024, 1), (97, 70, 2), (515, 333, 1)])
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("krylov", ["1", "0"])
@pytest.mark.parametrize("graph", [True, False])
def test_one_launch_sweep_matches_two_launch_sweeps(engine, monkeypatch, N1, N2, stype, prec, krylov, graph):
    """A red-black sweep in one launch (k_rb_tile: both colours per tile, a recomputed ring,
    ping-pong iterates) gives the two-launch sweeps' result bit for bit: the same cycles,
    residual and pressure, for CG and the stationary iteration (whose finest level keeps the
    two-launch sweep), in FP64 and mixed precision, with a Dirichlet row (stype 2), through
    the captured solve graph (replayed three times) and the host-driven loop."""
    E = engine
    import torch
    monkeypatch.setenv("IMPEC_MG_KRYLOV", krylov)
    out = []
    for tile in ("0", "1"):
        monkeypatch.setenv("IMPEC_MG_TILE_CELLS", tile)
        monkeypatch.setenv("IMPEC_MG_TILE_CELLS32", tile)
        P, ctx = _ctx(E, N1, N2, nu=1.0, stype=stype, precision=prec, max_cycles=200)
        OP = oparams(P)
        q = source(OP)
        c = _rand_c(N1, N2, 12)
        if graph:
            ctx.upload(cell_ghost(OP, c), q, ghost=2)
            res = [ctx.pressure_solve_resident() for _ in range(3)]
            ph = np.zeros(O.scalar_shape(OP))
            ctx.download(None, ph, None, ghost=2)
            out.append((res, O.interior(OP, ph).copy()))
        else:
            ctx.set_source(dev(q))
            p = torch.zeros((N1, N2), dtype=torch.float64, device="cuda")
            cyc, rr, _ = ctx.pressure_solve(dev(c), p, 1e-11)
            out.append(([(cyc, rr)], host(p)))
        ctx.close()
    assert out[0][0] == out[1][0], (out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
