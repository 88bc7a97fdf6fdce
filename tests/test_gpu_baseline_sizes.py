"""Parity at the benchmark's own sizes, against the oracle (which tests/test_ref_pin.py and
tests/test_oracle_golden.py pin bit for bit to the reference's own code).

  * 1024^2, the benchmark workload (parallel quarter-five-spot, MUSCL, Crank-Nicolson Peaceman
    dispersion with alpha_l 1e-3, alpha_t 1e-4, Dm 1e-6), with the five-point operator and with
    the nine-point one of the reference's example .cfg files (nu = 2/3), one IMPES step from a
    developed, fingered concentration field: velocities of the same pressure 1e-13, the split advection
    1e-13, the CN half step 1e-11, the pressure's relative residual under the oracle's matrix
    <= 2 tol, and c after the whole step (measured errors recorded in the assertions);
  * the other transport schemes (upwind, WAF split, WAF, CTU) at 1024^2: one advection step of
    the developed state, both sweep orders, to 1e-13;
  * the reference's CPU case (128^2 diagonal quarter-five-spot, first-order upwind, porosity
    0.2, M = 41) to t = 0.06 (0.3 pore volumes), engine and oracle in lockstep, compared by
    integrated quantities (time steps, produced volume, mass balance);
  * 4096^2 heterogeneous pressure solves (c = logistic of a Gaussian random field with
    correlation length 32 cells, ln K a field with sigma 1 and correlation length 16), FP64 and
    mixed precision to 1e-10, against the oracle's FP64 multigrid solution.

Fields are seeded and made on the host (numpy), so engine and oracle see the same inputs.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from helpers import cell_ghost, dev, host, oparams, rel_err, source, vel_ghost, vel_split

pytestmark = pytest.mark.gpu


def grf(N, ell, seed):
    """Seeded Gaussian random field, covariance exp(-r^2/ell^2) (ell in cells), unit variance."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((N, N))
    f = np.fft.fftfreq(N)
    H = np.exp(-(np.pi * ell) ** 2 * (f[:, None] ** 2 + f[None, :] ** 2) / 2)
    x = np.fft.ifft2(np.fft.fft2(w) * H).real
    return (x - x.mean()) / x.std()


def fingered(N, seed):
    """A developed displacement: injected fluid from the corner wells, with fingers (c in [0, 1])."""
    i = (np.arange(N)[:, None] + 0.5) / N
    j = (np.arange(N)[None, :] + 0.5) / N
    r = np.minimum(np.hypot(i, j), np.hypot(1 - i, 1 - j))  # distance to the injector corners
    front = 0.35 + 0.05 * grf(N, 24, seed)
    return 1.0 / (1.0 + np.exp((r - front) / 0.01))


@pytest.mark.parametrize("nu", [1.0, 2.0 / 3.0])
def test_developed_state_step_at_1024(engine, oracle_lib, nu):
    """nu = 1: the benchmark's five-point operator; nu = 2/3: the weighted nine-point operator of
    the reference's example .cfg files."""
    import torch
    E = engine
    N = 1024
    P = E.default_params(N, N, stype=E.PARALLEL, x_ub=2 ** 0.5, y_ub=2 ** 0.5, hmtype=E.MUSCL, diffusion=1,
                         alpha_l=1e-3, alpha_t=1e-4, Dm=1e-6, eps=1e-10, para_eps=1e-10, max_cycles=200, nu=nu)
    OP = oparams(P)
    q = source(OP)
    c0 = fingered(N, 7)
    cg = cell_ghost(OP, c0)
    ctx = E.Context(P)
    ctx.set_source(dev(q))
    # pressure: residual under the oracle's assembled system
    p = torch.zeros((N, N), dtype=torch.float64, device="cuda")
    cyc, rr, _ = ctx.pressure_solve(dev(c0), p, 1e-10)
    A, b = np.zeros(N * N * 9), np.zeros(N * N)
    oracle_lib.or_pressure_matrix(C.byref(OP), O.ptr(cg), O.ptr(A))
    oracle_lib.or_pressure_rhs(C.byref(OP), O.ptr(q), O.ptr(b))
    rr_or = oracle_lib.or_relres9(C.byref(OP), O.ptr(A), O.ptr(host(p).ravel().copy()), O.ptr(b))
    assert rr <= 1e-10 and rr_or <= 2e-10, (rr, rr_or)
    # the oracle's multigrid, continued from the GPU solution to 1e-12 (a two-well right-hand side
    # floors the relative residual of any FP64 solve near 1e-12 at this size)
    kappa_over_dA = A[(1 * N + 1) * 9]
    pin_value = b[1 * N + 1] / kappa_over_dA
    An = np.zeros_like(A)
    oracle_lib.or_pressure_matrix_neumann(C.byref(OP), O.ptr(cg), O.ptr(An))
    x = host(p).ravel().copy()
    cyc_o, rr_o = C.c_int(), C.c_double()
    assert oracle_lib.or_mg_solve(C.byref(OP), O.ptr(An), O.ptr(b), O.ptr(x), 2e-12, 200, C.byref(cyc_o),
                                  C.byref(rr_o), 1, 1, pin_value) == 0, (cyc_o.value, rr_o.value)
    del An
    err_p = rel_err(host(p).ravel(), x)
    assert err_p <= 1e-7, err_p  # a 1e-10 solve against a 2e-12 one
    # velocities, CFL step, split advection and a CN half step on the same pressure
    po = cell_ghost(OP, x.reshape(N, N))
    vo = np.zeros(O.vel_shape(OP))
    oracle_lib.or_calc_velocities(C.byref(OP), O.ptr(po.copy()), O.ptr(vo), O.ptr(cg))
    uo, vvo = vel_split(OP, vo)
    u = torch.zeros((N + 1, N), dtype=torch.float64, device="cuda")
    v = torch.zeros((N, N + 1), dtype=torch.float64, device="cuda")
    ctx.velocity(dev(O.interior(OP, po)), dev(c0), u, v)
    assert rel_err(host(u), uo) <= 1e-13 and rel_err(host(v), vvo) <= 1e-13
    dt = oracle_lib.or_max_stable_dt(C.byref(OP), O.ptr(vo))
    assert abs(ctx.max_stable_dt(dev(uo), dev(vvo)) - dt) <= 1e-14 * dt
    # one split advection and one CN half step with those velocities
    ca = dev(c0)
    ctx.advect_split(ca, dev(uo), dev(vvo), dt, 1)
    co = cg.copy()
    pfs = C.c_int(1)
    oracle_lib.or_advect_split(C.byref(OP), O.ptr(co), O.ptr(vo), dt, C.byref(pfs))
    assert rel_err(host(ca), O.interior(OP, co)) <= 1e-13
    cc = dev(c0)
    ctx.dispersion_cn(cc, dev(uo), dev(vvo), 0.5 * dt, 1e-13)
    cn = cg.copy()
    assert oracle_lib.or_cn_solve(C.byref(OP), O.ptr(cn), O.ptr(vo), 0.5 * dt, 1, 1e-13, None, None) == 0
    assert rel_err(host(cc), O.interior(OP, cn)) <= 1e-11
    ctx.close()
    # the whole step from the developed state: engine (graph) against the oracle.  Both solve the
    # pressure to 2e-12 (five-point) or 1e-11 (nine-point): about 1e-12 is the smallest relative
    # residual FP64 reaches on this state with the five-point operator (the rounding of A x beside
    # the wells), somewhat more with the nine-point one, and a solve below it stalls at max_cycles.
    tol_step = 2e-12 if nu == 1.0 else 1e-11
    P2 = E.default_params(N, N, stype=E.PARALLEL, x_ub=2 ** 0.5, y_ub=2 ** 0.5, hmtype=E.MUSCL, diffusion=1,
                          alpha_l=1e-3, alpha_t=1e-4, Dm=1e-6, eps=tol_step, para_eps=1e-12, max_cycles=200, nu=nu)
    ctx = E.Context(P2)
    ctx.upload(cg, q, ghost=2)
    ctx.set_time(0.0)
    info = ctx.step()
    OP2 = oparams(P2)
    c, pp, vv = cg.copy(), np.zeros(O.scalar_shape(OP2)), np.zeros(O.vel_shape(OP2))
    S = O.State()
    S.prev_first_sweep = 1
    tidx = C.c_int(0)
    assert oracle_lib.or_impes_step(C.byref(OP2), C.byref(S), O.ptr(c), O.ptr(pp), O.ptr(vv), O.ptr(q), None, 0,
                                    C.byref(tidx), 1, tol_step) == 0
    ch, ph = np.zeros_like(c), np.zeros_like(pp)
    ctx.download(ch, ph, None, ghost=2)
    err_c = rel_err(O.interior(OP2, ch), O.interior(OP2, c))
    err_pp = rel_err(O.interior(OP2, ph), O.interior(OP2, pp))
    print(f"1024^2 developed state, nu {nu:.4g}: pressure {err_p:.2e} against the oracle's multigrid ({cyc_o.value} further "
          f"cycles); one whole step: dt {abs(info.dt - S.dt) / S.dt:.2e}, c {err_c:.2e}, p {err_pp:.2e}")
    assert abs(info.dt - S.dt) <= 1e-8 * S.dt
    assert err_c <= 1e-9 and err_pp <= 1e-8, (err_c, err_pp)
    ctx.close()


@pytest.mark.parametrize("scheme", [0, 1, 2, 3])  # upwind, WAF split, WAF, CTU (MUSCL: the test above)
@pytest.mark.parametrize("mode", [4, 1])  # symmetric-parallel, x first
def test_transport_schemes_at_1024(engine, oracle_lib, scheme, mode):
    """The other transport schemes at the benchmark's size: one advection step of the developed
    fingered state with the Darcy velocities of a smooth pressure (a consistent field), each
    sweep order, against the oracle to 1e-13."""
    E = engine
    N = 1024
    P = E.default_params(N, N, stype=E.PARALLEL, x_ub=2 ** 0.5, y_ub=2 ** 0.5, hmtype=scheme, dim_splitting=mode,
                         porosity=0.7)
    OP = oparams(P)
    c0 = fingered(N, 11)
    cg = cell_ghost(OP, c0)
    p = 0.05 * grf(N, 48, 12)
    vg = np.zeros(O.vel_shape(OP))
    oracle_lib.or_calc_velocities(C.byref(OP), O.ptr(cell_ghost(OP, p)), O.ptr(vg), O.ptr(cg))
    u, v = vel_split(OP, vg)
    dt = 0.9 * oracle_lib.or_max_stable_advection_dt(C.byref(OP), O.ptr(vg)) * OP.porosity
    ctx = E.Context(P)
    for pfs0 in (0, 1):
        co = cg.copy()
        pfs = C.c_int(pfs0)
        oracle_lib.or_advect_split(C.byref(OP), O.ptr(co), O.ptr(vg), dt, C.byref(pfs))
        dc = dev(c0)
        assert ctx.advect_split(dc, dev(u), dev(v), dt, pfs0) == pfs.value
        err = rel_err(host(dc), O.interior(OP, co))
        assert err <= 1e-13, (pfs0, err)
    ctx.close()


def test_reference_cpu_case_128_to_0p3_pore_volumes(engine, oracle_lib):
    """The small CPU-runnable case: 128^2 diagonal, one-cell wells, upwind, porosity 0.2, M = 41, CFL 0.5,
    pressure to 1e-10, to t = 0.06 = 0.3 phi |Omega| / I.  The reference's time step ignores the
    porosity its flux divides by (unstable at phi = 0.2); the engine scales it by phi
    (gb300.cfl_porosity), and the oracle gets the same step through cfl * phi."""
    E = engine
    N = 128
    P = E.default_params(N, N, stype=E.DIAGONAL, hmtype=E.UPWINDSPLIT, nu=1.0, porosity=0.2, cfl=0.5,
                         cfl_porosity=1, mu_res=41.0, mu_inj=1.0, eps=1e-10, para_eps=1e-10, max_cycles=200)
    OP = oparams(P, cfl=0.5 * 0.2)
    q = source(OP)
    ctx = E.Context(P)
    ctx.upload(cell_ghost(OP, np.zeros((N, N))), q, ghost=2)
    ctx.set_time(0.0)
    c = cell_ghost(OP, np.zeros((N, N)))
    p, vv = np.zeros(O.scalar_shape(OP)), np.zeros(O.vel_shape(OP))
    S = O.State()
    S.prev_first_sweep = 1
    t_end = 0.06
    times = np.array([t_end])
    tidx = C.c_int(0)
    worst_dt = mass_e = mass_o = 0.0
    n = 0
    while S.t < t_end:
        assert oracle_lib.or_impes_step(C.byref(OP), C.byref(S), O.ptr(c), O.ptr(p), O.ptr(vv), O.ptr(q),
                                        O.ptr(times), 1, C.byref(tidx), 1, 1e-11) == 0
        info = ctx.step(t_end)
        n += 1
        worst_dt = max(worst_dt, abs(info.dt - S.dt) / S.dt)
        mass_e, mass_o = max(mass_e, info.mass_err), max(mass_o, S.mass_err)
    assert abs(info.t - t_end) <= 1e-15 and abs(S.t - t_end) <= 1e-15
    rel_out = abs(info.total_outflux - S.total_outflux) / S.total_outflux
    ch = np.zeros_like(c)
    ctx.download(ch, None, None, ghost=2)
    err_c = rel_err(O.interior(OP, ch), O.interior(OP, c))
    print(f"{n} steps: worst dt deviation {worst_dt:.2e}, produced volume rel {rel_out:.2e}, c {err_c:.2e}, "
          f"mass error engine {mass_e:.1e} oracle {mass_o:.1e}")
    assert n > 100
    # measured (3944 steps): dt 6.7e-8 (the 1e-10 pressure tolerance moves the peak velocity),
    # produced volume 3.7e-10, c 3.3e-9, mass errors 4e-15 / 2e-14
    assert worst_dt <= 1e-6 and rel_out <= 1e-8 and mass_e <= 1e-10 and mass_o <= 1e-10
    assert err_c <= 1e-7, err_c  # before breakthrough the upwind front is stable: fields still agree
    ctx.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_heterogeneous_4096_solve_against_oracle_multigrid(engine, oracle_lib, prec):
    """The mixed-precision pressure case at full size (4096^2): the FP64 and the FP32-in-FP64-refinement
    solves reach 1e-10 under the oracle's assembled (reference) system, and their solutions
    agree with the oracle's FP64 multigrid solution (warm-started from the GPU solution and run
    to 4e-11, where FP64 round-off floors the residual of the two-well problem at this size)
    within the error a 1e-10 solve allows."""
    import torch
    E = engine
    N = 4096
    c0 = 1.0 / (1.0 + np.exp(-4.0 * grf(N, 32, 11)))
    K = np.exp(1.0 * grf(N, 16, 12))
    P = E.default_params(N, N, stype=E.DIAGONAL, nu=1.0, mu_res=41.0, mu_inj=1.0, eps=1e-10, max_cycles=300,
                         precision=prec)
    OP = oparams(P, K11=K, K22=K)
    q = source(OP)
    ctx = E.Context(P)
    ctx.set_source(dev(q))
    Kd = dev(K)
    ctx.set_permeability(Kd, Kd)
    p = torch.zeros((N, N), dtype=torch.float64, device="cuda")
    cyc, rr, _ = ctx.pressure_solve(dev(c0), p, 1e-10)
    ph = host(p)
    ctx.close()
    del Kd
    torch.cuda.empty_cache()
    cg = cell_ghost(OP, c0)
    A, b = np.zeros(N * N * 9), np.zeros(N * N)
    oracle_lib.or_pressure_matrix(C.byref(OP), O.ptr(cg), O.ptr(A))
    oracle_lib.or_pressure_rhs(C.byref(OP), O.ptr(q), O.ptr(b))
    rr_or = oracle_lib.or_relres9(C.byref(OP), O.ptr(A), O.ptr(ph.ravel().copy()), O.ptr(b))
    assert rr <= 1e-10 and rr_or <= 2e-10, (rr, rr_or)
    # the oracle's multigrid to 1e-13 from the GPU solution
    kappa_over_dA = A[(1 * N + 1) * 9]
    pin_value = b[1 * N + 1] / kappa_over_dA
    oracle_lib.or_pressure_matrix_neumann(C.byref(OP), O.ptr(cg), O.ptr(A))
    x = ph.ravel().copy()
    cyc_o, rr_o = C.c_int(), C.c_double()
    # at 4096^2 the two-well right-hand side floors any FP64 solve's relative residual near 3.5e-11
    rc = oracle_lib.or_mg_solve(C.byref(OP), O.ptr(A), O.ptr(b), O.ptr(x), 4e-11, 100, C.byref(cyc_o),
                                C.byref(rr_o), 1, 1, pin_value)
    assert rc == 0, (cyc_o.value, rr_o.value)
    err = rel_err(ph.ravel(), x)
    print(f"{'mixed' if prec else 'fp64'} 4096^2: {cyc} iterations, relres {rr:.2e} (oracle matrix {rr_or:.2e}); "
          f"vs oracle MG at {rr_o.value:.1e} ({cyc_o.value} further cycles): {err:.2e}")
    assert err <= 1e-6, err
