"""The oracle against the reference itself, run here (CPU; skipped without a reference checkout).

oracle/_ref is the reference's own src/*.cpp compiled unchanged (recipe oracle/Makefile.ref)
against the stand-ins in oracle/refshim: a Blitz++ subset, libconfig++, one-rank MPI, and
HYPRE reduced to a recorded system with one direct solve.  Every operation that is reference
code -- assembly, fluxes, sweeps, sources, ghost fills, velocities, Peaceman tensors, the
Crank-Nicolson system, diagnostics -- must agree with the oracle BIT FOR BIT on seeded inputs.
Solves agree to rounding (both are direct), and whole runs to the accumulated rounding of
those solves.  IMPEC2D_REFERENCE names the checkout the recipe compiles.
"""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import oracle as O
from oracle import ref as R

pytestmark = pytest.mark.skipif(not R.available(), reason="no reference checkout to build oracle/_ref from")


def _params(**kw):
    d = dict(N1=24, N2=20, stype=O.DIAGONAL, hmtype=O.MUSCL, porosity=0.7, mu_res=41.0, nu=1.0)
    if kw.get("stype") == O.PARALLEL:
        d.update(N1=22, N2=22, x_ub=1.4142135623730951, y_ub=1.4142135623730951)
    d.update(kw)
    return O.make_params(**d)


def _fields(P, seed):
    rng = np.random.default_rng(seed)
    c = np.zeros(O.scalar_shape(P))
    c[P.g:P.g + P.N1, P.g:P.g + P.N2] = rng.uniform(0.0, 1.0, (P.N1, P.N2))
    O.lib().or_fill_scalar_neumann(C.byref(P), O.ptr(c))
    v = rng.uniform(-1.0, 1.0, O.vel_shape(P))
    v[np.abs(v) < 1e-3] = 1e-3  # the reference's Peaceman tensor divides by |u|
    O.lib().or_fill_velocity_neumann(C.byref(P), O.ptr(v))
    return c, v


def _same(a, b):
    assert a.shape == b.shape
    assert np.array_equal(a, b), f"max |diff| {np.abs(a - b).max():.3e}"


def test_ghost_fills():
    P = _params()
    rng = np.random.default_rng(0)
    with R.Case(P) as h:
        for fn in ("fill_scalar_neumann", "fill_scalar_periodic"):
            a = rng.uniform(size=O.scalar_shape(P))
            b = a.copy()
            getattr(h, fn)(a)
            getattr(O.lib(), "or_" + fn)(C.byref(P), O.ptr(b))
            _same(a, b)
        a = rng.uniform(size=O.vel_shape(P))
        b = a.copy()
        h.fill_velocity_neumann(a)
        O.lib().or_fill_velocity_neumann(C.byref(P), O.ptr(b))
        _same(a, b)


@pytest.mark.parametrize("avgproc", [O.HARMONIC, O.MEANCONC])
def test_mobility_and_face_values(avgproc):
    P = _params(avgproc=avgproc)
    c, _ = _fields(P, 1)
    with R.Case(P) as h:
        for x in (0.0, 0.3, 0.77, 1.0):
            assert h.mu(x) == O.lib().or_mu(C.byref(P), x)
        lx, ly = np.zeros((P.N1 + 1) * P.N2), np.zeros(P.N1 * (P.N2 + 1))
        ox, oy = lx.copy(), ly.copy()
        h.face_mobility(c, lx, ly)
        O.lib().or_face_mobility(C.byref(P), O.ptr(c), O.ptr(ox), O.ptr(oy))
        _same(lx, ox)
        _same(ly, oy)


@pytest.mark.parametrize("stype,nu,avgproc", [(O.DIAGONAL, 1.0, O.HARMONIC), (O.DIAGONAL, 2 / 3, O.HARMONIC),
                                              (O.PARALLEL, 1.0, O.HARMONIC), (O.PARALLEL, 2 / 3, O.MEANCONC),
                                              (O.HORIZONTAL, 1.0, O.HARMONIC), (O.HORIZONTAL, 2 / 3, O.HARMONIC)])
def test_pressure_system(stype, nu, avgproc):
    """SetMatrixCoefficients_Elliptic and SetRHS_Elliptic (src/MGSolver.cpp:268-590): every
    coefficient, Neumann folds and Dirichlet rows included."""
    P = _params(stype=stype, nu=nu, avgproc=avgproc)
    c, _ = _fields(P, 2)
    with R.Case(P) as h:
        n = P.N1 * P.N2
        A, B = np.zeros(n * 9), np.zeros(n * 9)
        h.pressure_matrix(c, A)
        O.lib().or_pressure_matrix(C.byref(P), O.ptr(c), O.ptr(B))
        _same(A, B)
        q = h.source()
        b1, b2 = np.zeros(n), np.zeros(n)
        h.pressure_rhs(q, b1)
        O.lib().or_pressure_rhs(C.byref(P), O.ptr(q), O.ptr(b2))
        _same(b1, b2)


@pytest.mark.parametrize("stype,nu", [(O.DIAGONAL, 1.0), (O.DIAGONAL, 2 / 3), (O.PARALLEL, 2 / 3), (O.HORIZONTAL, 1.0)])
def test_pressure_solve_and_velocities(stype, nu):
    """EllipticSolver::Solve (both direct: agreement to rounding) and CalcVelocities on the same
    pressure (bit for bit, ghost fills of p and v included)."""
    P = _params(stype=stype, nu=nu)
    c, _ = _fields(P, 3)
    with R.Case(P) as h:
        q = h.source()
        pr, po = np.zeros(O.scalar_shape(P)), np.zeros(O.scalar_shape(P))
        assert h.pressure_solve(c.copy(), q, pr) == 0
        assert O.lib().or_pressure_solve(C.byref(P), O.ptr(c), O.ptr(q), O.ptr(po), 0, 1e-14, None, None) == 0
        ip, io = O.interior(P, pr), O.interior(P, po)
        assert np.abs(ip - io).max() <= 1e-11 * np.abs(io).max()
        vr, vo = np.zeros(O.vel_shape(P)), np.zeros(O.vel_shape(P))
        p1, p2 = pr.copy(), pr.copy()
        h.calc_velocities(p1, vr, c)
        O.lib().or_calc_velocities(C.byref(P), O.ptr(p2), O.ptr(vo), O.ptr(c))
        _same(p1, p2)
        _same(vr, vo)


@pytest.mark.parametrize("is_test,diffusion", [(0, 0), (0, 1), (1, 0)])
def test_max_stable_timestep(is_test, diffusion):
    P = _params(is_test=is_test, diffusion=diffusion, alpha_l=0.3, alpha_t=0.05)
    c, v = _fields(P, 4)
    with R.Case(P) as h:
        assert h.max_stable_dt(c, v) == O.lib().or_max_stable_dt(C.byref(P), O.ptr(v))


@pytest.mark.parametrize("stype,well", [(O.DIAGONAL, O.ONECELL), (O.PARALLEL, O.ONECELL),
                                        (O.DIAGONAL, O.CIRCULAR), (O.PARALLEL, O.CIRCULAR)])
def test_sources(stype, well):
    """InitializeSource (src/Impec2DSolver.cpp:241-280): one-cell and circle wells
    (ExactVolFracCircle, src/Util.cpp:444-559), both orientations."""
    P = _params(stype=stype, well_profile=well, well_rc=0.15, I=1.3)
    with R.Case(P) as h:
        q = h.source()
        qo = np.zeros_like(q)
        O.lib().or_init_source(C.byref(P), O.ptr(qo), 0.0)
        _same(q, qo)
        assert (q != 0).sum() >= 2
    for args in [(0.1, 0.2, 0.3, 0.05, 0.05), (0.0, 0.0, 0.07, 0.1, 0.1), (0.31, 0.02, 0.2, 0.01, 0.03)]:
        assert R.lib().ref_exact_vol_frac_circle(*args) == O.lib().or_exact_vol_frac_circle(*args)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_horizontal_front_source(mode):
    """InitHorizontalFront (src/Util.cpp:607-639) at several times, pulsing / linear / constant."""
    P = _params(stype=O.HORIZONTAL, inj_mode=mode, q_freq=20.0, q_high_multiple=50.0, well_width=0.1)
    with R.Case(P) as h:
        for t in (0.0, 0.013, 0.05, 0.21):
            q, qo = np.zeros(P.N1 * P.N2), np.zeros(P.N1 * P.N2)
            h.horizontal_source(q, t)
            O.lib().or_init_source(C.byref(P), O.ptr(qo), t)
            _same(q, qo)


def test_tr_integrator():
    P = _params(well_profile=O.CIRCULAR, well_rc=0.2)
    c, _ = _fields(P, 5)
    with R.Case(P) as h:
        q = h.source()
        c1, c2 = c.copy(), c.copy()
        out1 = h.tr_integrate(c1, q, 3e-3)
        out2 = O.lib().or_tr_integrate(C.byref(P), O.ptr(c2), O.ptr(q), 3e-3)
        _same(c1, c2)
        assert out1 == out2


@pytest.mark.parametrize("scheme", [O.MUSCL, O.UPWINDSPLIT])
def test_intercell_fluxes(scheme):
    P = _params(hmtype=scheme)
    c, v = _fields(P, 6)
    with R.Case(P) as h:
        g = P.g
        F, Fo = np.zeros((P.N1 + 1) * (P.N2 + 2 * g)), np.zeros((P.N1 + 1) * (P.N2 + 2 * g))
        h.flux_F(scheme, F, c, v, 2e-3)
        O.lib().or_flux_F(C.byref(P), O.ptr(Fo), O.ptr(c), O.ptr(v), 2e-3)
        _same(F, Fo)
        G, Go = np.zeros((P.N1 + 2 * g) * (P.N2 + 1)), np.zeros((P.N1 + 2 * g) * (P.N2 + 1))
        h.flux_G(scheme, G, c, v, 2e-3)
        O.lib().or_flux_G(C.byref(P), O.ptr(Go), O.ptr(c), O.ptr(v), 2e-3)
        _same(G, Go)


@pytest.mark.parametrize("scheme", [O.MUSCL, O.UPWINDSPLIT])
@pytest.mark.parametrize("split", [O.ALTERNATING, O.X_FIRST, O.Y_FIRST, O.STRANG, O.SYMMETRIC_PARALLEL])
@pytest.mark.parametrize("is_test", [0, 1])
def test_advect_split(scheme, split, is_test):
    """AdvectSplit in all five modes (src/HyperbolicSplitSolver.cpp:51-159), three calls in a row
    (the alternating mode's state carries over), Neumann and periodic boundaries."""
    P = _params(hmtype=scheme, dim_splitting=split, is_test=is_test)
    c, v = _fields(P, 7)
    if is_test:
        O.lib().or_fill_scalar_periodic(C.byref(P), O.ptr(c))
    with R.Case(P) as h:
        c1, c2 = c.copy(), c.copy()
        s1, s2 = C.c_int(1), C.c_int(1)
        for _ in range(3):
            h.advect_split(scheme, c1, v, 1.5e-3, C.byref(s1))
            O.lib().or_advect_split(C.byref(P), O.ptr(c2), O.ptr(v), 1.5e-3, C.byref(s2))
            _same(c1, c2)
            assert s1.value == s2.value


@pytest.mark.parametrize("stype", [O.DIAGONAL, O.HORIZONTAL])
def test_peaceman_and_crank_nicolson_system(stype):
    """SetupDiffusionTensorF/G and the CN matrix and right-hand side (src/MGSolver.cpp:846-1371)."""
    P = _params(stype=stype, diffusion=1, alpha_l=0.4, alpha_t=0.07)
    c, v = _fields(P, 8)
    with R.Case(P) as h:
        for i in range(0, P.N1 + 1, 5):
            for j in range(0, P.N2, 4):
                a, b, x, y = C.c_double(), C.c_double(), C.c_double(), C.c_double()
                h.peaceman_F(v, i, j, C.byref(a), C.byref(b))
                O.lib().or_peaceman_F(C.byref(P), O.ptr(v), i, j, C.byref(x), C.byref(y))
                assert (a.value, b.value) == (x.value, y.value)
                h.peaceman_G(v, min(i, P.N1 - 1), j, C.byref(a), C.byref(b))
                O.lib().or_peaceman_G(C.byref(P), O.ptr(v), min(i, P.N1 - 1), j, C.byref(x), C.byref(y))
                assert (a.value, b.value) == (x.value, y.value)
        n = P.N1 * P.N2
        A, B = np.zeros(n * 9), np.zeros(n * 9)
        h.cn_matrix(v, 4e-3, A)
        O.lib().or_cn_matrix(C.byref(P), O.ptr(v), 4e-3, O.ptr(B))
        _same(A, B)
        b1, b2 = np.zeros(n), np.zeros(n)
        h.cn_rhs(c, v, 4e-3, b1)
        O.lib().or_cn_rhs(C.byref(P), O.ptr(c), O.ptr(v), 4e-3, O.ptr(b2))
        _same(b1, b2)
        c1, c2 = c.copy(), c.copy()
        assert h.cn_solve(c1, v, 4e-3) == 0
        assert O.lib().or_cn_solve(C.byref(P), O.ptr(c2), O.ptr(v), 4e-3, 0, 1e-14, None, None) == 0
        assert np.abs(c1 - c2).max() <= 1e-13


@pytest.mark.parametrize("diffusion", [0, 1])
def test_hyperbolic_split_solve(diffusion):
    """HyperbolicSplitSolver::Solve (src/HyperbolicSplitSolver.cpp:162-198): bit for bit without
    dispersion; with it the two Crank-Nicolson solves agree to rounding."""
    P = _params(diffusion=diffusion, alpha_l=0.3, alpha_t=0.03, well_profile=O.CIRCULAR, well_rc=0.2)
    c, v = _fields(P, 9)
    with R.Case(P) as h:
        q = h.source()
        c1, c2 = c.copy(), c.copy()
        s1, s2 = C.c_int(1), C.c_int(1)
        o1, o2 = C.c_double(0.25), C.c_double(0.25)
        for _ in range(2):
            assert h.hyperbolic_solve(O.MUSCL, c1, v, q, 1e-3, C.byref(s1), C.byref(o1)) == 0
            O.lib().or_hyperbolic_solve(C.byref(P), O.ptr(c2), O.ptr(v), O.ptr(q), 1e-3, C.byref(s2), C.byref(o2), 0)
        if diffusion:
            assert np.abs(c1 - c2).max() <= 1e-13 and abs(o1.value - o2.value) <= 1e-14
        else:
            _same(c1, c2)
            assert o1.value == o2.value


def test_diagnostics():
    """GetTotalMass, CalculateMassError, CalculateDivergenceError, CalculateVelocityBoundaryError
    (src/Impec2DSolver.cpp:530-620)."""
    for stype in (O.DIAGONAL, O.PARALLEL):
        P = _params(stype=stype)
        c, v = _fields(P, 10)
        with R.Case(P) as h:
            q = h.source()
            assert h.total_mass(c) == O.lib().or_total_mass(C.byref(P), O.ptr(c))
            assert h.mass_error(c, 0.37, 0.11) == O.lib().or_mass_error(C.byref(P), O.ptr(c), 0.37, 0.11)
            assert h.divergence_error(v) == O.lib().or_divergence_error(C.byref(P), O.ptr(v), O.ptr(q))
            assert h.velocity_boundary_error(v) == O.lib().or_velocity_boundary_error(C.byref(P), O.ptr(v))


@pytest.mark.parametrize("case", ["diagonal_muscl", "parallel_muscl_cn"])
def test_whole_run_matches_the_oracle_loop(case):
    """Impec2DSolver::Solve (src/Impec2DSolver.cpp:293-466), the reference's own loop, against the
    oracle's step loop with direct solves: the fields after every step differ only by the
    rounding of the solves.  The reference's loop always advects with MUSCL
    (src/Impec2DSolver.cpp:132, whatever hyper_method says), so both run MUSCL here."""
    if case == "diagonal_muscl":
        P = _params(N1=20, N2=20, hmtype=O.MUSCL, porosity=1.0, tfinal=0.05, eps=1e-14)
    else:
        P = _params(stype=O.PARALLEL, N1=20, N2=20, diffusion=1, alpha_l=0.05, alpha_t=0.005, tfinal=0.03,
                    eps=1e-14, para_eps=1e-14)
    with R.Case(P) as h:
        cr, pr, vr = np.zeros(O.scalar_shape(P)), np.zeros(O.scalar_shape(P)), np.zeros(O.vel_shape(P))
        steps = C.c_int(0)
        assert h.run(None, cr, pr, vr, C.byref(steps)) == 0
        q = h.source()
    c, p, v = np.zeros(O.scalar_shape(P)), np.zeros(O.scalar_shape(P)), np.zeros(O.vel_shape(P))
    S = O.State()
    S.prev_first_sweep = 1
    times = np.array([P.tfinal])
    tidx = C.c_int(0)
    n = 0
    while S.t < P.tfinal:
        assert O.lib().or_impes_step(C.byref(P), C.byref(S), O.ptr(c), O.ptr(p), O.ptr(v), O.ptr(q), O.ptr(times), 1,
                                     C.byref(tidx), 0, 1e-14) == 0
        n += 1
    assert n >= 5
    ci, cri = O.interior(P, c), O.interior(P, cr)
    assert np.abs(ci - cri).max() <= 1e-11, np.abs(ci - cri).max()
    assert np.abs(O.interior(P, p) - O.interior(P, pr)).max() <= 1e-10 * np.abs(O.interior(P, pr)).max()


def test_shipped_advection_convergence_case():
    """The reference's advection convergence test (examples/hyperbolic_test.cfg: MUSCL, sine, L1,
    CFL 0.95, 50^2 doubled over 4 levels, the shipped diagonal velocity) run through its own code:
    the oracle's errors are the same numbers, and the fitted order is 1.86712.  The value
    recorded in that file, 1.87621 (labelled y-advection), is not what the shipped code gives
    with either velocity (y-advection gives 1.94244), so it is kept as a loose anchor only."""
    from test_oracle import _advection_error
    d = tempfile.mkdtemp(prefix="impec_ref_adv_")
    P = O.make_params(N1=50, N2=50, stype=O.DIAGONAL, hmtype=O.MUSCL, porosity=1.0, cfl=0.95, is_test=1,
                      tstart=0.0, tfinal=1.0, dim_splitting=O.SYMMETRIC_PARALLEL)
    cfg = R.write_cfg(os.path.join(d, "t.cfg"), P, results_dir=d, test=dict(levels=4))
    lx, ln = np.zeros(4), np.zeros(4)
    assert R.lib().ref_advection_test(cfg.encode(), -1.0, 1.0, O.ptr(lx), O.ptr(ln)) == 0
    order = np.polyfit(lx, ln, 1)[0]
    assert abs(order - 1.86712) < 5e-5, order
    for k, N in enumerate([50, 100]):  # the two cheap levels, error for error
        assert np.log(_advection_error(O.lib(), N, (-1.0, 1.0))) == ln[k]
