"""The oracle against fixtures written by the reference itself (CPU; always runs).

tests/golden/ref_ops.npz, ref_runs/ and ref_advection.npz hold outputs of the reference's own
code (src/*.cpp compiled unchanged in oracle/_ref by tests/golden/make_ref_golden.py).  On the
same inputs the oracle must reproduce every assembled coefficient, flux, sweep, source, ghost
fill and diagnostic bit for bit; direct solves agree to rounding.  This pins the oracle where
no reference checkout is at hand.  The engine parses each fixture .cfg into the same
parameters the reference parsed.
"""
import ast
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLD, "ref_ops.npz"))


def _case(gold, name):
    kw = ast.literal_eval(str(gold[f"{name}/params"]))
    return O.make_params(**kw), (lambda k: gold[f"{name}/{k}"])


@pytest.mark.parametrize("name", ["diag", "par", "horiz"])
def test_oracle_reproduces_reference_operations(oracle_lib, gold, name):
    L = oracle_lib
    P, g = _case(gold, name)
    pP = C.byref(P)
    n = P.N1 * P.N2
    c, v, q = g("c"), g("v"), g("q")
    qo = np.zeros(n)
    L.or_init_source(pP, O.ptr(qo), float(g("q_t")) if P.stype == O.HORIZONTAL else 0.0)
    assert np.array_equal(qo, q)
    A = np.zeros(n * 9)
    L.or_pressure_matrix(pP, O.ptr(c), O.ptr(A))
    assert np.array_equal(A, g("A9"))
    b = np.zeros(n)
    L.or_pressure_rhs(pP, O.ptr(q), O.ptr(b))
    assert np.array_equal(b, g("b"))
    lx, ly = np.zeros((P.N1 + 1) * P.N2), np.zeros(P.N1 * (P.N2 + 1))
    L.or_face_mobility(pP, O.ptr(c), O.ptr(lx), O.ptr(ly))
    assert np.array_equal(lx, g("lamx")) and np.array_equal(ly, g("lamy"))
    p = np.zeros(O.scalar_shape(P))
    assert L.or_pressure_solve(pP, O.ptr(c), O.ptr(q), O.ptr(p), 0, 1e-14, None, None) == 0
    pr = O.interior(P, g("p"))
    assert np.abs(O.interior(P, p) - pr).max() <= 1e-11 * np.abs(pr).max()
    p = g("p").copy()
    vp = np.zeros(O.vel_shape(P))
    L.or_calc_velocities(pP, O.ptr(p), O.ptr(vp), O.ptr(c))
    assert np.array_equal(vp, g("v_of_p"))
    assert L.or_max_stable_dt(pP, O.ptr(vp)) == float(g("dt"))
    dt = float(g("dt_used"))
    ct = c.copy()
    assert L.or_tr_integrate(pP, O.ptr(ct), O.ptr(q), dt) == float(g("tr_outflux"))
    assert np.array_equal(ct, g("tr_c"))
    gg = P.g
    for scheme, tag in ((O.MUSCL, "muscl"), (O.UPWINDSPLIT, "upwind")):
        Ps = O.make_params(**{**ast.literal_eval(str(gold[f"{name}/params"])), "hmtype": scheme})
        F, G = np.zeros((P.N1 + 1) * (P.N2 + 2 * gg)), np.zeros((P.N1 + 2 * gg) * (P.N2 + 1))
        L.or_flux_F(C.byref(Ps), O.ptr(F), O.ptr(c), O.ptr(v), dt)
        L.or_flux_G(C.byref(Ps), O.ptr(G), O.ptr(c), O.ptr(v), dt)
        assert np.array_equal(F, g(f"F_{tag}")) and np.array_equal(G, g(f"G_{tag}"))
        ca = c.copy()
        s = C.c_int(1)
        L.or_advect_split(C.byref(Ps), O.ptr(ca), O.ptr(vp), dt, C.byref(s))
        assert np.array_equal(ca, g(f"advect_{tag}"))
    An = np.zeros(n * 9)
    L.or_cn_matrix(pP, O.ptr(vp), 0.5 * dt, O.ptr(An))
    assert np.array_equal(An, g("cn_A9"))
    bn = np.zeros(n)
    L.or_cn_rhs(pP, O.ptr(c), O.ptr(vp), 0.5 * dt, O.ptr(bn))
    assert np.array_equal(bn, g("cn_b"))
    cc = c.copy()
    assert L.or_cn_solve(pP, O.ptr(cc), O.ptr(vp), 0.5 * dt, 0, 1e-14, None, None) == 0
    assert np.abs(cc - g("cn_c")).max() <= 1e-13
    ch = c.copy()
    s, o = C.c_int(1), C.c_double(0.0)
    L.or_hyperbolic_solve(pP, O.ptr(ch), O.ptr(vp), O.ptr(q), dt, C.byref(s), C.byref(o), 0)
    assert np.abs(ch - g("hyp_c")).max() <= 1e-13 and abs(o.value - float(g("hyp_outflux"))) <= 1e-14
    if P.stype != O.HORIZONTAL:
        assert L.or_total_mass(pP, O.ptr(c)) == float(g("total_mass"))
        assert L.or_mass_error(pP, O.ptr(c), 0.37, 0.11) == float(g("mass_error"))
        assert L.or_divergence_error(pP, O.ptr(vp), O.ptr(q)) == float(g("div_error"))
        assert L.or_velocity_boundary_error(pP, O.ptr(vp)) == float(g("vel_error"))


def test_oracle_reproduces_reference_convergence_errors(oracle_lib):
    from test_oracle import _advection_error
    gold = np.load(os.path.join(GOLD, "ref_advection.npz"))
    for k, N in enumerate([50, 100]):  # the two cheap levels, error for error
        assert np.log(_advection_error(oracle_lib, N, (-1.0, 1.0))) == gold["lognorm"][k]
    assert abs(np.polyfit(gold["logdx"], gold["lognorm"], 1)[0] - 1.86712) < 5e-5


@pytest.mark.parametrize("case", sorted(os.listdir(os.path.join(GOLD, "ref_runs"))))
def test_engine_parses_the_fixture_cfgs_like_the_reference(case):
    import impec2d_gb300 as E
    from impec2d_gb300 import build as B
    B.build()
    P, t0, t1 = E.load_cfg(os.path.join(GOLD, "ref_runs", case, "case.cfg"))
    text = open(os.path.join(GOLD, "ref_runs", case, "case.cfg")).read()
    assert f"x_cells = {P.N1};" in text and f"y_cells = {P.N2};" in text and t0 == 0.0 and t1 > 0
    assert P.hmtype == E.MUSCL and P.eps == 1e-12


@pytest.mark.parametrize("case", sorted(os.listdir(os.path.join(GOLD, "ref_runs"))))
def test_engine_cfg_sources_equal_the_reference(oracle_lib, case):
    """The engine's own well sources of each fixture .cfg (impec_cfg_source: one-cell and circle
    wells, ExactVolFracCircle) equal the reference's InitializeSource (src/Impec2DSolver.cpp:
    241-280, src/Util.cpp:444-586) bit for bit, through the oracle that reproduces it."""
    import impec2d_gb300 as E
    from impec2d_gb300 import build as B
    B.build()
    path = os.path.join(GOLD, "ref_runs", case, "case.cfg")
    P, _, _ = E.load_cfg(path)
    q = E.cfg_source(path, P.N1, P.N2)
    text = open(path).read()
    well = O.CIRCULAR if '"circle"' in text else O.ONECELL
    rc = float(text.split("well_rc = ")[1].split(";")[0])
    OP = O.make_params(N1=P.N1, N2=P.N2, x_lb=P.x_lb, x_ub=P.x_ub, y_lb=P.y_lb, y_ub=P.y_ub, stype=P.stype,
                       I=P.I, well_profile=well, well_rc=rc)
    qo = np.zeros(P.N1 * P.N2)
    oracle_lib.or_init_source(C.byref(OP), O.ptr(qo), 0.0)
    assert np.array_equal(q, qo)
