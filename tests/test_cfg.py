"""The .cfg front end (libconfig subset, SimParams semantics of src/SimParams.cpp:45-468):
parses the reference's example files unchanged, reports missing keys as a status instead of
exiting, and maps the engine options."""
import glob
import os

import pytest

import impec2d_gb300 as E

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout, when one is at hand: IMPEC2D_REFERENCE names its root directory.
REF_EXAMPLES = os.path.join(os.environ.get("IMPEC2D_REFERENCE", ""), "examples") if os.environ.get("IMPEC2D_REFERENCE") else ""


@pytest.fixture(scope="module", autouse=True)
def _built():
    from impec2d_gb300 import build as B
    B.build()


def test_fixture_config1():
    P, t0, t1 = E.load_cfg(os.path.join(HERE, "golden", "quarter_five_spot_128_upwind.cfg"))
    assert (P.N1, P.N2) == (128, 128) and P.stype == E.DIAGONAL and P.hmtype == E.UPWINDSPLIT
    assert P.porosity == 0.2 and P.cfl == 0.5 and P.cfl_porosity == 1 and P.nu == 1.0
    assert (t0, t1) == (0.0, 0.06)
    q = E.cfg_source(os.path.join(HERE, "golden", "quarter_five_spot_128_upwind.cfg"), 128, 128)
    assert q[0] == pytest.approx(128 * 128) and q[-1] == pytest.approx(-128 * 128) and (q != 0).sum() == 2


def test_fixture_config2():
    P, t0, t1 = E.load_cfg(os.path.join(HERE, "golden", "parallel_1024_muscl_dispersion.cfg"))
    assert (P.N1, P.N2) == (1024, 1024) and P.stype == E.PARALLEL and P.hmtype == E.MUSCL
    assert P.diffusion == 1 and P.alpha_l == 1e-3 and P.alpha_t == 1e-4 and P.Dm == 1e-6
    assert P.eps == 1e-10 and P.precision == E.PREC_FP64 and P.bc == E.BC_NEUMANN


def test_fixture_horizontal_front():
    """source_type horizontal: injection over the first and production over the last
    round(well_width L / dx) rows (InitHorizontalFront, src/Util.cpp:607-639)."""
    path = os.path.join(HERE, "golden", "horizontal_pulsing_64x48.cfg")
    P, t0, t1 = E.load_cfg(path)
    assert (P.N1, P.N2) == (64, 48) and P.stype == E.HORIZONTAL and P.diffusion == 1
    q = E.cfg_source(path, 64, 48)
    rows = 3  # round(0.05 * 1 / (1 / 64))
    val = 1.0 / (48 * (1 / 64) * (1 / 48) * rows)
    assert q[:48 * rows] == pytest.approx(val) and q[-48 * rows:] == pytest.approx(-val)
    assert (q != 0).sum() == 2 * 48 * rows


@pytest.mark.gpu
def test_run_horizontal_pulsing_cfg():
    """The whole .cfg through the executable's entry point: Dirichlet rows in the pressure and
    CN systems and the pulsing rate updated every step."""
    path = os.path.join(HERE, "golden", "horizontal_pulsing_64x48.cfg")
    assert E.lib().impec_run_cfg(path.encode(), 1) == 0, E.last_error()
    rows = [list(map(float, l.split())) for l in open("/tmp/impec2d_horizontal/concentration.dat") if l.strip()]
    c = [r[2] for r in rows]
    assert len(c) == 64 * 48 and min(c) > -1e-6 and max(c) < 1.0 + 1e-6
    # after t = 0.004 the three injection rows hold about q t = 64 / 3 * 0.004 (less what has moved on)
    first = sum(c[:3 * 48]) / (3 * 48)
    rest = sum(c[10 * 48:]) / (54 * 48)
    assert 0.05 < first < 0.0854 and rest < 1e-3


@pytest.mark.skipif(not REF_EXAMPLES or not os.path.isdir(REF_EXAMPLES),
                    reason="IMPEC2D_REFERENCE does not name a reference checkout")
def test_reference_examples_parse_unchanged():
    files = sorted(glob.glob(os.path.join(REF_EXAMPLES, "*.cfg")))
    assert len(files) == 5
    for f in files:
        P, t0, t1 = E.load_cfg(f)
        assert P.N1 >= 2 and P.N2 >= 2 and t1 > t0
        name = os.path.basename(f)
        if name == "parallel.cfg":
            assert (P.N1, P.stype, P.nu) == (141, E.PARALLEL, pytest.approx(2 / 3))
        if name == "diagonal_dispersion.cfg":
            assert (P.N1, P.N2, P.diffusion) == (100, 50, 1)
        if name == "hyperbolic_test.cfg":
            assert P.is_test == 1 and P.bc == E.BC_PERIODIC and P.cfl == 0.95


def _write(tmp_path, text):
    p = tmp_path / "x.cfg"
    p.write_text(text)
    return str(p)


def test_missing_key_is_a_status(tmp_path):
    base = open(os.path.join(HERE, "golden", "quarter_five_spot_128_upwind.cfg")).read()
    bad = base.replace("mu_res = 41.0;", "")
    with pytest.raises(E.ImpecError) as ei:
        E.load_cfg(_write(tmp_path, bad))
    assert ei.value.status == 6


@pytest.mark.parametrize("edit", [("\"diagonal\"", "\"sideways\""), ("\"upwind_split\"", "\"weno\""),
                                  ("dimensional_splitting = \"parallel\"", "dimensional_splitting = \"zigzag\""), ("{ para_method", "( para_method")])
def test_invalid_values_are_rejected(tmp_path, edit):
    base = open(os.path.join(HERE, "golden", "quarter_five_spot_128_upwind.cfg")).read()
    with pytest.raises(E.ImpecError):
        E.load_cfg(_write(tmp_path, base.replace(*edit)))


def test_comments_lists_and_unknown_keys(tmp_path):
    base = open(os.path.join(HERE, "golden", "quarter_five_spot_128_upwind.cfg")).read()
    txt = base.replace("log_time_list = [];", "log_time_list = [0.01, 0.02, 3e-2]; /* block */ extra_key = \"x\";")
    P, t0, t1 = E.load_cfg(_write(tmp_path, txt))
    assert P.N1 == 128


def _learned_cfg(tmp_path, weights, extra=""):
    base = open(os.path.join(HERE, "golden", "quarter_five_spot_128_upwind.cfg")).read()
    txt = base.replace("cfl_porosity = true;", f"cfl_porosity = true;  learned_weights = \"{weights}\"; {extra}")
    txt = txt.replace("endtime = 0.06;", "endtime = 0.0005;").replace("/tmp/impec2d_c1", str(tmp_path / "out"))
    return _write(tmp_path, txt)


def test_learned_keys(tmp_path):
    """gb300.learned_weights turns the previous-pressure start on (the network moves it);
    gb300.learned_factor accepts the supported averaging factors only."""
    P, _, _ = E.load_cfg(_learned_cfg(tmp_path, tmp_path / "w.npy"))
    assert P.warm_start == 1
    P, _, _ = E.load_cfg(_learned_cfg(tmp_path, tmp_path / "w.npy", "learned_factor = 2;"))
    with pytest.raises(E.ImpecError):
        E.load_cfg(_learned_cfg(tmp_path, tmp_path / "w.npy", "learned_factor = 3;"))


@pytest.mark.gpu
def test_run_cfg_with_learned_weights(tmp_path):
    """The executable's entry point loads trained parameters from the .npy that
    `bench.py --study learned --net-out` writes and runs with the network attached; a file of
    the wrong size is a status, not a crash."""
    import numpy as np
    net = E.Net(seed=4)
    w = net.parameters()
    net.close()
    np.save(tmp_path / "w.npy", w)
    assert E.lib().impec_run_cfg(str(_learned_cfg(tmp_path, tmp_path / "w.npy")).encode(), 1) == 0, E.last_error()
    np.save(tmp_path / "short.npy", w[:100])
    assert E.lib().impec_run_cfg(str(_learned_cfg(tmp_path, tmp_path / "short.npy")).encode(), 1) != 0
    assert "parameters" in E.last_error()
