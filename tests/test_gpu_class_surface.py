"""The engine's C++ class surface (the reference's EllipticSolver / MGSolver / HyperbolicSplitSolver
/ TRIntegrator names and signatures over reference-layout host arrays) against the reference's
own outputs (tests/golden/ref_ops.npz, written by the reference's code compiled in oracle/_ref).

tests/cpp/class_surface.cpp is compiled here against libimpec2d.so and run on the fixture
inputs; interiors are compared with the same tolerances as tests/test_gpu_ref_golden.py.
"""
import ast
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from oracle import ref as R

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def program(engine, tmp_path_factory):
    from impec2d_gb300 import build as B
    lib = B.build()
    d = tmp_path_factory.mktemp("class_surface")
    exe = str(d / "class_surface")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-O2", "-std=c++17", os.path.join(HERE, "cpp", "class_surface.cpp"), "-o", exe,
           f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(ROOT, 'impec2d_gb300', 'csrc', 'host')}",
           f"-L{libdir}", "-limpec2d", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", ["diag", "par", "horiz"])
def test_class_surface_against_reference_outputs(program, tmp_path, name):
    gold = np.load(os.path.join(HERE, "golden", "ref_ops.npz"))
    g = lambda k: gold[f"{name}/{k}"]  # noqa: E731
    kw = ast.literal_eval(str(g("params")))
    P = O.make_params(**{**kw, "eps": 1e-12, "para_eps": 1e-14})
    cfg = R.write_cfg(str(tmp_path / "case.cfg"), P, results_dir=str(tmp_path))
    for k in ("c", "v", "v_of_p", "p", "q"):
        np.ascontiguousarray(g(k), dtype=np.float64).tofile(tmp_path / f"{k}.bin")
    dt = float(g("dt_used"))
    r = subprocess.run([program, cfg, str(tmp_path), repr(dt)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    sc = dict(line.split() for line in open(tmp_path / "out_scalars.txt"))
    inner = lambda a: O.interior(P, a.reshape(O.scalar_shape(P)))  # noqa: E731
    out = lambda k: np.fromfile(tmp_path / f"out_{k}.bin")  # noqa: E731
    # EllipticSolver::Solve: the reference's system to 1e-12
    assert sc["solve_ok"] == "1" and float(sc["relres"]) <= 1e-12
    assert _rel(inner(out("p_solve")), O.interior(P, g("p"))) <= 1e-9
    # CalcVelocities (ghost fills included), MaxStableTimestep, TRIntegrator
    vo, vr = out("v_of_p").reshape(O.vel_shape(P)), g("v_of_p")
    assert np.abs(vo - vr).max() <= 1e-13 * np.abs(vr).max()
    assert abs(float(sc["dt"]) - float(g("dt"))) <= 1e-14 * float(g("dt"))
    assert _rel(inner(out("tr_c")), O.interior(P, g("tr_c"))) <= 1e-13
    assert abs(float(sc["tr_outflux"]) - float(g("tr_outflux"))) <= 1e-13 * abs(float(g("tr_outflux")))
    # Advect_X / Advect_Y from the reference's MUSCL fluxes, AdvectSplit
    gg, N1, N2 = P.g, P.N1, P.N2
    F = g("F_muscl").reshape(N1 + 1, N2 + 2 * gg)[:, gg:gg + N2]
    G = g("G_muscl").reshape(N1 + 2 * gg, N2 + 1)[gg:gg + N1, :]
    c0 = O.interior(P, g("c"))
    dx, dy = (P.x_ub - P.x_lb) / N1, (P.y_ub - P.y_lb) / N2
    assert _rel(inner(out("advect_x")), c0 + dt / dx * (F[:-1] - F[1:])) <= 1e-13
    assert _rel(inner(out("advect_y")), c0 + dt / dy * (G[:, :-1] - G[:, 1:])) <= 1e-13
    assert _rel(inner(out("advect_split")), O.interior(P, g("advect_muscl"))) <= 1e-13
    # Solve_Parabolic_cc_to_c and HyperbolicSplitSolver::Solve
    assert sc["cn_ok"] == "1" and _rel(inner(out("cn_c")), O.interior(P, g("cn_c"))) <= 1e-12
    assert sc["hyp_ok"] == "1" and _rel(inner(out("hyp_c")), O.interior(P, g("hyp_c"))) <= 1e-12
    assert abs(float(sc["hyp_outflux"]) - float(g("hyp_outflux"))) <= 1e-12 * abs(float(g("hyp_outflux")))
