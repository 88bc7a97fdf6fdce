"""ctypes binding of the reference Impec2D build (oracle/_ref) -- TEST INFRASTRUCTURE ONLY.

``oracle/_ref/libimpec2d_ref.so`` is the reference's own ``src/*.cpp`` compiled unchanged
against the stand-ins in ``oracle/refshim`` (recipe: ``oracle/Makefile.ref``), plus the C entry
points of ``oracle/ref_driver.cpp``.  It exists only where a reference checkout is at hand
(``IMPEC2D_REFERENCE`` names it; the recipe has a default), so everything here reports
``available() == False`` elsewhere and the tests that need it skip.  The tests use it to pin
the oracle bit for bit; ``tests/golden/make_ref_golden.py`` uses it to write fixtures.

The reference reads its parameters from a ``.cfg`` file.  ``write_cfg`` turns an oracle
``Params`` into one, with the reference's own key names (``src/SimParams.cpp:45-468``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

from . import Params, ptr

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_ref", "libimpec2d_ref.so")
_lib = None

_STYPE = {0: "parallel", 1: "diagonal", 2: "horizontal"}
_HM = {0: "upwind_split", 1: "waf_split", 2: "waf", 3: "ctu", 4: "muscl"}
_SPLIT = {0: "alternating_sweeps", 1: "x_sweep_first", 2: "y_sweep_first", 3: "strang", 4: "parallel"}
_WELL = {0: "circle", 1: "gauss", 2: "one_cell"}
_MODE = {0: "pulsing", 1: "linear", 2: "constant"}
_AVG = {0: "mean_concentration", 1: "harmonic"}
_PARA = {0: "explicit", 1: "crank-nicolson"}


def reference_dir() -> str | None:
    d = os.environ.get("IMPEC2D_REFERENCE")
    if d:
        return d if os.path.isdir(os.path.join(d, "src")) else None
    return None


def build() -> str | None:
    """Builds _ref with the committed recipe when a reference checkout is at hand."""
    args = ["make", "-s", "-j8", "-C", _HERE, "-f", "Makefile.ref"]
    d = reference_dir()
    if d:
        args.append(f"REFERENCE={d}")
    r = subprocess.run(args, capture_output=True, text=True)
    return _LIB if r.returncode == 0 and os.path.exists(_LIB) else None


def available() -> bool:
    try:
        lib()
        return True
    except OSError:
        return False


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB) and build() is None:
            raise OSError("the reference build (oracle/_ref) is not available: no reference checkout")
        _lib = C.CDLL(_LIB)
        _declare(_lib)
    return _lib


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_V = C.c_void_p


def _declare(L):
    def d(name, res, *args):
        f = getattr(L, name)
        f.restype = res
        f.argtypes = list(args)

    d("ref_open", _V, C.c_char_p)
    d("ref_close", None, _V)
    d("ref_dims", None, _V, _I, _I, _I, _D, _D)
    d("ref_source", None, _V, _D)
    d("ref_horizontal_source", None, _V, _D, C.c_double)
    d("ref_exact_vol_frac_circle", C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double)
    d("ref_fill_scalar_neumann", None, _V, _D)
    d("ref_fill_scalar_periodic", None, _V, _D)
    d("ref_fill_velocity_neumann", None, _V, _D)
    d("ref_mu", C.c_double, _V, C.c_double)
    d("ref_face_mobility", None, _V, _D, _D, _D)
    d("ref_pressure_matrix", None, _V, _D, _D)
    d("ref_pressure_rhs", None, _V, _D, _D)
    d("ref_pressure_solve", C.c_int, _V, _D, _D, _D)
    d("ref_calc_velocities", None, _V, _D, _D, _D)
    d("ref_max_stable_dt", C.c_double, _V, _D, _D)
    d("ref_tr_integrate", C.c_double, _V, _D, _D, C.c_double)
    d("ref_flux_F", None, _V, C.c_int, _D, _D, _D, C.c_double)
    d("ref_flux_G", None, _V, C.c_int, _D, _D, _D, C.c_double)
    d("ref_advect_x", None, _V, C.c_int, _D, _D, C.c_double)
    d("ref_advect_y", None, _V, C.c_int, _D, _D, C.c_double)
    d("ref_advect_split", None, _V, C.c_int, _D, _D, C.c_double, _I)
    d("ref_hyperbolic_solve", C.c_int, _V, C.c_int, _D, _D, _D, C.c_double, _I, _D)
    d("ref_peaceman_F", None, _V, _D, C.c_int, C.c_int, _D, _D)
    d("ref_peaceman_G", None, _V, _D, C.c_int, C.c_int, _D, _D)
    d("ref_cn_matrix", None, _V, _D, C.c_double, _D)
    d("ref_cn_rhs", None, _V, _D, _D, C.c_double, _D)
    d("ref_cn_solve", C.c_int, _V, _D, _D, C.c_double)
    d("ref_run", C.c_int, _V, _D, _D, _D, _D, _I)
    d("ref_run_component", C.c_int, _V)
    d("ref_total_mass", C.c_double, _V, _D)
    d("ref_mass_error", C.c_double, _V, _D, C.c_double, C.c_double)
    d("ref_divergence_error", C.c_double, _V, _D)
    d("ref_velocity_boundary_error", C.c_double, _V, _D)
    d("ref_advection_norm", C.c_double, _V, _D, C.c_double, C.c_int)
    d("ref_advection_test", C.c_int, C.c_char_p, C.c_double, C.c_double, _D, _D)


def _b(x) -> str:
    return "true" if x else "false"


def _f(x) -> str:
    # libconfig types a value by its literal: floats must carry a point or an exponent.
    s = repr(float(x))
    return s if any(ch in s for ch in ".einf") else s + ".0"


def write_cfg(path: str, P: Params, *, results_dir: str, tstart: float | None = None, tfinal: float | None = None,
              log_to_file: bool = False, check_mass: bool = True, check_noflow: bool = True,
              check_div: bool = True, test: dict | None = None, init_file: str | None = None) -> str:
    """Writes a .cfg that the reference's SimParams reads into the parameters of P.

    Extensions of the engine that the reference lacks (per-cell K, Dm, the Peaceman guard)
    have no key: a P that uses them is rejected, since the reference would silently ignore them.
    """
    if P.K11 or P.K22 or P.Dm != 0.0:
        raise ValueError("the reference has K = 1 and no molecular diffusion")
    t0 = P.tstart if tstart is None else tstart
    t1 = P.tfinal if tfinal is None else tfinal
    gen = [
        f"starttime = {_f(t0)}; endtime = {_f(t1)};",
        f"x_lb = {_f(P.x_lb)}; x_ub = {_f(P.x_ub)}; y_lb = {_f(P.y_lb)}; y_ub = {_f(P.y_ub)};",
        f'source_type = "{_STYPE[P.stype]}";',
        f"x_cells = {P.N1}; y_cells = {P.N2}; num_ghostcells = {P.g};",
        f"I = {_f(P.I)};",
        f"log_to_file = {_b(log_to_file)};",
        "log_counter_list = []; log_time_list = [];",
        "log_skip_steps = 0; time_matching = false; log_mass_conservation = false;",
        f'log_dir = "{results_dir}";',
        f"check_mass_conservation = {_b(check_mass)}; max_mass_frac_error = 0.0;",
        f"check_noflow_boundary = {_b(check_noflow)}; check_divergence = {_b(check_div)};",
        f'results_dir = "{results_dir}";',
        f"is_test = {_b(P.is_test)}; gnuplot = false; levelset = false; syncmode = \"sync\";",
    ]
    if init_file:
        gen.append(f'init_file = "{init_file}";')
    ell = [
        f'eps = {_f(P.eps)}; ell_method = "mg"; bound_type = "neumann"; const_bound_val = 0.0;',
        f'mu_res = {_f(P.mu_res)}; mu_inj = {_f(P.mu_inj)}; average_procedure = "{_AVG[P.avgproc]}";',
    ]
    wells = [
        f'well_rc = {_f(P.well_rc)}; well_profile = "{_WELL[P.well_profile]}"; mode = "{_MODE[P.inj_mode]}";',
        "q_rand_max = 0.001; front_const_width = 3; front_rand_width = 1;",
        f"q_high_multiple = {_f(P.q_high_multiple)}; well_width = {_f(P.well_width)}; q_freq = {_f(P.q_freq)};",
    ]
    para = [f'para_method = "{_PARA[P.ptype]}"; eps = {_f(P.para_eps)};']
    hyp = [
        f'inj_fluid_conc = {_f(P.inj_fluid_conc)}; hyper_method = "{_HM[P.hmtype]}";',
        f'dimensional_splitting = "{_SPLIT[P.dim_splitting]}";',
        f"cfl = {_f(P.cfl)}; dt_diff_limiter = {_f(P.dt_diff_limit)}; porosity = {_f(P.porosity)};",
        'time_integration = "tr"; ti_eps = 1.0e-15;',
        f"nu = {_f(P.nu)}; diffusion = {_b(P.diffusion)}; alpha_t = {_f(P.alpha_t)}; alpha_l = {_f(P.alpha_l)};",
    ]
    groups = [("general", gen), ("elliptic", ell), ("wells", wells), ("parabolic", para), ("hyperbolic", hyp)]
    if test is not None or P.is_test:  # the reference reads a test group whenever is_test is set
        test = test or {}
        t = dict(component="hyperbolic", testno=1, profile="sine", hyp_norm=1, initial_x_cells=P.N1,
                 initial_y_cells=P.N2, levels=1)
        t.update(test)
        lines = []
        for k, v in t.items():
            lines.append(f'{k} = "{v}";' if isinstance(v, str) else f"{k} = {v};")
        for k in ("num_result_file", "ex_result_file", "norm_file", "num_u_file", "ex_u_file", "num_v_file",
                  "ex_v_file"):
            if k not in t:
                lines.append(f'{k} = "{os.path.join(results_dir, k)}";')
        groups.append(("test", lines))
    text = "application:\n{\n" + "".join(
        f"  {name}:\n  {{\n" + "".join(f"    {ln}\n" for ln in body) + "  };\n" for name, body in groups) + "};\n"
    with open(path, "w") as f:
        f.write(text)
    return path


class Case:
    """A reference solver opened on the parameters of an oracle Params (via a written .cfg)."""

    def __init__(self, P: Params, workdir: str | None = None, **cfg_kw):
        self._tmp = None
        if workdir is None:
            self._tmp = tempfile.TemporaryDirectory(prefix="impec_ref_")
            workdir = self._tmp.name
        self.dir = workdir
        self.cfg = write_cfg(os.path.join(workdir, "case.cfg"), P, results_dir=workdir, **cfg_kw)
        self.P = P
        self.h = lib().ref_open(self.cfg.encode())
        n1, n2, g = C.c_int(), C.c_int(), C.c_int()
        dx, dy = C.c_double(), C.c_double()
        lib().ref_dims(self.h, C.byref(n1), C.byref(n2), C.byref(g), C.byref(dx), C.byref(dy))
        assert (n1.value, n2.value, g.value) == (P.N1, P.N2, P.g), "the reference parsed other dimensions"
        self.dx, self.dy = dx.value, dy.value

    def close(self):
        if self.h:
            lib().ref_close(self.h)
            self.h = None
        if self._tmp is not None:
            self._tmp.cleanup()
            self._tmp = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __getattr__(self, name):
        f = getattr(lib(), "ref_" + name)

        def call(*args):
            conv = [ptr(a) if isinstance(a, np.ndarray) else a for a in args]
            return f(self.h, *conv)

        return call

    def source(self) -> np.ndarray:
        q = np.zeros(self.P.N1 * self.P.N2)
        lib().ref_source(self.h, ptr(q))
        return q
