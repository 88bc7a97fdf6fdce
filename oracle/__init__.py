"""ctypes binding of the Impec2D CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle (``oracle_core.cpp``, ``oracle_solve.cpp``) restates the reference
Impec2D discretisation in plain FP64 C++.  Only ``tests/``, the smoke check and
the CPU-baseline leg of ``bench.py`` may import this module; the product path
never does.  See ``oracle.h`` for the parity status: pinned bit for bit to the reference's
own code compiled in ``oracle/_ref`` (``oracle/ref.py``), except HYPRE's iterates.

Arrays use the reference's ghost-cell layouts (``src/Impec2DSolver.cpp:151-182``):
scalar ``(N1+2g, N2+2g)``, velocity ``(N1+1+2g, N2+1+2g, 2)``, source ``N1*N2``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")

MEANCONC, HARMONIC = 0, 1
EXPLICIT, CRANKNICOLSON = 0, 1
ALTERNATING, X_FIRST, Y_FIRST, STRANG, SYMMETRIC_PARALLEL = 0, 1, 2, 3, 4
UPWINDSPLIT, WAFSPLIT, WAF, CTU, MUSCL = 0, 1, 2, 3, 4
PARALLEL, DIAGONAL, HORIZONTAL = 0, 1, 2
CIRCULAR, GAUSSIAN, ONECELL = 0, 1, 2


class Params(C.Structure):
    _fields_ = [
        ("N1", C.c_int), ("N2", C.c_int), ("g", C.c_int),
        ("x_lb", C.c_double), ("x_ub", C.c_double), ("y_lb", C.c_double), ("y_ub", C.c_double),
        ("mu_res", C.c_double), ("mu_inj", C.c_double),
        ("avgproc", C.c_int), ("nu", C.c_double),
        ("porosity", C.c_double), ("cfl", C.c_double), ("inj_fluid_conc", C.c_double), ("I", C.c_double),
        ("diffusion", C.c_int), ("alpha_l", C.c_double), ("alpha_t", C.c_double), ("Dm", C.c_double),
        ("ptype", C.c_int), ("dt_diff_limit", C.c_double),
        ("dim_splitting", C.c_int), ("hmtype", C.c_int), ("stype", C.c_int),
        ("is_test", C.c_int), ("testno", C.c_int),
        ("eps", C.c_double), ("para_eps", C.c_double),
        ("well_profile", C.c_int), ("well_rc", C.c_double),
        ("well_width", C.c_double), ("q_high_multiple", C.c_double), ("q_freq", C.c_double),
        ("tstart", C.c_double), ("tfinal", C.c_double), ("inj_mode", C.c_int),
        ("K11", C.POINTER(C.c_double)), ("K22", C.POINTER(C.c_double)),
        ("peaceman_guard", C.c_int),
    ]


class State(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("dt", C.c_double), ("total_outflux", C.c_double),
        ("counter", C.c_int), ("prev_first_sweep", C.c_int), ("its", C.c_int), ("para_its", C.c_int),
        ("mass_err", C.c_double), ("vel_err", C.c_double), ("div_err", C.c_double), ("relres", C.c_double),
    ]


def build() -> str:
    """Compile liboracle.so with the committed Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        _lib = C.CDLL(_LIB)
        _declare(_lib)
    return _lib


_D = C.POINTER(C.c_double)
_PP = C.POINTER(Params)


def _declare(L):
    def d(name, res, *args):
        f = getattr(L, name)
        f.restype = res
        f.argtypes = list(args)

    d("or_fill_scalar_neumann", None, _PP, _D)
    d("or_fill_scalar_periodic", None, _PP, _D)
    d("or_fill_velocity_neumann", None, _PP, _D)
    d("or_mu", C.c_double, _PP, C.c_double)
    d("or_pressure_matrix", None, _PP, _D, _D)
    d("or_pressure_matrix_neumann", None, _PP, _D, _D)
    d("or_pressure_rhs", None, _PP, _D, _D)
    d("or_face_mobility", None, _PP, _D, _D, _D)
    d("or_project_diagonal", None, _PP, _D, C.c_int, C.c_int, _D)
    d("or_matvec9", None, _PP, _D, _D, _D)
    d("or_relres9", C.c_double, _PP, _D, _D, _D)
    d("or_solve_banded", C.c_int, _PP, _D, _D, _D)
    d("or_pressure_solve", C.c_int, _PP, _D, _D, _D, C.c_int, C.c_double, C.POINTER(C.c_int), _D)
    d("or_calc_velocities", None, _PP, _D, _D, _D)
    d("or_max_stable_dt", C.c_double, _PP, _D)
    d("or_max_stable_advection_dt", C.c_double, _PP, _D)
    d("or_tr_integrate", C.c_double, _PP, _D, _D, C.c_double)
    d("or_flux_F", None, _PP, _D, _D, _D, C.c_double)
    d("or_flux_G", None, _PP, _D, _D, _D, C.c_double)
    d("or_advect_x", None, _PP, _D, _D, C.c_double)
    d("or_advect_y", None, _PP, _D, _D, C.c_double)
    d("or_advect_split", None, _PP, _D, _D, C.c_double, C.POINTER(C.c_int))
    d("or_ctu_advect", None, _PP, _D, _D, C.c_double)
    d("or_peaceman_F", None, _PP, _D, C.c_int, C.c_int, _D, _D)
    d("or_peaceman_G", None, _PP, _D, C.c_int, C.c_int, _D, _D)
    d("or_cn_matrix", None, _PP, _D, C.c_double, _D)
    d("or_cn_rhs", None, _PP, _D, _D, C.c_double, _D)
    d("or_cn_solve", C.c_int, _PP, _D, _D, C.c_double, C.c_int, C.c_double, C.POINTER(C.c_int), _D)
    d("or_hyperbolic_solve", C.c_int, _PP, _D, _D, _D, C.c_double, C.POINTER(C.c_int), _D, C.c_int)
    d("or_impes_step", C.c_int, _PP, C.POINTER(State), _D, _D, _D, _D, _D, C.c_int, C.POINTER(C.c_int),
      C.c_int, C.c_double)
    d("or_total_mass", C.c_double, _PP, _D)
    d("or_mass_error", C.c_double, _PP, _D, C.c_double, C.c_double)
    d("or_divergence_error", C.c_double, _PP, _D, _D)
    d("or_velocity_boundary_error", C.c_double, _PP, _D)
    d("or_init_source", None, _PP, _D, C.c_double)
    d("or_exact_vol_frac_circle", C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double)
    d("or_profile", C.c_double, _PP, C.c_int, C.c_double, C.c_double)
    d("or_advection_norm", C.c_double, _PP, _D, C.c_int, C.c_int)
    d("or_elliptic_test", C.c_int, _PP, _D)
    d("or_mg_solve", C.c_int, _PP, _D, _D, _D, C.c_double, C.c_int, C.POINTER(C.c_int), _D, C.c_int,
      C.c_int, C.c_double)
    d("or_num_threads", C.c_int)
    d("or_set_num_threads", C.c_int, C.c_int)


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


def make_params(**kw) -> Params:
    """Params with the reference's example defaults (examples/parallel.cfg) overridden by kw."""
    P = Params()
    defaults = dict(
        N1=64, N2=64, g=2, x_lb=0.0, x_ub=1.0, y_lb=0.0, y_ub=1.0, mu_res=41.0, mu_inj=1.0,
        avgproc=HARMONIC, nu=1.0, porosity=1.0, cfl=0.5, inj_fluid_conc=1.0, I=1.0,
        diffusion=0, alpha_l=1.0, alpha_t=1.0, Dm=0.0, ptype=CRANKNICOLSON, dt_diff_limit=0.9,
        dim_splitting=SYMMETRIC_PARALLEL, hmtype=MUSCL, stype=DIAGONAL, is_test=0, testno=1,
        eps=1e-10, para_eps=1e-14, well_profile=ONECELL, well_rc=0.05, well_width=0.05,
        q_high_multiple=50.0, q_freq=20.0, tstart=0.0, tfinal=0.4, inj_mode=2, peaceman_guard=1,
    )
    defaults.update(kw)
    keep = {}
    for k, v in defaults.items():
        if k in ("K11", "K22"):
            keep[k] = v
            continue
        setattr(P, k, v)
    for k, v in keep.items():
        if v is not None:
            arr = np.ascontiguousarray(v, dtype=np.float64).ravel()
            setattr(P, k, ptr(arr))
            setattr(P, "_keep_" + k, arr)  # keep the buffer alive with the struct
    return P


def scalar_shape(P):
    return (P.N1 + 2 * P.g, P.N2 + 2 * P.g)


def vel_shape(P):
    return (P.N1 + 1 + 2 * P.g, P.N2 + 1 + 2 * P.g, 2)


def interior(P, a):
    g = P.g
    return a[g:g + P.N1, g:g + P.N2]


def with_ghosts(P, interior_field, fill="neumann"):
    a = np.zeros(scalar_shape(P))
    interior(P, a)[...] = interior_field
    if fill == "neumann":
        lib().or_fill_scalar_neumann(C.byref(P), ptr(a))
    elif fill == "periodic":
        lib().or_fill_scalar_periodic(C.byref(P), ptr(a))
    return a
