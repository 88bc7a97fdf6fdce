"""GB300-native Impec2D IMPES engine: Python binding of the C ABI (include/impec2d.h).

The numerical work runs in hand-written CUDA kernels for sm_103a inside
``libimpec2d.so``; this module only loads that library with ctypes and passes device
pointers (torch CUDA tensors) and plain scalars across.  There is no CPU fallback:
if the library is missing or no GPU is present, calls raise.

Device layout (no ghost cells): cell fields ``(N1, N2)``, x-face field ``u``
``(N1+1, N2)``, y-face field ``v`` ``(N1, N2+1)``, all float64, row-major.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libimpec2d.so")

MEANCONC, HARMONIC = 0, 1
EXPLICIT, CRANKNICOLSON = 0, 1
ALTERNATING, X_FIRST, Y_FIRST, STRANG, SYMMETRIC_PARALLEL = 0, 1, 2, 3, 4
UPWINDSPLIT, WAFSPLIT, WAF, CTU, MUSCL = 0, 1, 2, 3, 4
PARALLEL, DIAGONAL, HORIZONTAL = 0, 1, 2
BC_NEUMANN, BC_PERIODIC = 0, 1
PREC_FP64, PREC_MIXED = 0, 1

STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_NOT_CONVERGED", 4: "ERR_NAN", 5: "ERR_NO_DEVICE",
          6: "ERR_CONFIG"}


class ImpecError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)}: {last_error()}")


class Params(C.Structure):
    _fields_ = [
        ("N1", C.c_int), ("N2", C.c_int),
        ("x_lb", C.c_double), ("x_ub", C.c_double), ("y_lb", C.c_double), ("y_ub", C.c_double),
        ("mu_res", C.c_double), ("mu_inj", C.c_double),
        ("avgproc", C.c_int), ("nu", C.c_double),
        ("porosity", C.c_double), ("cfl", C.c_double), ("inj_fluid_conc", C.c_double), ("I", C.c_double),
        ("diffusion", C.c_int), ("alpha_l", C.c_double), ("alpha_t", C.c_double), ("Dm", C.c_double),
        ("ptype", C.c_int), ("dt_diff_limit", C.c_double),
        ("dim_splitting", C.c_int), ("hmtype", C.c_int), ("stype", C.c_int),
        ("is_test", C.c_int), ("testno", C.c_int), ("bc", C.c_int),
        ("eps", C.c_double), ("para_eps", C.c_double),
        ("peaceman_guard", C.c_int), ("cfl_porosity", C.c_int), ("precision", C.c_int),
        ("max_cycles", C.c_int), ("warm_start", C.c_int),
    ]


class StepInfo(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("dt", C.c_double), ("total_outflux", C.c_double), ("relres", C.c_double),
        ("mass_err", C.c_double),
        ("counter", C.c_int), ("its", C.c_int), ("para_its", C.c_int), ("prev_first_sweep", C.c_int),
        ("clipped", C.c_int),
    ]


_lib = None
_VP = C.c_void_p
_PI = C.POINTER(C.c_int)
_PD = C.POINTER(C.c_double)

# name -> (restype, argtypes)
_SIGS = {
    "impec_last_error": (C.c_char_p, []),
    "impec_default_params": (None, [C.POINTER(Params), C.c_int, C.c_int]),
    "impec_ctx_create": (C.c_int, [C.POINTER(Params), _VP, C.POINTER(_VP)]),
    "impec_ctx_destroy": (C.c_int, [_VP]),
    "impec_ctx_params": (C.c_int, [_VP, C.POINTER(Params)]),
    "impec_set_permeability": (C.c_int, [_VP, _VP, _VP]),
    "impec_set_source": (C.c_int, [_VP, _VP]),
    "impec_pressure_solve": (C.c_int, [_VP, _VP, _VP, C.c_double, _PI, _PD]),
    "impec_face_mobility": (C.c_int, [_VP, _VP, _VP, _VP]),
    "impec_pressure_apply": (C.c_int, [_VP, _VP, _VP, _VP]),
    "impec_velocity": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "impec_max_stable_dt": (C.c_int, [_VP, _VP, _VP, _PD]),
    "impec_tr_integrate": (C.c_int, [_VP, _VP, C.c_double, _PD]),
    "impec_advect_x": (C.c_int, [_VP, _VP, _VP, C.c_double]),
    "impec_advect_y": (C.c_int, [_VP, _VP, _VP, C.c_double]),
    "impec_advect_split": (C.c_int, [_VP, _VP, _VP, _VP, C.c_double, _PI]),
    "impec_dispersion_cn": (C.c_int, [_VP, _VP, _VP, _VP, C.c_double, C.c_double, _PI, _PD]),
    "impec_hyperbolic_solve": (C.c_int, [_VP, _VP, _VP, _VP, C.c_double, _PI, _PD]),
    "impec_diagnostics": (C.c_int, [_VP, _VP, _VP, _VP, _PD]),
    "impec_state": (C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP)]),
    "impec_step": (C.c_int, [_VP, C.c_double, C.POINTER(StepInfo)]),
    "impec_run_steps": (C.c_int, [_VP, C.c_int, C.POINTER(StepInfo)]),
    "impec_state_upload": (C.c_int, [_VP, _PD, _PD, C.c_int]),
    "impec_state_download": (C.c_int, [_VP, _PD, _PD, _PD, C.c_int]),
    "impec_set_time": (C.c_int, [_VP, C.c_double]),
    "impec_checkpoint_save": (C.c_int, [_VP, C.c_char_p]),
    "impec_checkpoint_load": (C.c_int, [_VP, C.c_char_p]),
    "impec_velocity_upload": (C.c_int, [_VP, _PD, C.c_int]),
    "impec_pressure_upload": (C.c_int, [_VP, _PD, C.c_int]),
    "impec_set_pin_kappa": (C.c_int, [_VP, C.c_double]),
    "impec_cfg_load": (C.c_int, [C.c_char_p, C.POINTER(Params), _PD, _PD]),
    "impec_cfg_source": (C.c_int, [C.c_char_p, _PD]),
    "impec_run_cfg": (C.c_int, [C.c_char_p, C.c_int]),
    "impec_launch_count": (C.c_int, [_VP, C.POINTER(C.c_longlong)]),
    "impec_pressure_solve_resident": (C.c_int, [_VP, C.c_int, _PI, _PD]),
    "impec_advect_symmetric_noalloc": (C.c_int, [C.POINTER(Params), _VP, _VP, _VP, C.c_double, _VP]),
    "impec_time_kernel": (C.c_int, [_VP, C.c_int, C.c_int, _PD, _PD]),
    "impec_time_kernel_cold": (C.c_int, [_VP, C.c_int, C.c_int, _VP, C.c_size_t, _PD, _PD, _PD]),
    "impec_measure_fp64": (C.c_int, [_PD]),
    "impec_selftest_bounded_wait": (C.c_int, [C.c_uint, C.c_int, _PI]),
    "impec_set_tuning": (C.c_int, [_VP, C.c_char_p, C.c_long]),
    "impec_get_tuning": (C.c_int, [_VP, C.c_char_p, C.POINTER(C.c_long)]),
    "impec_autotune": (C.c_int, [_VP, C.c_int, C.c_char_p, C.c_int]),
    "impec_gemm_bf16": (C.c_int, [_VP, C.c_int, _VP, C.c_int, _VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP]),
    "impec_conv3x3_forward": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP, C.c_int, C.c_int, _VP, _VP,
                                        _VP, _VP, _VP]),
    "impec_conv3x3_input_grad": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, C.c_int, _VP, _VP, _VP, _VP,
                                           _VP]),
    "impec_conv3x3_weight_grad": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "impec_net_create": (C.c_int, [C.c_ulonglong, C.POINTER(C.c_void_p)]),
    "impec_net_destroy": (C.c_int, [_VP]),
    "impec_net_train_batch": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _PD, _VP]),
    "impec_net_backprop": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_int, C.c_int, _PD, _VP]),
    "impec_net_forward": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "impec_net_parameters": (C.c_int, [_VP, _VP, _VP, C.POINTER(C.c_size_t), C.c_int]),
    "impec_last_solve": (C.c_int, [_VP, C.POINTER(C.c_int), _PD, _PD]),
    "impec_learned_attach": (C.c_int, [_VP, _VP, C.c_int, C.c_int]),
    "impec_learned_features": (C.c_int, [_VP, _VP]),
    "impec_learned_target": (C.c_int, [_VP, _VP]),
    "impec_learned_alpha": (C.c_int, [_VP, _PD]),
    "impec_ensemble_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]),
    "impec_ensemble_step": (C.c_int, [_VP, C.c_int, C.c_int]),
    "impec_ensemble_destroy": (C.c_int, [_VP]),
    "impec_project_diagonal": (C.c_int, [_VP, C.c_int, _VP, C.c_int, C.c_int]),
    "impec_project_diagonal_download": (C.c_int, [_VP, C.c_int, _PD, C.c_int, C.c_int]),
}

KERNELS = {0: "k_rb_face5<double> (fine RB-GS sweep, FP64)", 1: "k_rb_face5<float> (fine RB-GS sweep, FP32)",
           2: "k_fine_resid (FP64 residual + norm)", 3: "k_sweep_x (MUSCL x-sweep)", 4: "k_sweep_y (MUSCL y-sweep)"}


def launch_count(ctx) -> int:
    n = C.c_longlong()
    _chk(lib().impec_launch_count(ctx.h, C.byref(n)), "launch_count")
    return n.value


def measure_fp64() -> float:
    """FP64 fused multiply-adds per second of the current device (measured)."""
    v = C.c_double()
    _chk(lib().impec_measure_fp64(C.byref(v)), "measure_fp64")
    return v.value


def time_kernel(ctx, which: int, reps: int = 20):
    ms, b = C.c_double(), C.c_double()
    _chk(lib().impec_time_kernel(ctx.h, which, reps, C.byref(ms), C.byref(b)), "time_kernel")
    return ms.value, b.value


def roofline_probe(ctx, P, precision: str, flush=None, peaks_path: str | None = None, traffic_path: str | None = None,
                   reps: int = 20):
    """Achieved bandwidth of the dominant kernel, the fine-level red-black sweep, against the
    measured HBM copy bandwidth, and its FP64 operation rate against the measured DFMA rate.
    Each repetition is timed cold: L2 is overwritten first (``flush``, a CUDA tensor larger
    than L2), then CUDA events on the engine's stream bracket the sweep.  Algorithmic bytes
    follow the five-point model: x read and written, b, and the two face planes (40 B per cell in
    FP64).  ``traffic`` (DRAM bytes per sweep) comes from the ncu capture recorded in
    profiles/traffic.json when that file names the kernel and grid."""
    import json
    which = 1 if precision == "mixed" else 0
    if P.nu != 1.0:  # nine-point operator: four-colour sweeps, timed back to back
        ms, b = time_kernel(ctx, which)
        t = "double" if which == 0 else "float"
        return {"bound": "hbm", "kernel": f"k_gs4_exp9<{t}> (fine four-colour GS sweep, nine-point)",
                "grid": f"{P.N1}x{P.N2}", "achieved": b / (ms * 1e-3) / 1e9, "peak": 6800.0, "unit": "GB/s",
                "frac": b / (ms * 1e-3) / 1e9 / 6800.0, "peak_source": "fallback", "bytes_per_launch": b,
                "ms_per_launch": ms, "timing": "back-to-back launches", "traffic": None}
    if flush is None:
        import torch
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ms, ms_min, b = C.c_double(), C.c_double(), C.c_double()
    _chk(lib().impec_time_kernel_cold(ctx.h, which, reps, C.c_void_p(flush.data_ptr()), flush.numel() * flush.element_size(),
                                      C.byref(ms), C.byref(ms_min), C.byref(b)), "time_kernel_cold")
    ms, ms_min, b = ms.value, ms_min.value, b.value
    peak, src = 6800.0, "fallback"
    path = peaks_path or os.path.join(os.path.dirname(HERE), "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            peak, src = float(json.load(open(path))["hbm_gbs"]), "measured"
        except Exception:  # noqa: BLE001
            pass
    ach = b / (ms * 1e-3) / 1e9
    tile = ctx.get_tuning("tile_cells")
    if which == 1:
        tile = ctx.get_tuning("tile_cells32")
    one_launch = tile > 0 and P.N1 * P.N2 >= tile
    t = "double" if which == 0 else "float"
    name = (f"k_rb_tile<{t}> (fine red-black sweep, both colours in one launch)" if one_launch
            else f"k_rb_face5<{t}> (fine red-black sweep, one launch per colour)")
    out = {"bound": "hbm", "kernel": name, "grid": f"{P.N1}x{P.N2}", "achieved": ach, "peak": peak, "unit": "GB/s",
           "frac": ach / peak, "peak_source": src, "bytes_per_launch": b, "bytes_model": "x r+w, b, tx, ty",
           "ms_per_launch": ms, "ms_per_launch_min": ms_min, "timing": "cold (L2 overwritten before each sweep)",
           "traffic": None}
    tpath = traffic_path or os.path.join(os.path.dirname(HERE), "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            rec = json.load(open(tpath)).get(f"{name.split(' ')[0]}@{P.N1}x{P.N2}")
            if rec:
                out["traffic"] = float(rec["dram_bytes_per_launch"])
                out["traffic_source"] = rec["source"]
        except Exception:  # noqa: BLE001
            pass
    if which == 0:
        ops = 5.0 * float(P.N1) * float(P.N2)  # 4 DFMA + 1 DMUL per cell (ncu instruction counts)
        fma = measure_fp64()
        out["fp64"] = {"achieved_ops_per_s": ops / (ms * 1e-3), "peak_ops_per_s": fma,
                       "frac": ops / (ms * 1e-3) / fma, "ops_per_launch": ops,
                       "peak_source": "measured (impec_measure_fp64: DFMA lanes per second)"}
    return out


class Net:
    """Learned warm start: the convolutional encoder-decoder of the tensor-core kernels."""

    def __init__(self, seed: int = 0):
        h = C.c_void_p()
        _chk(lib().impec_net_create(seed, C.byref(h)), "net_create")
        self.h = h

    @staticmethod
    def _ptr(t):
        return C.c_void_p(t.data_ptr())

    def train_batch(self, X, T, lr=3e-4, weight_decay=1e-4) -> float:
        B, H, W, _ = X.shape
        loss = C.c_double()
        _chk(lib().impec_net_train_batch(self.h, self._ptr(X), self._ptr(T), B, H, W, lr, weight_decay,
                                          C.byref(loss), None), "net_train_batch")
        return loss.value

    def backprop(self, X, T) -> float:
        B, H, W, _ = X.shape
        loss = C.c_double()
        _chk(lib().impec_net_backprop(self.h, self._ptr(X), self._ptr(T), B, H, W, C.byref(loss), None),
             "net_backprop")
        return loss.value

    def forward(self, X):
        import torch
        B, H, W, _ = X.shape
        out = torch.empty((B, H, W), dtype=torch.float32, device=X.device)
        _chk(lib().impec_net_forward(self.h, self._ptr(X), B, H, W, self._ptr(out), None), "net_forward")
        return out

    def parameters(self, which: int = 0):
        import numpy as np
        n = C.c_size_t()
        _chk(lib().impec_net_parameters(self.h, None, None, C.byref(n), which), "net_parameters")
        a = np.empty(n.value, dtype=np.float32)
        _chk(lib().impec_net_parameters(self.h, a.ctypes.data_as(C.c_void_p), None, C.byref(n), which),
             "net_parameters")
        return a

    def set_parameters(self, a):
        import numpy as np
        a = np.ascontiguousarray(a, dtype=np.float32)
        n = C.c_size_t()
        _chk(lib().impec_net_parameters(self.h, None, a.ctypes.data_as(C.c_void_p), C.byref(n), 0),
             "net_parameters")

    def attach(self, ctx, factor: int = 1, mode: int = 1):
        """Use this network as the initial guess of ctx's pressure solves (mode 1), or only
        record their features and targets (mode 2)."""
        _chk(lib().impec_learned_attach(ctx.h, self.h, factor, mode), "learned_attach")

    @staticmethod
    def detach(ctx):
        _chk(lib().impec_learned_attach(ctx.h, None, 1, 0), "learned_attach")

    @staticmethod
    def last_features(ctx, X):
        _chk(lib().impec_learned_features(ctx.h, C.c_void_p(X.data_ptr())), "learned_features")

    @staticmethod
    def last_target(ctx, T):
        _chk(lib().impec_learned_target(ctx.h, C.c_void_p(T.data_ptr())), "learned_target")

    @staticmethod
    def last_alpha(ctx) -> float:
        a = C.c_double()
        _chk(lib().impec_learned_alpha(ctx.h, C.byref(a)), "learned_alpha")
        return a.value

    def close(self):
        if self.h:
            _chk(lib().impec_net_destroy(self.h), "net_destroy")
            self.h = None


class Ensemble:
    """Independent contexts advanced together by one graph launch per IMPES step."""

    def __init__(self, members):
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.h.value if isinstance(m.h, C.c_void_p) else m.h
                                                   for m in self.members])
        h = C.c_void_p()
        _chk(lib().impec_ensemble_create(arr, len(self.members), C.byref(h)), "ensemble_create")
        self.h = h

    def step(self, n: int = 1, sync: bool = True):
        _chk(lib().impec_ensemble_step(self.h, n, 1 if sync else 0), "ensemble_step")

    def close(self):
        if self.h:
            lib().impec_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def load_cfg(path: str):
    """Parse a reference .cfg file: returns (Params, tstart, tfinal)."""
    P = Params()
    t0, t1 = C.c_double(), C.c_double()
    _chk(lib().impec_cfg_load(path.encode(), C.byref(P), C.byref(t0), C.byref(t1)), f"cfg_load({path})")
    return P, t0.value, t1.value


def cfg_source(path: str, N1: int, N2: int):
    """Source term q (numpy, N1*N2) of a .cfg's wells."""
    import numpy as np
    q = np.zeros(N1 * N2)
    _chk(lib().impec_cfg_source(path.encode(), q.ctypes.data_as(_PD)), f"cfg_source({path})")
    return q


def lib():
    """Load libimpec2d.so (built by ``impec2d_gb300.build.build()``); raise if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run impec2d_gb300.build.build() first "
                               "(the engine has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    try:
        return lib().impec_last_error().decode()
    except Exception:  # noqa: BLE001 - error path of an error path
        return ""


def _chk(status: int, what: str):
    if status != 0:
        raise ImpecError(status, what)


def default_params(N1: int, N2: int, **kw) -> Params:
    P = Params()
    lib().impec_default_params(C.byref(P), N1, N2)
    for k, v in kw.items():
        if not hasattr(P, k):
            raise AttributeError(k)
        setattr(P, k, v)
    return P


def _p(t):
    if t is None:
        return None
    if isinstance(t, int):  # raw device address (e.g. from Context.state_ptrs)
        return C.c_void_p(t)
    import torch
    assert t.is_cuda and t.dtype == torch.float64 and t.is_contiguous(), "float64 contiguous CUDA tensor expected"
    return C.c_void_p(t.data_ptr())


class Context:
    """One grid's device workspaces (C handle ``impec_ctx``)."""

    def __init__(self, P: Params, stream: int | None = None):
        self.P = P
        h = C.c_void_p()
        _chk(lib().impec_ctx_create(C.byref(P), C.c_void_p(stream) if stream else None, C.byref(h)), "ctx_create")
        self.h = h

    def close(self):
        if self.h:
            _chk(lib().impec_ctx_destroy(self.h), "ctx_destroy")
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def set_source(self, q):
        _chk(lib().impec_set_source(self.h, _p(q)), "set_source")

    def set_permeability(self, K11, K22=None):
        _chk(lib().impec_set_permeability(self.h, _p(K11), _p(K22)), "set_permeability")

    def pressure_solve(self, c, p, tol=None, check=True):
        cyc, rr = C.c_int(), C.c_double()
        s = lib().impec_pressure_solve(self.h, _p(c), _p(p), self.P.eps if tol is None else tol, C.byref(cyc),
                                       C.byref(rr))
        if check:
            _chk(s, "pressure_solve")
        return cyc.value, rr.value, s

    def face_mobility(self, c, lamx, lamy):
        _chk(lib().impec_face_mobility(self.h, _p(c), _p(lamx), _p(lamy)), "face_mobility")

    def pressure_apply(self, c, x, y):
        _chk(lib().impec_pressure_apply(self.h, _p(c), _p(x), _p(y)), "pressure_apply")

    def velocity(self, p, c, u, v):
        _chk(lib().impec_velocity(self.h, _p(p), _p(c), _p(u), _p(v)), "velocity")

    def max_stable_dt(self, u, v) -> float:
        dt = C.c_double()
        _chk(lib().impec_max_stable_dt(self.h, _p(u), _p(v), C.byref(dt)), "max_stable_dt")
        return dt.value

    def tr_integrate(self, c, dt) -> float:
        tmo = C.c_double()
        _chk(lib().impec_tr_integrate(self.h, _p(c), dt, C.byref(tmo)), "tr_integrate")
        return tmo.value

    def advect_x(self, c, u, dt):
        _chk(lib().impec_advect_x(self.h, _p(c), _p(u), dt), "advect_x")

    def advect_y(self, c, v, dt):
        _chk(lib().impec_advect_y(self.h, _p(c), _p(v), dt), "advect_y")

    def advect_split(self, c, u, v, dt, prev_first_sweep=1) -> int:
        pfs = C.c_int(prev_first_sweep)
        _chk(lib().impec_advect_split(self.h, _p(c), _p(u), _p(v), dt, C.byref(pfs)), "advect_split")
        return pfs.value

    def dispersion_cn(self, c, u, v, dt, tol=None):
        its, rr = C.c_int(), C.c_double()
        _chk(lib().impec_dispersion_cn(self.h, _p(c), _p(u), _p(v), dt, self.P.para_eps if tol is None else tol,
                                       C.byref(its), C.byref(rr)), "dispersion_cn")
        return its.value, rr.value

    def hyperbolic_solve(self, c, u, v, dt, prev_first_sweep=1, outflux=0.0):
        pfs, of = C.c_int(prev_first_sweep), C.c_double(outflux)
        _chk(lib().impec_hyperbolic_solve(self.h, _p(c), _p(u), _p(v), dt, C.byref(pfs), C.byref(of)),
             "hyperbolic_solve")
        return pfs.value, of.value

    def diagnostics(self, c, u, v):
        out = (C.c_double * 5)()
        _chk(lib().impec_diagnostics(self.h, _p(c), _p(u), _p(v), out), "diagnostics")
        return list(out)

    def state_ptrs(self):
        ps = [C.c_void_p() for _ in range(5)]
        _chk(lib().impec_state(self.h, *[C.byref(x) for x in ps]), "state")
        return [x.value for x in ps]

    def project_diagonal(self, field: int, out, dN1: int, dN2: int):
        """Project the resident c (field 0) or p (field 1) of a parallel run onto the dN1 x dN2
        diagonal grid (out: float64 CUDA tensor of dN1*dN2)."""
        _chk(lib().impec_project_diagonal(self.h, field, _p(out), dN1, dN2), "project_diagonal")

    def set_tuning(self, name: str, value: int):
        _chk(lib().impec_set_tuning(self.h, name.encode(), value), f"set_tuning({name})")

    def get_tuning(self, name: str) -> int:
        v = C.c_long()
        _chk(lib().impec_get_tuning(self.h, name.encode(), C.byref(v)), f"get_tuning({name})")
        return v.value

    def autotune(self, reps: int = 3) -> str:
        """Pick the fastest smoother schedule / cluster choice for this context's pressure solve."""
        buf = C.create_string_buffer(4096)
        _chk(lib().impec_autotune(self.h, reps, buf, len(buf)), "autotune")
        return buf.value.decode()

    def pressure_solve_resident(self, sync=True):
        cyc, rr = C.c_int(), C.c_double()
        _chk(lib().impec_pressure_solve_resident(self.h, 1 if sync else 0, C.byref(cyc), C.byref(rr)),
             "pressure_solve_resident")
        return cyc.value, rr.value

    def last_solve(self):
        """(cycles, relres, initial relres) of the last pressure solve."""
        cyc, rr, r0 = C.c_int(), C.c_double(), C.c_double()
        _chk(lib().impec_last_solve(self.h, C.byref(cyc), C.byref(rr), C.byref(r0)), "last_solve")
        return cyc.value, rr.value, r0.value

    def set_time(self, t0: float):
        _chk(lib().impec_set_time(self.h, t0), "set_time")

    def step(self, t_clip=-1.0) -> StepInfo:
        info = StepInfo()
        _chk(lib().impec_step(self.h, t_clip, C.byref(info)), "step")
        return info

    def run_steps(self, n: int) -> StepInfo:
        info = StepInfo()
        _chk(lib().impec_run_steps(self.h, n, C.byref(info)), "run_steps")
        return info

    def checkpoint_save(self, path: str):
        _chk(lib().impec_checkpoint_save(self.h, os.fsencode(path)), "checkpoint_save")

    def checkpoint_load(self, path: str):
        _chk(lib().impec_checkpoint_load(self.h, os.fsencode(path)), "checkpoint_load")

    def upload(self, c_host=None, q_host=None, ghost=2):
        import numpy as np

        def ptr(a):
            if a is None:
                return None
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
            return a.ctypes.data_as(_PD)
        _chk(lib().impec_state_upload(self.h, ptr(c_host), ptr(q_host), ghost), "state_upload")

    def download(self, c_host=None, p_host=None, v_host=None, ghost=2):
        import numpy as np

        def ptr(a):
            if a is None:
                return None
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
            return a.ctypes.data_as(_PD)
        _chk(lib().impec_state_download(self.h, ptr(c_host), ptr(p_host), ptr(v_host), ghost), "state_download")
