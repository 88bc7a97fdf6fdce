"""Synthetic workloads shared by the benchmark studies and the learned warm start: seeded
Gaussian random fields on the GPU and the heterogeneous quarter-five-spot realisations of the
batched-ensemble workload (lognormal permeability, M from {5, 20, 41, 100}, diagonal or
parallel orientation by seed)."""
from __future__ import annotations

import math

import numpy as np


def grf(N: int, ell: float, seed: int):
    """Seeded Gaussian random field on the GPU: white noise (Philox, seeded) filtered in Fourier
    space to the covariance exp(-r^2 / ell^2) (ell in cells, periodic), zero mean, unit variance."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    w = torch.randn((N, N), generator=g, device="cuda", dtype=torch.float64)
    f = torch.fft.fftfreq(N, device="cuda", dtype=torch.float64)
    H = torch.exp(-(math.pi * ell) ** 2 * (f[:, None] ** 2 + f[None, :] ** 2) / 2)
    x = torch.fft.ifft2(torch.fft.fft2(w) * H).real
    return ((x - x.mean()) / x.std()).contiguous()


def realisation(E, N: int, seed: int, precision: str = "mixed", ell: float = 16.0, sigma: float = 0.5,
                warm_start: int = 0):
    """One heterogeneous quarter-five-spot realisation: lognormal K (sigma, correlation ell
    cells), M = (5, 20, 41, 100)[seed % 4], diagonal (unit square, injector and producer in
    opposite corner cells) or parallel (sqrt 2 square, four corner wells) when (seed // 4) is odd;
    MUSCL + Peaceman dispersion (alpha_l 1e-3, alpha_t 1e-4), porosity 1, CFL 0.5, FP64
    transport, pressure to 1e-10 in the given precision.  Returns a Context at t = 0, c = 0."""
    M = (5.0, 20.0, 41.0, 100.0)[seed % 4]
    parallel = (seed // 4) % 2 == 1
    L = math.sqrt(2.0) if parallel else 1.0
    P = E.default_params(N, N, x_ub=L, y_ub=L, stype=E.PARALLEL if parallel else E.DIAGONAL, hmtype=E.MUSCL,
                         nu=1.0, diffusion=1, alpha_l=1e-3, alpha_t=1e-4, cfl=0.5, porosity=1.0, eps=1e-10,
                         para_eps=1e-10, mu_res=M, mu_inj=1.0, max_cycles=200, warm_start=warm_start,
                         precision=E.PREC_MIXED if precision == "mixed" else E.PREC_FP64)
    ctx = E.Context(P)
    dx = L / N
    qv = 1.0 / (dx * dx)
    q = np.zeros(N * N)
    q[0] = qv
    if parallel:
        q[-1], q[N - 1], q[(N - 1) * N] = qv, -qv, -qv
    else:
        q[-1] = -qv
    import torch
    K = torch.exp(sigma * grf(N, ell, 5000 + seed)).contiguous()
    ctx.upload(np.zeros((N + 4, N + 4)), q, ghost=2)
    ctx.set_permeability(K, K)
    ctx.set_time(0.0)
    return ctx


class _Dev:
    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


def device_view(ptr: int, shape, dtype: str = "<f8"):
    """A torch view (no copy) of device memory owned by the engine, e.g. Context.state_ptrs()."""
    import torch
    return torch.as_tensor(_Dev(ptr, shape, dtype), device="cuda")
