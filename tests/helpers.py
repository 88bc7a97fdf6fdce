"""Layout conversions between the oracle (reference ghost layouts) and the engine (device,
ghost-free) plus comparison helpers.  Test infrastructure."""
import ctypes as C

import numpy as np

import oracle as O


def oparams(P, **kw):
    """Oracle parameters equivalent to engine parameters P."""
    d = dict(N1=P.N1, N2=P.N2, x_lb=P.x_lb, x_ub=P.x_ub, y_lb=P.y_lb, y_ub=P.y_ub, mu_res=P.mu_res,
             mu_inj=P.mu_inj, avgproc=P.avgproc, nu=P.nu, porosity=P.porosity, cfl=P.cfl,
             inj_fluid_conc=P.inj_fluid_conc, I=P.I, diffusion=P.diffusion, alpha_l=P.alpha_l,
             alpha_t=P.alpha_t, Dm=P.Dm, ptype=P.ptype, dt_diff_limit=P.dt_diff_limit,
             dim_splitting=P.dim_splitting, hmtype=P.hmtype, stype=P.stype, is_test=P.is_test,
             testno=P.testno, eps=P.eps, para_eps=P.para_eps, peaceman_guard=P.peaceman_guard)
    d.update(kw)
    return O.make_params(**d)


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def cell_ghost(OP, interior, periodic=False):
    return O.with_ghosts(OP, interior, "periodic" if periodic else "neumann")


def vel_ghost(OP, u, v):
    """Reference velocity array from device-layout u ((N1+1),N2) and v (N1,(N2+1)), ghosts filled."""
    g = OP.g
    a = np.zeros(O.vel_shape(OP))
    a[g:g + OP.N1 + 1, g:g + OP.N2, 0] = u
    a[g:g + OP.N1, g:g + OP.N2 + 1, 1] = v
    O.lib().or_fill_velocity_neumann(C.byref(OP), O.ptr(a))
    return a


def vel_split(OP, a):
    g = OP.g
    return (np.ascontiguousarray(a[g:g + OP.N1 + 1, g:g + OP.N2, 0]),
            np.ascontiguousarray(a[g:g + OP.N1, g:g + OP.N2 + 1, 1]))


def rel_err(a, b):
    """max |a-b| / max |b| (0 if both vanish)."""
    a, b = np.asarray(a), np.asarray(b)
    s = np.abs(b).max()
    d = np.abs(a - b).max()
    return d / s if s > 0 else d


def smooth_field(N1, N2, seed, lo=0.0, hi=1.0):
    """Seeded smooth random field in [lo, hi] (sum of a few Fourier modes)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(N1)[:, None] + 0.5) / N1
    y = (np.arange(N2)[None, :] + 0.5) / N2
    f = np.zeros((N1, N2))
    for _ in range(6):
        kx, ky = rng.integers(1, 5, 2)
        f += rng.normal() * np.cos(np.pi * kx * x + rng.uniform(0, 6)) * np.cos(np.pi * ky * y + rng.uniform(0, 6))
    f = (f - f.min()) / (f.max() - f.min() + 1e-300)
    return lo + (hi - lo) * f


def source(OP):
    q = np.zeros(OP.N1 * OP.N2)
    O.lib().or_init_source(C.byref(OP), O.ptr(q), 0.0)
    return q
