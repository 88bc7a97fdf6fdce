"""The allocation-free transport step (impec_advect_symmetric_noalloc).

Some callers cannot allocate device memory: they run inside a host framework that owns every
device allocation, or must not trigger cudaMalloc's device-wide synchronisation, so they cannot
create a context.  This entry point serves them from a static device scratch array.  Its result
must match the context path (impec_advect_split, symmetric-parallel splitting) to 1e-13 of the
field maximum, on two calls in a row (the second call sees the scratch left by the first), and
it must reject grids larger than its scratch and splittings other than symmetric-parallel.
A call must also leave the device's free memory unchanged, on the NULL stream and on a
stream of the caller's own.  Collected last on purpose: it runs after every
other GPU test and also alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _smooth(n1, n2, seed, lo, hi):
    rng = np.random.default_rng(seed)
    x = (np.arange(n1)[:, None] + 0.5) / n1
    y = (np.arange(n2)[None, :] + 0.5) / n2
    f = np.zeros((n1, n2))
    for _ in range(5):
        kx, ky = rng.integers(1, 4, 2)
        f += rng.normal() * np.cos(np.pi * kx * x + rng.uniform(0, 6)) * np.cos(np.pi * ky * y + rng.uniform(0, 6))
    f = (f - f.min()) / (f.max() - f.min())
    return lo + (hi - lo) * f


def _call_noalloc(E, P, c, u, v, dt, stream=None):
    return E.lib().impec_advect_symmetric_noalloc(C.byref(P), C.c_void_p(c.data_ptr()), C.c_void_p(u.data_ptr()),
                                                  C.c_void_p(v.data_ptr()), dt, stream)


@pytest.mark.parametrize("scheme,bc,own_stream", [("muscl", "neumann", False), ("upwind", "neumann", False),
                                                  ("muscl", "periodic", True)])
def test_noalloc_matches_context_path_on_two_calls(engine, scheme, bc, own_stream):
    import torch
    E = engine
    N1, N2 = 96, 80
    hm = E.MUSCL if scheme == "muscl" else E.UPWINDSPLIT
    P = E.default_params(N1, N2, hmtype=hm, porosity=0.7, dim_splitting=E.SYMMETRIC_PARALLEL)
    if bc == "periodic":
        P.bc = E.BC_PERIODIC
    ctx = E.Context(P)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    c = dev(_smooth(N1, N2, 1, 0.0, 1.0))
    u = dev(_smooth(N1 + 1, N2, 2, -1.0, 1.0))
    v = dev(_smooth(N1, N2 + 1, 3, -1.0, 1.0))
    dx = 1.0 / N1
    dt = 0.4 * P.porosity * dx / max(float(u.abs().max()), float(v.abs().max()))
    c_ctx, c_na = c.clone(), c.clone()
    stream = torch.cuda.Stream() if own_stream else None
    handle = C.c_void_p(stream.cuda_stream) if own_stream else None
    # One call on a scratch copy first: the library's module and the symbol lookup may take
    # device memory once per process; what is checked below is that a call itself takes none.
    warm = c.clone()
    assert _call_noalloc(E, P, warm, u, v, dt, handle) == 0, E.last_error()
    torch.cuda.synchronize()
    for call in range(2):
        ctx.advect_split(c_ctx, u, v, dt, 1)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = _call_noalloc(E, P, c_na, u, v, dt, handle)
        assert st == 0, E.last_error()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before, "the allocation-free step changed free device memory"
        ref = c_ctx.cpu().numpy()
        got = c_na.cpu().numpy()
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max(), (call, np.abs(got - ref).max())
    ctx.close()


def test_noalloc_rejects_other_splittings(engine):
    import torch
    E = engine
    P = E.default_params(64, 64, dim_splitting=E.STRANG)
    c = torch.zeros(4, dtype=torch.float64, device="cuda")  # never touched: rejected before any launch
    assert _call_noalloc(E, P, c, c, c, 1e-3) == 1 and "symmetric-parallel" in E.last_error()


def test_noalloc_rejects_grids_beyond_its_scratch(engine):
    import torch
    E = engine
    P = E.default_params(1025, 1024)  # 1,049,600 cells > 1,048,576
    c = torch.zeros(4, dtype=torch.float64, device="cuda")  # never touched: rejected before any launch
    st = E.lib().impec_advect_symmetric_noalloc(C.byref(P), C.c_void_p(c.data_ptr()), C.c_void_p(c.data_ptr()),
                                                C.c_void_p(c.data_ptr()), 1e-3, None)
    assert st == 1 and "1048576" in E.last_error()
