"""Failure paths, made on the host or with bounded waits only (no GPU fault, trap or hang):
a NaN in the concentration surfaces as IMPEC_ERR_NAN; a cycle limit below what the tolerance
needs surfaces as IMPEC_ERR_NOT_CONVERGED; a bounded mbarrier wait that nothing completes gives
up and reports instead of hanging.  After each, the same context (or the device) keeps working:
a clean state steps normally."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from helpers import cell_ghost, oparams, source

pytestmark = pytest.mark.gpu


def _ctx(E, N, **kw):
    P = E.default_params(N, N, stype=E.DIAGONAL, hmtype=E.MUSCL, eps=1e-10, para_eps=1e-10, **kw)
    ctx = E.Context(P)
    OP = oparams(P)
    return P, OP, ctx


@pytest.mark.parametrize("graph", ["1", "0"])
def test_nan_in_concentration_is_reported(engine, monkeypatch, graph):
    E = engine
    monkeypatch.setenv("IMPEC_NO_GRAPH", "0" if graph == "1" else "1")
    P, OP, ctx = _ctx(E, 48)
    q = source(OP)
    c = np.zeros((48, 48))
    c[20, 17] = np.nan
    ctx.upload(cell_ghost(OP, c), q, ghost=2)
    ctx.set_time(0.0)
    with pytest.raises(E.ImpecError) as ei:
        ctx.step()
    assert ei.value.status == 4, ei.value  # IMPEC_ERR_NAN
    # the context stays usable: a clean state steps and converges
    ctx.upload(cell_ghost(OP, np.zeros((48, 48))), q, ghost=2)
    ctx.set_time(0.0)
    info = ctx.step()
    assert info.relres <= 1e-10 and np.isfinite(info.dt)
    ctx.close()


@pytest.mark.parametrize("graph", ["1", "0"])
def test_cycle_limit_is_reported(engine, monkeypatch, graph):
    E = engine
    monkeypatch.setenv("IMPEC_NO_GRAPH", "0" if graph == "1" else "1")
    P, OP, ctx = _ctx(E, 64, max_cycles=1)
    q = source(OP)
    ctx.upload(cell_ghost(OP, np.zeros((64, 64))), q, ghost=2)
    ctx.set_time(0.0)
    with pytest.raises(E.ImpecError) as ei:
        ctx.step()
    assert ei.value.status == 3, ei.value  # IMPEC_ERR_NOT_CONVERGED
    assert "max_cycles" in E.last_error()
    ctx.close()
    P, OP, ctx = _ctx(E, 64, max_cycles=200)
    ctx.upload(cell_ghost(OP, np.zeros((64, 64))), q, ghost=2)
    ctx.set_time(0.0)
    assert ctx.step().relres <= 1e-10
    ctx.close()


def test_pressure_solve_cycle_limit_status(engine):
    """The direct entry point reports the limit as a status and still returns its best iterate."""
    import torch
    from helpers import dev
    E = engine
    P, OP, ctx = _ctx(E, 64, max_cycles=2)
    ctx.set_source(dev(source(OP)))
    p = torch.zeros((64, 64), dtype=torch.float64, device="cuda")
    cyc, rr, st = ctx.pressure_solve(dev(np.zeros((64, 64))), p, 1e-12, check=False)
    assert st == 3 and cyc == 2 and rr > 1e-12 and np.isfinite(rr)
    ctx.close()


def test_bounded_wait_gives_up_and_reports(engine):
    E = engine
    out = C.c_int(-1)
    # nothing arrives: the wait runs out after 4096 polls and says so
    assert E.lib().impec_selftest_bounded_wait(4096, 0, C.byref(out)) == 0, E.last_error()
    assert out.value == 1
    # the positive control completes
    assert E.lib().impec_selftest_bounded_wait(4096, 1, C.byref(out)) == 0
    assert out.value == 0
    # limits outside [1, 2^20] are refused on the host
    assert E.lib().impec_selftest_bounded_wait(0, 0, C.byref(out)) == 1
    assert E.lib().impec_selftest_bounded_wait((1 << 20) + 1, 0, C.byref(out)) == 1
    # and the device keeps working
    P, OP, ctx = _ctx(E, 32)
    ctx.upload(cell_ghost(OP, np.zeros((32, 32))), source(OP), ghost=2)
    ctx.set_time(0.0)
    assert ctx.step().relres <= 1e-10
    ctx.close()
