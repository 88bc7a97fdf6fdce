"""Binary checkpoint of a resident run (impec_checkpoint_save / impec_checkpoint_load).

A run of six steps and a run of three steps, a checkpoint, a fresh context restored from it and
three more steps must end with the same concentration, pressure, velocities, clock and step
counter, bit for bit.  The pressure solve starts from the previous pressure (warm start) and the
splitting alternates its sweep order, so the restored pressure and sweep order are both read by
the steps after the restart.  Loading refuses a file of another grid size, a damaged file and a
missing one, with IMPEC_ERR_ARG and a message, and leaves the context usable."""
import os

import numpy as np
import pytest

from helpers import cell_ghost, oparams, source

pytestmark = pytest.mark.gpu


def _fingers(N, seed=3):
    rng = np.random.default_rng(seed)
    i = (np.arange(N)[:, None] + 0.5) / N
    j = (np.arange(N)[None, :] + 0.5) / N
    r = np.minimum(np.hypot(i, j), np.hypot(1 - i, 1 - j))
    front = 0.3 + 0.02 * rng.standard_normal((N, N))
    return 1.0 / (1.0 + np.exp((r - front) / 0.02))


def _run(E, N, **kw):
    P = E.default_params(N, N, stype=E.PARALLEL, x_ub=2 ** 0.5, y_ub=2 ** 0.5, hmtype=E.MUSCL, diffusion=1,
                         alpha_l=1e-3, alpha_t=1e-4, dim_splitting=E.ALTERNATING, eps=1e-10, para_eps=1e-10,
                         max_cycles=200, **kw)
    P.warm_start = 1
    ctx = E.Context(P)
    OP = oparams(P)
    q = source(OP)
    ctx.upload(cell_ghost(OP, _fingers(N)), q, ghost=2)
    ctx.set_time(0.0)
    return ctx, OP, q


def _state(ctx, OP):
    shape = (OP.N1 + 4, OP.N2 + 4)
    c, p = np.zeros(shape), np.zeros(shape)
    v = np.zeros((OP.N1 + 5, OP.N2 + 5, 2))
    ctx.download(c, p, v, ghost=2)
    return c, p, v


def test_checkpoint_restart_continues_bit_for_bit(engine, tmp_path):
    E = engine
    N = 96
    path = str(tmp_path / "run.ckpt")
    a, OP, _ = _run(E, N)
    for _ in range(3):
        a.step()
    a.checkpoint_save(path)
    for _ in range(3):
        ia = a.step()
    ca, pa, va = _state(a, OP)
    b, _, _ = _run(E, N)
    b.checkpoint_load(path)
    for _ in range(3):
        ib = b.step()
    cb, pb, vb = _state(b, OP)
    assert ib.t == ia.t and ib.dt == ia.dt and ib.counter == ia.counter == 6
    assert ib.prev_first_sweep == ia.prev_first_sweep
    assert ib.total_outflux == ia.total_outflux and ib.mass_err == ia.mass_err
    assert np.array_equal(ca, cb) and np.array_equal(pa, pb) and np.array_equal(va, vb)
    a.close()
    b.close()


def test_checkpoint_load_rejects_bad_files(engine, tmp_path):
    E = engine
    path = str(tmp_path / "run.ckpt")
    a, OP, _ = _run(E, 64)
    a.step()
    a.checkpoint_save(path)
    other, _, _ = _run(E, 48)
    with pytest.raises(E.ImpecError) as ei:
        other.checkpoint_load(path)
    assert ei.value.status == 1 and "48x48" in E.last_error()
    data = bytearray(open(path, "rb").read())
    data[len(data) // 2] ^= 0x40  # one flipped bit in the payload
    bad = str(tmp_path / "bad.ckpt")
    open(bad, "wb").write(bytes(data))
    with pytest.raises(E.ImpecError) as ei:
        a.checkpoint_load(bad)
    assert ei.value.status == 1 and "checksum" in E.last_error()
    with pytest.raises(E.ImpecError):
        a.checkpoint_load(os.path.join(str(tmp_path), "missing.ckpt"))
    assert a.step().relres <= 1e-10  # the context still steps
    a.close()
    other.close()
