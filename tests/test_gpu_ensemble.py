"""Ensembles (one graph launch advances every member) and the per-context tuning / autotuner."""
import numpy as np
import pytest

from helpers import dev, host, oparams, smooth_field, source

pytestmark = pytest.mark.gpu

SPECS = [
    (48, 48, dict(stype=1, hmtype=4, nu=1.0)),
    (64, 40, dict(stype=1, hmtype=0, nu=2.0 / 3.0, diffusion=1, alpha_l=1e-2, alpha_t=1e-3)),
    (40, 40, dict(stype=0, hmtype=4, nu=1.0, diffusion=1, alpha_l=1e-3, alpha_t=1e-4)),
    (56, 48, dict(stype=2, hmtype=4, nu=1.0)),
]


def _member(E, N1, N2, kw, precision=0):
    P = E.default_params(N1, N2, precision=precision, **kw)
    ctx = E.Context(P)
    ctx.upload(np.zeros((N1 + 4, N2 + 4)), source(oparams(P)), ghost=2)
    ctx.set_time(0.0)
    return ctx


@pytest.mark.parametrize("precision", [0, 1])
def test_ensemble_matches_members_stepped_alone(engine, precision):
    """Every member of an ensemble ends bit-identical to the same realisation stepped alone:
    the members' graph branches share no buffer, scalar or reduction scratch."""
    E = engine
    ens_members = [_member(E, N1, N2, kw, precision) for N1, N2, kw in SPECS]
    solo = [_member(E, N1, N2, kw, precision) for N1, N2, kw in SPECS]
    ens = E.Ensemble(ens_members)
    ens.step(3)
    ens.step(2, sync=False)
    for ctx in solo:
        for _ in range(5):
            ctx.step()
    for (N1, N2, _), a, b in zip(SPECS, ens_members, solo):
        ca, pa = np.zeros((N1 + 4, N2 + 4)), np.zeros((N1 + 4, N2 + 4))
        cb, pb = np.zeros_like(ca), np.zeros_like(pa)
        a.download(ca, pa, None, ghost=2)
        b.download(cb, pb, None, ghost=2)
        assert np.array_equal(ca, cb) and np.array_equal(pa, pb)
        assert ca.max() > 0.0  # the members did advance
    ens.close()


def test_ensemble_rejects_duplicates_and_alternating_sweeps(engine):
    E = engine
    a = _member(E, 32, 32, dict(stype=1))
    with pytest.raises(E.ImpecError):
        E.Ensemble([a, a])
    b = _member(E, 32, 32, dict(stype=1, dim_splitting=0))
    with pytest.raises(E.ImpecError):
        E.Ensemble([b])


def test_tuning_and_autotune(engine):
    """Tunables are per context; the autotuner keeps the fastest schedule, and the solve with it
    still reaches the tolerance."""
    E = engine
    import torch
    N = 200
    ctx = _member(E, N, N, dict(stype=1, nu=1.0, eps=1e-10))
    c = torch.from_numpy(smooth_field(N, N, 3)).cuda()
    assert ctx.get_tuning("mg_pre") == 1 and ctx.get_tuning("mg_post") == 2  # five-point default V(1,2)
    ctx.set_tuning("mg_pre", 1)
    assert ctx.get_tuning("mg_pre") == 1
    with pytest.raises(E.ImpecError):
        ctx.set_tuning("no_such_knob", 1)
    ctx.set_tuning("mg_post", 0)
    with pytest.raises(E.ImpecError):
        ctx.set_tuning("mg_pre", 0)  # at least one sweep in the cycle
    ctx.set_tuning("mg_post", 2)
    ctx.set_tuning("mg_pre", 2)
    report = ctx.autotune(reps=2)
    assert "chosen:" in report and report.count("iterations") >= 4
    p = torch.zeros((N, N), dtype=torch.float64, device="cuda")
    cyc, rr, _ = ctx.pressure_solve(c, p, 1e-10)
    assert rr <= 1e-10


def test_ensemble_members_keep_their_buffers(engine):
    """While an ensemble's graph holds a member's buffers, calls that would free or move them
    are refused (the graph would read freed memory); in-place permeability updates pass."""
    import numpy as np
    import torch
    from impec2d_gb300.workloads import realisation
    E = engine
    a, b = realisation(E, 64, 1), realisation(E, 64, 2)
    ens = E.Ensemble([a, b])
    net = E.Net(seed=0)
    with pytest.raises(E.ImpecError):
        a.close()
    assert a.h is not None
    with pytest.raises(E.ImpecError):
        net.attach(a, factor=1, mode=2)
    q = np.zeros(64 * 64)
    q[5], q[-7] = 1.0, -1.0
    with pytest.raises(E.ImpecError):
        a.set_source(torch.from_numpy(q).cuda())
    K = torch.full((64, 64), 2.0, dtype=torch.float64, device="cuda")
    a.set_permeability(K, K)  # same layout: in place
    ens.step(1)
    ens.close()
    a.close()
    b.close()
    net.close()


def test_ensemble_with_learned_members_matches_solo(engine):
    """Members with the learned initial guess attached (one shared network) run their hooks
    (features, forward pass, step along the prediction) inside the ensemble graph's parallel
    branches and end bit-identical to the same members stepped alone."""
    from impec2d_gb300.workloads import realisation
    E = engine
    net = E.Net(seed=11)
    specs = [(64, 3), (128, 4), (64, 5)]
    ens_members = [realisation(E, N, s, warm_start=1) for N, s in specs]
    solo = [realisation(E, N, s, warm_start=1) for N, s in specs]
    for cx in ens_members + solo:
        cx.run_steps(2)
        net.attach(cx, factor=1, mode=1)
    ens = E.Ensemble(ens_members)
    ens.step(4)
    for cx in solo:
        for _ in range(4):
            info = cx.step()
            assert info.relres <= 1e-10
    for (N, _), a, b in zip(specs, ens_members, solo):
        ca, pa = np.zeros((N + 4, N + 4)), np.zeros((N + 4, N + 4))
        cb, pb = np.zeros_like(ca), np.zeros_like(pa)
        a.download(ca, pa, None, ghost=2)
        b.download(cb, pb, None, ghost=2)
        assert np.array_equal(ca, cb) and np.array_equal(pa, pb)
        assert E.Net.last_alpha(a) == E.Net.last_alpha(b)
    ens.close()
    for cx in ens_members + solo:
        E.Net.detach(cx)
        cx.close()
    net.close()
