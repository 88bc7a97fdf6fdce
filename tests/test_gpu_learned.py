"""Tensor-core (tcgen05) kernels of the learned warm start against fp32 references of the same
bf16 inputs.  Tolerances: fp32 accumulation in a different order, relative 1e-5 of the
largest |C|."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def _gemm(E, A, B):
    import torch
    M, K = A.shape
    N = B.shape[0]
    out = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    s = E.lib().impec_gemm_bf16(C.c_void_p(A.data_ptr()), A.stride(0), C.c_void_p(B.data_ptr()), B.stride(0),
                                C.c_void_p(out.data_ptr()), out.stride(0), M, N, K, None)
    assert s == 0, E.last_error()
    return out


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (128, 128, 256), (300, 200, 192), (1024, 256, 576)])
def test_gemm_bf16_matches_fp32_reference(engine, M, N, K):
    import torch
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn((N, K), generator=g, device="cuda").to(torch.bfloat16)
    got = _gemm(engine, A, B)
    ref = A.float() @ B.float().T
    assert torch.isfinite(got).all()
    assert (got - ref).abs().max().item() <= 1e-5 * ref.abs().max().item() + 1e-6


def _vp(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _conv_setup(B, H, W, cin, cout, seed):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    X = torch.randn((B, H, W, cin), generator=g, device="cuda").to(torch.bfloat16)
    Kp = (9 * cin + 63) // 64 * 64
    Wt = torch.zeros((cout, Kp), device="cuda", dtype=torch.bfloat16)
    Wt[:, :9 * cin] = (torch.randn((cout, 9 * cin), generator=g, device="cuda") / (3.0 * cin ** 0.5)).to(torch.bfloat16)
    bias = torch.randn(cout, generator=g, device="cuda") * 0.1
    return X, Wt, bias


def _w4(Wt, cin, cout):
    """(cout, Kp) with k = tap * cin + c, tap = 3 (dy + 1) + (dx + 1)  ->  conv2d weights (cout, cin, 3, 3)."""
    return Wt[:, :9 * cin].float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2).contiguous()


@pytest.mark.parametrize("B,H,W,cin,cout", [
    # cp.async staging: 8 channels, or widths that do not tile 128 pixels
    (2, 20, 20, 8, 32), (1, 37, 29, 32, 64), (2, 16, 24, 64, 256), (1, 12, 12, 128, 128),
    # TMA staging: rows of 128 pixels, several rows per box, whole images per box; 32 / 64 channel stages
    (1, 64, 128, 32, 32), (1, 16, 256, 64, 64), (2, 16, 16, 64, 128), (1, 8, 8, 32, 64), (3, 4, 4, 256, 256),
    (2, 32, 32, 128, 256),
    # one halo box for the 9 taps (cin 32 / 64, rows of 128 pixels): 8 outputs, two channel tiles,
    # several images of two rows
    (2, 8, 128, 32, 8), (1, 4, 256, 64, 128), (3, 2, 128, 64, 32),
    # 8 input channels: halo boxes padded to 16 channels; weight gradients on 32-channel boxes
    (2, 4, 128, 8, 32), (1, 8, 256, 8, 64)])
def test_conv3x3_forward_and_gradients(engine, B, H, W, cin, cout):
    """Implicit-GEMM convolution on tcgen05: forward (linear; GELU with a skip add), input
    gradient (plain; times gelu'(z) with an added gradient) and weight gradient, against
    PyTorch fp32 conv2d / autograd of the same bf16 inputs.  Shapes cover both operand
    stagings (cp.async gathers and TMA boxes with zero-filled halos)."""
    import torch
    import torch.nn.functional as F
    E = engine
    L = E.lib()
    X, Wt, bias = _conv_setup(B, H, W, cin, cout, B * 1000 + cin * 10 + cout)
    w4 = _w4(Wt, cin, cout)
    x = X.float().permute(0, 3, 1, 2).contiguous().requires_grad_(True)
    z_ref = F.conv2d(x, w4, bias, padding=1)
    zf = torch.empty((B, H, W, cout), device="cuda")
    assert L.impec_conv3x3_forward(_vp(X), B, H, W, cin, _vp(Wt), _vp(bias), cout, 0, None, None, _vp(zf), None,
                                   None) == 0, E.last_error()
    zr = z_ref.detach().permute(0, 2, 3, 1)
    scale = zr.abs().max().item()
    assert (zf - zr).abs().max().item() <= 2e-5 * scale + 1e-6
    # GELU + skip, bf16 outputs
    skip = torch.randn((B, H, W, cout), device="cuda").to(torch.bfloat16)
    Z = torch.empty((B, H, W, cout), device="cuda", dtype=torch.bfloat16)
    Y = torch.empty_like(Z)
    assert L.impec_conv3x3_forward(_vp(X), B, H, W, cin, _vp(Wt), _vp(bias), cout, 1, _vp(Z), _vp(Y), None, _vp(skip),
                                   None) == 0, E.last_error()
    y_ref = F.gelu(zr) + skip.float()
    assert (Z.float() - zr).abs().max().item() <= 1e-2 * scale
    assert (Y.float() - y_ref).abs().max().item() <= 1e-2 * (y_ref.abs().max().item() + 1)
    # gradients
    dZ = (torch.randn((B, H, W, cout), device="cuda") * 0.5).to(torch.bfloat16)
    z_ref.backward(dZ.float().permute(0, 3, 1, 2))
    dx_ref = x.grad.permute(0, 2, 3, 1)
    dxf = torch.empty((B, H, W, cin), device="cuda")
    assert L.impec_conv3x3_input_grad(_vp(dZ), B, H, W, cout, _vp(Wt), cin, None, None, None, _vp(dxf), None) == 0, \
        E.last_error()
    assert (dxf - dx_ref).abs().max().item() <= 2e-5 * dx_ref.abs().max().item() + 1e-6
    gz = torch.randn((B, H, W, cin), device="cuda").to(torch.bfloat16)
    add = torch.randn((B, H, W, cin), device="cuda").to(torch.bfloat16)
    dgf = torch.empty((B, H, W, cin), device="cuda")
    assert L.impec_conv3x3_input_grad(_vp(dZ), B, H, W, cout, _vp(Wt), cin, _vp(gz), _vp(add), None, _vp(dgf),
                                      None) == 0, E.last_error()
    gzf = gz.float()
    gelu_d = 0.5 * (1 + torch.erf(gzf / 2 ** 0.5)) + gzf * torch.exp(-0.5 * gzf * gzf) / (2 * torch.pi) ** 0.5
    dg_ref = (dx_ref + add.float()) * gelu_d
    assert (dgf - dg_ref).abs().max().item() <= 1e-4 * dg_ref.abs().max().item() + 1e-5
    Kp = Wt.shape[1]
    dW = torch.zeros((cout, Kp), device="cuda")
    assert L.impec_conv3x3_weight_grad(_vp(dZ), _vp(X), B, H, W, cin, cout, _vp(dW), None) == 0, E.last_error()
    dw_ref = torch.zeros_like(dW)
    dw_ref[:, :9 * cin] = torch.autograd.grad(
        F.conv2d(X.float().permute(0, 3, 1, 2), w4.requires_grad_(True), None, padding=1),
        w4, dZ.float().permute(0, 3, 1, 2))[0].permute(0, 2, 3, 1).reshape(cout, 9 * cin)
    assert (dW - dw_ref).abs().max().item() <= 2e-5 * dw_ref.abs().max().item() + 1e-5


def test_net_gradients_match_the_cpu_oracle(engine):
    """Forward + backward of the whole encoder-decoder on the tensor cores against the CPU
    restatement (oracle/learned_ref.py, bf16 rounding where the GPU stores bf16): loss and every
    layer's weight and bias gradients."""
    import numpy as np
    import torch
    from oracle import learned_ref as R
    E = engine
    net = E.Net(seed=3)
    H = W = 16
    g = torch.Generator(device="cuda").manual_seed(5)
    X = torch.zeros((1, H, W, 8), device="cuda")
    X[..., :4] = torch.randn((1, H, W, 4), generator=g, device="cuda")
    X = X.to(torch.bfloat16)
    T = torch.randn((1, H, W), generator=g, device="cuda")
    loss = net.backprop(X, T)
    grads = net.parameters(which=1)
    params = net.parameters(which=0)
    loss_ref, grads_ref = R.forward_backward(params, X[0].float().cpu().numpy(), T[0].cpu().numpy())
    assert abs(loss - loss_ref) <= 1e-3 * abs(loss_ref)
    off = 0
    for l, (cin, cout, *_) in enumerate(R.LAYERS):
        n = cout * R.kp(cin) + cout
        a, b = grads[off:off + n], grads_ref[off:off + n]
        assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b) + 1e-12, (l, np.linalg.norm(a - b), np.linalg.norm(b))
        off += n
    net.close()


def test_net_training_reduces_the_loss(engine):
    """AdamW steps on a fixed batch drive its loss down (the target is a smooth function of the
    input channels)."""
    import torch
    E = engine
    net = E.Net(seed=1)
    B, H, W = 4, 32, 32
    g = torch.Generator(device="cuda").manual_seed(9)
    X = torch.zeros((B, H, W, 8), device="cuda")
    X[..., :4] = torch.randn((B, H, W, 4), generator=g, device="cuda")
    T = (0.5 * X[..., 3] + 0.25 * torch.tanh(X[..., 0])).contiguous()
    X = X.to(torch.bfloat16)
    first = net.train_batch(X, T, lr=1e-3)
    for _ in range(60):
        last = net.train_batch(X, T, lr=1e-3)
    assert last < 0.2 * first
    out = net.forward(X)
    assert torch.isfinite(out).all()
    net.close()


def _member(E, N, seed, warm_start=1):
    from impec2d_gb300.workloads import realisation
    return realisation(E, N, seed, precision="mixed", ell=8.0, warm_start=warm_start)


def test_learned_record_mode_leaves_the_solve_unchanged(engine):
    """Recording features and targets does not move the initial iterate: the run is bit-identical
    to the same run without the hook; the features and targets have their stated normalisation."""
    import numpy as np
    import torch
    E = engine
    N, f = 64, 2
    a, b = _member(E, N, 1), _member(E, N, 1)
    rec = E.Net(seed=0)
    rec.attach(b, factor=f, mode=2)
    h = N // f
    X = torch.empty((h, h, 8), dtype=torch.bfloat16, device="cuda")
    T = torch.empty((h, h), dtype=torch.float32, device="cuda")
    for _ in range(5):
        ia, ib = a.step(), b.step()
        assert ia.its == ib.its and ia.relres == ib.relres
    E.Net.last_features(b, X)
    E.Net.last_target(b, T)
    out = []
    for cx in (a, b):
        ch, ph = np.zeros((N + 4, N + 4)), np.zeros((N + 4, N + 4))
        cx.download(ch, ph, None, ghost=2)
        out.append((ch, ph))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    x = X.float()
    assert (x[..., 5:] == 0).all()
    assert abs(float(x[..., 2].sum())) < 1e-3 and float(x[..., 2].max()) == 1.0  # injector +1, producer -1
    assert abs(float(x[..., 3].mean())) < 2e-2 and abs(float(x[..., 3].pow(2).mean().sqrt()) - 1) < 2e-2
    assert abs(float(x[..., 4].pow(2).mean().sqrt()) - 1) < 2e-2
    assert abs(float(T.mean())) < 1e-4 and abs(float(T.pow(2).mean().sqrt()) - 1) < 1e-4
    with pytest.raises(E.ImpecError):
        rec.close()  # still attached
    E.Net.detach(b)
    rec.close()
    a.close()
    b.close()


def test_learned_guess_keeps_the_solve_converging(engine):
    """An attached (untrained) network only moves the initial iterate along its prediction by
    the A-norm-optimal step: every solve still reaches 1e-10."""
    import math
    E = engine
    N = 64
    ctx = _member(E, N, 2)
    net = E.Net(seed=2)
    ctx.run_steps(2)
    net.attach(ctx, factor=1, mode=1)
    for _ in range(4):
        info = ctx.step()
        assert info.relres <= 1e-10
        assert math.isfinite(E.Net.last_alpha(ctx))
    E.Net.detach(ctx)
    net.close()
    ctx.close()


def test_learned_attach_rejections(engine):
    E = engine
    net = E.Net(seed=0)
    ctx = _member(E, 64, 3, warm_start=0)
    with pytest.raises(E.ImpecError):
        net.attach(ctx, factor=1, mode=1)  # no warm start
    ctx.close()
    ctx = _member(E, 72, 3)
    with pytest.raises(E.ImpecError):
        net.attach(ctx, factor=2, mode=1)  # 72 / 2 is not a multiple of 8
    with pytest.raises(E.ImpecError):
        net.attach(ctx, factor=3, mode=1)
    ctx.close()
    net.close()


def test_trained_network_saves_cycles_over_the_previous_step(engine):
    """What the learned part gains: a network trained (AdamW, the engine's kernels) on pairs that
    the solver wrote from 64^2 realisations starts held-out solves closer to the solution than
    the previous pressure alone, so they need fewer V-cycles to the same 1e-10 (counted over the
    same IMPES steps of three held-out realisations run side by side)."""
    from impec2d_gb300 import learned as LW
    from impec2d_gb300.workloads import realisation
    E = engine
    N, ell = 64, 4.0
    X, T, _ = LW.generate_pairs(E, 16, 40, N=N, every=2, skip=2, ell=ell)
    net = E.Net(seed=5)
    v0 = LW.validation_mse(net, X[:40], T[:40])
    LW.train(net, X[40:], T[40:], epochs=25, batch=32, lr=1e-3, weight_decay=1e-4, evals=1)
    v1 = LW.validation_mse(net, X[:40], T[:40])
    assert v1 < 0.5 * v0, (v0, v1)
    its = {"previous": 0, "learned": 0}
    for seed in (100, 101, 102):
        runs = {k: realisation(E, N, seed, precision="mixed", ell=ell, warm_start=1) for k in its}
        for cx in runs.values():
            cx.run_steps(3)
        net.attach(runs["learned"], factor=1, mode=1)
        for _ in range(12):
            for k, cx in runs.items():
                info = cx.step()
                assert info.relres <= 1e-10
                its[k] += info.its
        E.Net.detach(runs["learned"])
        for cx in runs.values():
            cx.close()
    print(f"validation MSE {v0:.3f} -> {v1:.3f}; V-cycles over 36 solves: {its}")
    assert its["learned"] < its["previous"], its
    net.close()


@pytest.mark.parametrize("factor", [1, 2])
def test_learned_features_match_a_recomputation(engine, factor):
    """The features a solve records equal a recomputation from the state it started from
    (bf16 rounding): mean 4 log(1 - c + M^(1/4) c), mean log K, the summed well rates q dA / I,
    and the centred previous pressure over its RMS, each over factor x factor cells."""
    import math
    import torch
    from impec2d_gb300.workloads import device_view, realisation
    E = engine
    N = 64
    ctx = realisation(E, N, 6, ell=8.0, warm_start=1)  # lognormal K, M from the seed
    rec = E.Net(seed=0)
    ctx.run_steps(3)
    rec.attach(ctx, factor=factor, mode=2)
    cptr, pptr, _, _, qptr = ctx.state_ptrs()
    c0 = device_view(cptr, (N, N)).clone()
    p0 = device_view(pptr, (N, N)).clone()
    q = device_view(qptr, (N, N)).clone()
    ctx.step()
    h = N // factor
    X = torch.empty((h, h, 8), dtype=torch.bfloat16, device="cuda")
    E.Net.last_features(ctx, X)
    P = ctx.P
    m14 = (P.mu_res / P.mu_inj) ** 0.25
    dA = (P.x_ub - P.x_lb) / N * (P.y_ub - P.y_lb) / N
    from impec2d_gb300.workloads import grf
    K = torch.exp(0.5 * grf(N, 8.0, 5000 + 6))
    pool = lambda a: a.reshape(h, factor, h, factor).mean(dim=(1, 3))
    ref = [pool(4.0 * torch.log(1.0 - c0 + m14 * c0)), pool(torch.log(K)),
           (q * dA / P.I).reshape(h, factor, h, factor).sum(dim=(1, 3))]
    xm = pool(p0)
    ref.append((xm - xm.mean()) / xm.std(unbiased=False))
    for ch, r in enumerate(ref):
        got = X[..., ch].double()
        scale = max(r.abs().max().item(), 1e-30)
        assert (got - r).abs().max().item() <= 8e-3 * scale + 1e-6, (ch, (got - r).abs().max().item(), scale)
    assert math.isclose(X[..., 4].double().pow(2).mean().sqrt().item(), 1.0, rel_tol=2e-2)
    E.Net.detach(ctx)
    rec.close()
    ctx.close()
