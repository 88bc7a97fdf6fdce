"""Learned warm start: training pairs written by the solver itself, and AdamW training of the
encoder-decoder on them (all compute in the engine's CUDA kernels; torch only holds the
device tensors and draws the batches).

A pair is one pressure solve of an IMPES run: the features the solve computes at its start
(mobility, permeability, wells, previous pressure, its residual under the new mobility) and
the target, the converged pressure minus the previous one, averaged to the feature grid,
centred and scaled to unit RMS (impec_learned_features / impec_learned_target)."""
from __future__ import annotations

import time

from . import Net
from .workloads import realisation


def generate_pairs(E, n_members: int, pairs_per_member: int, N: int = 256, every: int = 2, skip: int = 2,
                   factor: int = 1, seed0: int = 0, precision: str = "mixed", ell: float = 16.0, log=None):
    """Run n_members realisations (seeds seed0, seed0 + 1, ...) with the previous pressure as
    the initial guess, recording one pair every `every` steps after `skip` steps.  Returns
    X [P][N/f][N/f][8] bf16 and T [P][N/f][N/f] fp32 on the device, and the generation time."""
    import torch
    h = N // factor
    P = n_members * pairs_per_member
    X = torch.empty((P, h, h, 8), dtype=torch.bfloat16, device="cuda")
    T = torch.empty((P, h, h), dtype=torch.float32, device="cuda")
    rec = Net(seed=0)  # record mode never evaluates the network
    t0 = time.perf_counter()
    i = 0
    for m in range(n_members):
        ctx = realisation(E, N, seed0 + m, precision=precision, ell=ell, warm_start=1)
        rec.attach(ctx, factor=factor, mode=2)
        k = 0
        while k < skip + every * pairs_per_member:
            ctx.step()
            k += 1
            if k > skip and (k - skip) % every == 0:
                Net.last_features(ctx, X[i])
                Net.last_target(ctx, T[i])
                i += 1
        Net.detach(ctx)
        ctx.close()
        if log and (m + 1) % max(1, n_members // 10) == 0:
            log(f"members {m + 1}/{n_members}: {i} pairs, {time.perf_counter() - t0:.1f} s")
    rec.close()
    torch.cuda.synchronize()
    return X[:i], T[:i], time.perf_counter() - t0


def validation_mse(net: Net, X, T, batch: int = 64) -> float:
    """Mean squared error of the prediction (channel 0) over a set of pairs."""
    import torch
    tot, n = 0.0, 0
    for b in range(0, X.shape[0], batch):
        out = net.forward(X[b:b + batch])
        tot += float(((out - T[b:b + batch]) ** 2).sum())
        n += out.numel()
    return tot / max(n, 1)


def train(net: Net, X, T, epochs: float = 1.0, batch: int = 64, lr: float = 3e-4, weight_decay: float = 1e-4,
          seed: int = 0, Xval=None, Tval=None, log=None, evals: int = 10):
    """AdamW on random batches (without replacement within an epoch).  Returns the history:
    (step, batch loss, validation MSE or None) at `evals` points, and the training time."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    P = X.shape[0]
    per_epoch = P // batch
    total = max(1, int(round(epochs * per_epoch)))
    hist = []
    t_train = 0.0
    step = 0
    every = max(1, total // evals)
    while step < total:
        perm = torch.randperm(P, generator=g, device="cuda")
        for b in range(per_epoch):
            if step >= total:
                break
            idx = perm[b * batch:(b + 1) * batch]
            Xb, Tb = X.index_select(0, idx), T.index_select(0, idx)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            loss = net.train_batch(Xb, Tb, lr=lr, weight_decay=weight_decay)
            t_train += time.perf_counter() - t0
            step += 1
            if step % every == 0 or step == total:
                v = validation_mse(net, Xval, Tval) if Xval is not None else None
                hist.append((step, loss, v))
                if log:
                    log(f"step {step}/{total}: batch loss {loss:.4f}" + (f", validation {v:.4f}" if v is not None else ""))
    return hist, t_train
