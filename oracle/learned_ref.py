"""CPU restatement of the learned warm-start network -- TEST INFRASTRUCTURE ONLY.

numpy (fp32 arithmetic) forward and backward pass of the 15-convolution encoder-decoder that
impec2d_gb300/csrc/learned_net.cu trains on the tensor cores, with values rounded to bf16
exactly where the GPU stores bf16 (pre-activations, activations, pooled / upsampled maps,
gradients), so the GPU's gradients can be checked against it.  Only tests load this module.

Layouts follow the GPU: activations [H][W][C] (one sample), weights [cout][Kp] with
k = tap * cin + c, tap = 3 (dy + 1) + (dx + 1).

forward_backward(..., exact=True) drops the bf16 rounding and works in float64: that variant is
checked against central finite differences of the loss, which pins the restatement's calculus;
the rounded variant is what the GPU's gradients are compared with.
"""
import numpy as np
from scipy.special import erf

# cin, cout, level, act, skip_from  (the table of learned_net.cu)
LAYERS = [(8, 32, 0, 1, -1), (32, 32, 0, 1, -1), (32, 64, 1, 1, -1), (64, 64, 1, 1, -1), (64, 128, 2, 1, -1),
          (128, 128, 2, 1, -1), (128, 256, 3, 1, -1), (256, 256, 3, 1, -1), (256, 128, 2, 1, 5), (128, 128, 2, 1, -1),
          (128, 64, 1, 1, 3), (64, 64, 1, 1, -1), (64, 32, 0, 1, 1), (32, 32, 0, 1, -1), (32, 8, 0, 0, -1)]


def kp(cin):
    return (9 * cin + 63) // 64 * 64


def bf16(x):
    """Round fp32 to bf16 (nearest, ties to even), returned as fp32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def gelu(x):
    return (0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))).astype(x.dtype)


def gelu_d(x):
    return (0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)).astype(x.dtype)


def patches(x, sign=1):
    """[H][W][9*C] neighbourhoods (zero outside), tap-major like the GPU's K index."""
    H, W, C = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (0, 0)))
    out = np.empty((H, W, 9 * C), x.dtype)
    for tap in range(9):
        dy, dx = sign * (tap // 3 - 1), sign * (tap % 3 - 1)
        out[:, :, tap * C:(tap + 1) * C] = xp[1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :]
    return out


def conv(x, w, cin):
    return np.einsum("hwk,ok->hwo", patches(x), w[:, :9 * cin], optimize=True).astype(x.dtype)


def conv_t(dz, w, cin, cout):
    """Input gradient: sum over taps and cout of dz(p - d) w[co][tap, ci]."""
    wt = w[:, :9 * cin].reshape(cout, 9, cin)            # [co][tap][ci]
    wd = np.transpose(wt, (2, 1, 0)).reshape(cin, 9 * cout)  # [ci][tap * cout + co]
    return np.einsum("hwk,ik->hwi", patches(dz, -1), wd, optimize=True).astype(dz.dtype)


def pool(x, q=bf16):
    return q(0.25 * (x[0::2, 0::2] + x[0::2, 1::2] + x[1::2, 0::2] + x[1::2, 1::2]))


def up(x):
    return np.repeat(np.repeat(x, 2, axis=0), 2, axis=1)


def unflatten(params, dtype=np.float32):
    """Host parameter vector (impec_net_parameters order) -> [(w [cout][Kp], b [cout])]."""
    out, off = [], 0
    for cin, cout, *_ in LAYERS:
        nw = cout * kp(cin)
        out.append((params[off:off + nw].reshape(cout, kp(cin)).astype(dtype),
                    params[off + nw:off + nw + cout].astype(dtype)))
        off += nw + cout
    return out


def forward_backward(params, X, T, exact=False):
    """Loss and parameter gradients (flattened like impec_net_parameters) for one sample.
    X: [H][W][8] (bf16 values), T: [H][W] fp32.  exact: float64 without bf16 rounding."""
    dtype = np.float64 if exact else np.float32
    bf16 = (lambda a: np.asarray(a, np.float64)) if exact else globals()["bf16"]
    X = np.asarray(X, dtype)
    T = np.asarray(T, dtype)
    P = unflatten(params, dtype)
    W = [bf16(w) for w, _ in P]
    b = [bb for _, bb in P]
    n = len(LAYERS)
    z, zs, y, inp = [None] * n, [None] * n, [None] * n, [None] * n
    d = {}
    for l, (cin, cout, level, act, skip) in enumerate(LAYERS):
        if l == 0:
            x = X
        elif l in (2, 4, 6):
            x = d[l]
        elif l in (8, 10, 12):
            x = d[l]
        else:
            x = y[l - 1]
        inp[l] = x
        zf = conv(x, W[l], cin) + b[l]
        zs[l] = bf16(zf)
        if l == n - 1:
            y[l] = zf
        else:
            yy = gelu(zf) if act else zf
            if skip >= 0:
                yy = yy + y[skip]
            y[l] = bf16(yy)
        if l == 1:
            d[2] = pool(y[1], bf16)
        if l == 3:
            d[4] = pool(y[3], bf16)
        if l == 5:
            d[6] = pool(y[5], bf16)
        if l == 7:
            d[8] = up(y[7])
        if l == 9:
            d[10] = up(y[9])
        if l == 11:
            d[12] = up(y[11])
    out = y[n - 1][:, :, 0]
    Pix = out.size
    e = out - T
    loss = float(np.sum(e.astype(np.float64) ** 2) / Pix)
    dz = [None] * n
    g = np.zeros_like(y[n - 1])
    g[:, :, 0] = 2.0 * e / Pix
    dz[n - 1] = bf16(g)
    gw, gb = [None] * n, [None] * n
    ds = {}
    for l in range(n - 1, -1, -1):
        cin, cout, level, act, skip = LAYERS[l]
        gw_l = np.zeros((cout, kp(cin)), dtype)
        gw_l[:, :9 * cin] = np.einsum("hwo,hwk->ok", dz[l], patches(inp[l]), optimize=True)
        gw[l] = gw_l
        gb[l] = dz[l].sum(axis=(0, 1), dtype=dtype)
        if l == 0:
            continue
        raw = conv_t(dz[l], W[l], cin, cout)
        if l in (14, 7, 5, 3, 1):
            dz[l - 1] = bf16(raw * gelu_d(zs[l - 1]))
        elif l in (13, 11, 9):
            ds[l] = bf16(raw)
            dz[l - 1] = bf16(raw * gelu_d(zs[l - 1]))
        elif l in (12, 10, 8):
            r = bf16(raw)
            s = r[0::2, 0::2] + r[0::2, 1::2] + r[1::2, 0::2] + r[1::2, 1::2]
            dz[l - 1] = bf16(s * gelu_d(zs[l - 1]))
        else:  # 6, 4, 2: pooled input; the encoder output also feeds a skip
            r = bf16(raw)
            skipg = {6: ds[9], 4: ds[11], 2: ds[13]}[l]
            dz[l - 1] = bf16((0.25 * up(r) + skipg) * gelu_d(zs[l - 1]))
    flat = []
    for l in range(n):
        flat.append(gw[l].ravel())
        flat.append(gb[l].ravel())
    return loss, np.concatenate(flat)
