"""CPU oracle of the learned initial-guess network (test infrastructure only).

A plain numpy restatement of the U-Net the CUDA kernels implement (nn.cu):
forward pass, mean-squared-error loss and the gradient with respect to every
parameter, in FP64.  With ``bf16=True`` it rounds to bfloat16 at exactly the
points where the GPU stores BF16 (inputs, weights, stored activations and
gradients), so the only remaining differences are FP32 accumulation order.

Layout: activations (D, H, W, C) C-order (channels innermost, x fastest);
parameters layer by layer, weights [27][cin][cout] (tap = dz*9 + dy*3 + dx for
offsets -1..1) followed by bias[cout].
"""
import numpy as np

CIN = 5  # input channels: cc, rhs, defect of p1, p1, p2 (scaled)
LAYERS = [(CIN, 16, True), (16, 32, True), (32, 64, True), (64, 64, True), (64, 32, True), (32, 16, True),
          (16, 1, False)]


def param_count():
    return sum(27 * ci * co + co for ci, co, _ in LAYERS)


def split_params(flat):
    out, off = [], 0
    for ci, co, _ in LAYERS:
        w = np.asarray(flat[off:off + 27 * ci * co], np.float64).reshape(27, ci, co)
        off += 27 * ci * co
        b = np.asarray(flat[off:off + co], np.float64)
        off += co
        out.append((w, b))
    return out


def join_params(parts):
    return np.concatenate([np.concatenate([w.reshape(-1), b]) for w, b in parts])


def to_bf16(a):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(a, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def _taps():
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                yield dz * 9 + dy * 3 + dx, dz, dy, dx


def conv(x, w, b=None):
    D, H, W, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((D, H, W, w.shape[2]))
    for t, dz, dy, dx in _taps():
        y += xp[dz:dz + D, dy:dy + H, dx:dx + W, :] @ w[t]
    if b is not None:
        y += b
    return y


def conv_dgrad(g, w):
    D, H, W, _ = g.shape
    dxp = np.zeros((D + 2, H + 2, W + 2, w.shape[1]))
    for t, dz, dy, dx in _taps():
        dxp[dz:dz + D, dy:dy + H, dx:dx + W, :] += g @ w[t].T
    return dxp[1:-1, 1:-1, 1:-1, :]


def conv_wgrad(x, g):
    D, H, W, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    dw = np.zeros((27, x.shape[3], g.shape[3]))
    gf = g.reshape(-1, g.shape[3])
    for t, dz, dy, dx in _taps():
        dw[t] = xp[dz:dz + D, dy:dy + H, dx:dx + W, :].reshape(-1, x.shape[3]).T @ gf
    return dw


def pool(x):
    D, H, W, C = x.shape
    return x.reshape(D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(1, 3, 5))


def up(x):
    return x.repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2)


def pool_back(g):
    return up(g) / 8.0


def up_back(g):
    D, H, W, C = g.shape
    return g.reshape(D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(1, 3, 5))


def forward(params, x, bf16=True):
    """x: (D, H, W, CIN).  Returns (y (D,H,W), cache)."""
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    P = [(r(w), np.asarray(b, np.float64)) for w, b in split_params(params)]
    c = {"x0": r(x)}
    c["e1"] = r(np.maximum(conv(c["x0"], *P[0]), 0.0))
    c["p1"] = r(pool(c["e1"]))
    c["e2"] = r(np.maximum(conv(c["p1"], *P[1]), 0.0))
    c["p2"] = r(pool(c["e2"]))
    c["e3"] = r(np.maximum(conv(c["p2"], *P[2]), 0.0))
    c["p3"] = r(pool(c["e3"]))
    c["e4"] = r(np.maximum(conv(c["p3"], *P[3]), 0.0))
    c["u3"] = r(up(c["e4"]) + c["e3"])
    c["d3"] = r(np.maximum(conv(c["u3"], *P[4]), 0.0))
    c["u2"] = r(up(c["d3"]) + c["e2"])
    c["d2"] = r(np.maximum(conv(c["u2"], *P[5]), 0.0))
    c["u1"] = r(up(c["d2"]) + c["e1"])
    y = conv(c["u1"], *P[6])[..., 0]
    c["P"] = P
    return y, c


def loss_and_grad(params, x, t, bf16=True):
    """Mean squared error of forward(x) against t and its parameter gradient."""
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    y, c = forward(params, x, bf16)
    P = c["P"]
    n = y.size
    loss = float(np.mean((y - t) ** 2))
    grads = [None] * 7

    def layer(l, dacc, act, xin, want_dx):
        g_full = dacc * (act > 0) if act is not None else dacc
        db = g_full.reshape(-1, g_full.shape[-1]).sum(axis=0)
        g = r(g_full)
        dw = conv_wgrad(xin, g)
        grads[l] = (dw, db)
        return r(conv_dgrad(g, P[l][0])) if want_dx else None

    dy = np.zeros(y.shape + (1,))
    dy[..., 0] = np.asarray(2.0 * (y - t) / n, np.float32)
    du1 = layer(6, dy, None, c["u1"], True)
    acc_e1 = du1.copy()
    du2 = layer(5, up_back(du1), c["d2"], c["u2"], True)
    acc_e2 = du2.copy()
    du3 = layer(4, up_back(du2), c["d3"], c["u3"], True)
    acc_e3 = du3.copy()
    dp3 = layer(3, up_back(du3), c["e4"], c["p3"], True)
    acc_e3 = acc_e3 + pool_back(dp3)
    dp2 = layer(2, acc_e3, c["e3"], c["p2"], True)
    acc_e2 = acc_e2 + pool_back(dp2)
    dp1 = layer(1, acc_e2, c["e2"], c["p1"], True)
    acc_e1 = acc_e1 + pool_back(dp1)
    layer(0, acc_e1, c["e1"], c["x0"], False)
    return loss, join_params(grads), y
