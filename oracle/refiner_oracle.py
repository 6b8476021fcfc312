"""FP64 numpy restatement of the subpixel refiner (test infrastructure only).

The checker for the CUDA refiner kernels: forward pass, loss, gradients of
every parameter, and one Adam step, in float64.  The network (valid 3x3
convolutions, GELU):

    x0 [1][9][9]  -> conv 32 -> [32][7][7] -> GELU
                  -> conv 32 -> [32][5][5] -> GELU
                  -> conv 32 -> [32][3][3] -> GELU -> flatten (c, i, j) = 288
                  -> dense 64 -> GELU -> dense 3 = (fx, fy, s)

fx, fy: subpixel position of the correlation peak relative to the integer
peak (surface pixels); s: log variance of that estimate.  Loss per sample:
0.5 r^2 + 0.5 stopgrad(r^2) exp(-s) + s, r^2 = (fx-tx)^2 + (fy-ty)^2, mean over
the batch.  The flat parameter vector is laid out as PARAM_LAYOUT.
"""
from __future__ import annotations

import math

import numpy as np

PARAM_LAYOUT = [("W1", (32, 1, 3, 3)), ("b1", (32,)), ("W2", (32, 32, 3, 3)), ("b2", (32,)),
                ("W3", (32, 32, 3, 3)), ("b3", (32,)), ("F1", (64, 288)), ("c1", (64,)),
                ("F2", (3, 64)), ("c2", (3,))]
NPARAM = sum(int(np.prod(s)) for _, s in PARAM_LAYOUT)


def unpack(theta):
    out, o = {}, 0
    for name, shape in PARAM_LAYOUT:
        n = int(np.prod(shape))
        out[name] = np.asarray(theta[o:o + n], np.float64).reshape(shape)
        o += n
    return out


def pack(p):
    return np.concatenate([np.asarray(p[name], np.float64).ravel() for name, _ in PARAM_LAYOUT])


def init(seed=0):
    """He-normal weights, zero biases, log-variance bias -4."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, shape in PARAM_LAYOUT:
        if name.startswith(("W", "F")):
            fan_in = int(np.prod(shape[1:]))
            p[name] = rng.standard_normal(shape) * math.sqrt(2.0 / fan_in)
        else:
            p[name] = np.zeros(shape)
    p["F2"] *= 0.1
    p["c2"][2] = -4.0
    return pack(p)


_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def conv_valid(a, W, b):
    """a [N][Ci][H][H], W [Co][Ci][3][3] -> [N][Co][H-2][H-2]."""
    N, Ci, H, _ = a.shape
    Ho = H - 2
    out = np.zeros((N, W.shape[0], Ho, Ho))
    for di in range(3):
        for dj in range(3):
            out += np.einsum("nkij,ck->ncij", a[:, :, di:di + Ho, dj:dj + Ho], W[:, :, di, dj])
    return out + b[None, :, None, None]


def forward(theta, x):
    """x [N][81] -> outputs [N][3] and the cache for backward."""
    p = unpack(theta)
    x0 = np.asarray(x, np.float64).reshape(-1, 1, 9, 9)
    y1 = conv_valid(x0, p["W1"], p["b1"]); a1 = gelu(y1)
    y2 = conv_valid(a1, p["W2"], p["b2"]); a2 = gelu(y2)
    y3 = conv_valid(a2, p["W3"], p["b3"]); a3 = gelu(y3)
    h = a3.reshape(len(x0), 288)
    z1 = h @ p["F1"].T + p["c1"]; g1 = gelu(z1)
    out = g1 @ p["F2"].T + p["c2"]
    return out, dict(x0=x0, y1=y1, a1=a1, y2=y2, a2=a2, y3=y3, a3=a3, h=h, z1=z1, g1=g1, out=out, p=p)


def loss_and_dout(out, t):
    t = np.asarray(t, np.float64).reshape(-1, 2)
    n = len(out)
    r2 = (out[:, 0] - t[:, 0]) ** 2 + (out[:, 1] - t[:, 1]) ** 2
    s = out[:, 2]
    loss = np.mean(0.5 * r2 + 0.5 * r2 * np.exp(-s) + s)
    d = np.zeros_like(out)
    d[:, 0] = (out[:, 0] - t[:, 0]) / n
    d[:, 1] = (out[:, 1] - t[:, 1]) / n
    d[:, 2] = (1.0 - 0.5 * r2 * np.exp(-s)) / n
    return loss, d


def conv_back(dy, a_in, W):
    """dy [N][Co][Ho][Ho], a_in [N][Ci][H][H] -> (d a_in, dW, db)."""
    N, Co, Ho, _ = dy.shape
    dW = np.zeros_like(W)
    da = np.zeros_like(a_in)
    for di in range(3):
        for dj in range(3):
            dW[:, :, di, dj] = np.einsum("ncij,nkij->ck", dy, a_in[:, :, di:di + Ho, dj:dj + Ho])
            da[:, :, di:di + Ho, dj:dj + Ho] += np.einsum("ncij,ck->nkij", dy, W[:, :, di, dj])
    return da, dW, dy.sum(axis=(0, 2, 3))


def backward(cache, dout):
    p = cache["p"]
    g = {}
    g["F2"] = dout.T @ cache["g1"]
    g["c2"] = dout.sum(0)
    dg1 = dout @ p["F2"]
    dz1 = dg1 * gelu_grad(cache["z1"])
    g["F1"] = dz1.T @ cache["h"]
    g["c1"] = dz1.sum(0)
    dh = dz1 @ p["F1"]
    dy3 = dh.reshape(cache["y3"].shape) * gelu_grad(cache["y3"])
    da2, g["W3"], g["b3"] = conv_back(dy3, cache["a2"], p["W3"])
    dy2 = da2 * gelu_grad(cache["y2"])
    da1, g["W2"], g["b2"] = conv_back(dy2, cache["a1"], p["W2"])
    dy1 = da1 * gelu_grad(cache["y1"])
    _, g["W1"], g["b1"] = conv_back(dy1, cache["x0"], p["W1"])
    return pack(g)


def loss_grad(theta, x, t):
    out, cache = forward(theta, x)
    loss, dout = loss_and_dout(out, t)
    return loss, backward(cache, dout), out


def adam(theta, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
