"""CPU FP64 model of the learned-skin network (TEST INFRASTRUCTURE ONLY).

The checker of the GPU's FP16 forward / backward kernels (rockable_gb300/csrc/
rk_skin.cu): same layer sizes (16 -> 64 -> 64 -> 2, ReLU), same parameter
layout W1[64][16] b1[64] W2[64][64] b2[64] W3[2][64] b3[2], same mean-squared
loss.  `half=True` rounds the inputs, weights and hidden activations to FP16
like the device does before accumulating in higher precision.
"""
import numpy as np

NIN, NH, NOUT = 16, 64, 2
SIZES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NOUT, NH)), ("b3", (NOUT,))]
NP = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, k = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[k:k + n], dtype=np.float64).reshape(shape)
        k += n
    return out


def pack(d):
    return np.concatenate([d[name].ravel() for name, _ in SIZES])


def _h(x, half):
    return x.astype(np.float16).astype(np.float64) if half else x


def forward(p, X, half=True):
    w = {k: _h(v, half) for k, v in unpack(p).items()}
    X = _h(np.asarray(X, dtype=np.float64), half)
    a1 = X @ w["W1"].T + w["b1"]
    h1 = _h(np.maximum(a1, 0.0), half)
    a2 = h1 @ w["W2"].T + w["b2"]
    h2 = _h(np.maximum(a2, 0.0), half)
    y = h2 @ w["W3"].T + w["b3"]
    return y, (X, a1, h1, a2, h2, w)


def loss_and_grad(p, X, T, half=True):
    y, (Xh, a1, h1, a2, h2, w) = forward(p, X, half)
    T = np.asarray(T, dtype=np.float64)
    r = y - T
    loss = float(np.mean(r * r))
    dy = 2.0 * r / r.size
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    d2 = (dy @ w["W3"]) * (h2 > 0)
    g["W2"] = d2.T @ h1
    g["b2"] = d2.sum(0)
    d1 = (d2 @ w["W2"]) * (h1 > 0)
    g["W1"] = d1.T @ Xh
    g["b1"] = d1.sum(0)
    return loss, pack(g)
