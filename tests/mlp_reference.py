"""NumPy reference of the learned-truncation network (5-64-64-64-1, SiLU):
forward, mean-squared-error loss and analytic gradient, in float64.  Parameter
layout as in the library: W1[64][5] b1 W2[64][64] b2 W3[64][64] b3 W4[64] b4."""
import numpy as np

H, NIN = 64, 5
SIZES = [("W1", (H, NIN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)), ("W4", (H,)), ("b4", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, o = {}, 0
    for k, s in SIZES:
        n = int(np.prod(s))
        out[k] = np.asarray(p[o:o + n], dtype=np.float64).reshape(s)
        o += n
    return out


def pack(d):
    return np.concatenate([d[k].ravel() for k, _ in SIZES])


def silu(z):
    return z / (1 + np.exp(-z))


def dsilu(z):
    s = 1 / (1 + np.exp(-z))
    return s * (1 + z * (1 - s))


def loss_grad(p, X, y):
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    z1 = X @ w["W1"].T + w["b1"]; h1 = silu(z1)
    z2 = h1 @ w["W2"].T + w["b2"]; h2 = silu(z2)
    z3 = h2 @ w["W3"].T + w["b3"]; h3 = silu(z3)
    yhat = h3 @ w["W4"] + w["b4"][0]
    r = yhat - y
    n = len(y)
    loss = np.mean(r * r)
    d4 = 2 * r / n
    g = {"W4": h3.T @ d4, "b4": np.array([d4.sum()])}
    dz3 = np.outer(d4, w["W4"]) * dsilu(z3)
    g["W3"] = dz3.T @ h2; g["b3"] = dz3.sum(0)
    dz2 = (dz3 @ w["W3"]) * dsilu(z2)
    g["W2"] = dz2.T @ h1; g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ w["W2"]) * dsilu(z1)
    g["W1"] = dz1.T @ X; g["b1"] = dz1.sum(0)
    return loss, pack(g), yhat
