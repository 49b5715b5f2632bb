"""numpy reference of the learned-stop perceptron (float64): the CPU checker
of the engine's FP32 training and inference kernels."""
from __future__ import annotations

import numpy as np
from scipy.special import erf

F, H = 10, 64
O_MU, O_SD = 0, F
O_W1 = 2 * F
O_B1 = O_W1 + H * F
O_W2 = O_B1 + H
O_B2 = O_W2 + H * H
O_W3 = O_B2 + H
O_B3 = O_W3 + H
O_YMU = O_B3 + 1
O_YSD = O_YMU + 1
NP = O_YSD + 1


def gelu(z):
    return 0.5 * z * (1 + erf(z / np.sqrt(2)))


def gelu_grad(z):
    return 0.5 * (1 + erf(z / np.sqrt(2))) + z * np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)


def unpack(P):
    P = np.asarray(P, np.float64)
    return dict(mu=P[O_MU:O_MU + F], sd=P[O_SD:O_SD + F], W1=P[O_W1:O_B1].reshape(H, F), b1=P[O_B1:O_W2],
                W2=P[O_W2:O_B2].reshape(H, H), b2=P[O_B2:O_W3], W3=P[O_W3:O_B3], b3=P[O_B3], ymu=P[O_YMU],
                ysd=P[O_YSD])


def forward(P, x):
    p = unpack(P)
    xs = (np.asarray(x, np.float64) - p["mu"]) / p["sd"]
    z1 = xs @ p["W1"].T + p["b1"]
    h1 = gelu(z1)
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = gelu(z2)
    out = h2 @ p["W3"] + p["b3"]
    return out, dict(xs=xs, z1=z1, h1=h1, z2=z2, h2=h2)


def predict(P, x):
    p = unpack(P)
    return forward(P, x)[0] * p["ysd"] + p["ymu"]


def loss_grad(P, x, y):
    """Mean squared error of the standardised target and its gradient with
    respect to W1..b3 (zero at the other offsets)."""
    p = unpack(P)
    out, c = forward(P, x)
    ys = (np.asarray(y, np.float64) - p["ymu"]) / p["ysd"]
    B = len(ys)
    d = out - ys
    loss = float(np.mean(d * d))
    dout = 2 * d / B
    g = np.zeros(NP)
    g[O_W3:O_B3] = c["h2"].T @ dout
    g[O_B3] = dout.sum()
    dz2 = np.outer(dout, p["W3"]) * gelu_grad(c["z2"])
    g[O_W2:O_B2] = (dz2.T @ c["h1"]).ravel()
    g[O_B2:O_W3] = dz2.sum(0)
    dz1 = (dz2 @ p["W2"]) * gelu_grad(c["z1"])
    g[O_W1:O_B1] = (dz1.T @ c["xs"]).ravel()
    g[O_B1:O_W2] = dz1.sum(0)
    return loss, g
