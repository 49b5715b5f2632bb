"""The numpy reference of the learned-stop perceptron checked against finite
differences (CPU), and the weight layout against the C ABI constants."""
from __future__ import annotations

import numpy as np

import mlp_reference as ref


def _data(seed=0, n=40):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, ref.F))
    y = rng.normal(size=n) * 0.3 - 0.2
    P = rng.normal(size=ref.NP) * 0.2
    P[ref.O_MU:ref.O_MU + ref.F] = x.mean(0)
    P[ref.O_SD:ref.O_SD + ref.F] = x.std(0)
    P[ref.O_YMU], P[ref.O_YSD] = y.mean(), y.std()
    return P, x, y


def test_reference_gradient_matches_finite_differences():
    P, x, y = _data()
    loss, g = ref.loss_grad(P, x, y)
    rng = np.random.default_rng(1)
    idx = np.concatenate([rng.choice(np.arange(ref.O_W1, ref.O_B3 + 1), 40, replace=False), [ref.O_B3]])
    for i in idx:
        h = 1e-6
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (ref.loss_grad(Pp, x, y)[0] - ref.loss_grad(Pm, x, y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_layout_matches_abi(engine_lib):
    from periodsearch_gb300 import _abi, learned

    assert ref.NP == _abi.MLP_FLOATS == learned.NP
    assert (ref.O_W1, ref.O_W2, ref.O_W3, ref.O_YSD) == (learned.O_W1, learned.O_W2, learned.O_W3, learned.O_YSD)
    text = (__import__("conftest").ROOT / "include" / "ps_gb300.h").read_text()
    assert f"#define PS_MLP_FLOATS {ref.NP}" in text
