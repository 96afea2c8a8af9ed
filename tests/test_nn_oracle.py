"""The CPU restatement of the surrogate network: its hand-written backward
pass against central finite differences in float64, and the BF16 rounding
helper."""
import numpy as np
import pytest

from oracle import nn_oracle as NO


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 0.0], np.float32)
    r = NO.to_bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # exact tie -> even (down)
    assert r[2] == 1.0                      # below half an ulp
    assert r[3] == 1.0 + 2 ** -7            # above half an ulp
    assert r[4] == -2.5 and r[5] == 0.0
    y = np.random.default_rng(0).standard_normal(1000).astype(np.float32)
    assert np.all(np.abs(NO.to_bf16(y) - y) <= np.abs(y) * 2 ** -8)


@pytest.mark.parametrize("name,idx", [("e1a", (3, 10)), ("e4b", (7, 100)), ("d2a", (5, 50)), ("head", (1, 4)),
                                      ("d1b", (0, 0))])
def test_backward_matches_finite_differences(name, idx):
    rng = np.random.default_rng(1)
    p = NO.init_params(3)
    x = rng.standard_normal((2, 16, 16, 8))
    y = rng.standard_normal((2, 16, 16, 3))
    m = (rng.random((2, 16, 16)) > 0.2).astype(np.float64)
    net = NO.Net(p, bf16=False)
    loss, dpred = net.loss(net.forward(x), y, m)
    g = net.backward(dpred)[name][0][idx]
    h = 1e-6
    Wt, b = p[name]
    for sgn, store in ((1, "lp"), (-1, "lm")):
        W2 = Wt.copy()
        W2[idx] += sgn * h
        q = dict(p)
        q[name] = (W2, b)
        n2 = NO.Net(q, bf16=False)
        val = n2.loss(n2.forward(x), y, m)[0]
        if store == "lp":
            lp = val
        else:
            lm = val
    fd = (lp - lm) / (2 * h)
    assert abs(fd - g) <= 1e-6 * max(1.0, abs(g)) + 1e-7, (fd, g)
