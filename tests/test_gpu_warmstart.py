"""What the trained surrogate gains: on held-out lid-driven cavities the warm
start (feq + f_neq from the network's prediction) reaches the FP64 residual
1e-8 in fewer steps than the start from rest, and its initial velocity field
is closer to the converged one than rest is.  Small cases so the whole
generate / train / judge cycle runs in about a minute."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases(ws, n, seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        re, u = float(rng.uniform(100, 300)), float(rng.uniform(0.05, 0.1))
        out.append({"kind": "cavity", "n": n, "Re": re, "U": u, "tau": 0.5 + 3 * u * n / re, "boxes": []})
    return out


def test_warm_start_beats_rest(mph):
    from muphfasa_gb300 import warmstart as ws
    n = 32
    train, test = _cases(ws, n, 1, 96), _cases(ws, n, 2, 8)
    _, fields, _, last = ws.solve(train, max_steps=40000, tol=0.0, precision="f32", check_every=5000)
    assert np.all(np.isfinite(last))
    X, Y, M = ws.dataset(train, fields)
    net, hist = ws.train(X, Y, M, epochs=40, batch=8, lr=2e-3)
    assert hist[-1] < 0.1 * hist[0]
    preds, _ = ws.predict(net, test)
    sp, ref, _, _ = ws.solve(test, None, max_steps=200000, precision="f64")
    sw, _, _, _ = ws.solve(test, preds, max_steps=200000, precision="f64")
    assert np.all(sp > 0) and np.all(sw > 0), (sp, sw)
    err_net = np.median([ws.field_error(c, p, r) for c, p, r in zip(test, preds, ref)])
    print("steps from rest", sp, "warm", sw, "surrogate u error", err_net)
    assert err_net < 0.5                      # rest has error 1.0
    assert np.median(sw) < np.median(sp)
