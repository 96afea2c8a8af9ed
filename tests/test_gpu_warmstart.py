"""What the trained surrogate gains: on held-out lid-driven cavities the warm
start (feq + f_neq from the network's prediction) reaches the FP64-accurate
residual 1e-8 in fewer steps than the start from rest, and its initial
velocity field is closer to the converged one than rest is.  The training
fields are converged to 1e-8 by the fixed-point batch solver (converged
cases leave the batch).  The perturbation curve falls monotonically: the
smaller the initial error, the fewer steps.  Small cases so the whole
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
    st, fields, _, last = ws.solve(train, max_steps=100000, tol=1e-8)
    assert np.all(st > 0), st
    X, Y, M = ws.dataset(train, fields)
    net, hist = ws.train(X, Y, M, epochs=40, batch=8, lr=2e-3)
    assert hist[-1] < 0.1 * hist[0]
    preds, _ = ws.predict(net, test)
    sp, ref, _, _ = ws.solve(test, None, max_steps=200000)
    sw, _, _, _ = ws.solve(test, preds, max_steps=200000)
    assert np.all(sp > 0) and np.all(sw > 0), (sp, sw)
    err_net = np.median([ws.field_error(c, p, r) for c, p, r in zip(test, preds, ref)])
    print("steps from rest", sp, "warm", sw, "surrogate u error", err_net)
    assert err_net < 0.5                      # rest has error 1.0
    assert np.median(sw) < np.median(sp)


def test_perturbation_curve_is_monotone(mph):
    """Steps to 1e-8 from converged fields plus smooth noise of relative size
    e: every start converges, a large error costs more steps than a small
    one, and smaller errors never cost more, up to the 1000-step resolution
    of the residual checks.  (The start from the converged field itself,
    e = 0, shows the floor that the feq + f_neq initialisation leaves; errors
    below that floor's own size all land on it.)"""
    from muphfasa_gb300 import warmstart as ws
    cases = _cases(ws, 32, 3, 4)
    st, fields, _, _ = ws.solve(cases, max_steps=100000, tol=1e-8)
    assert np.all(st > 0)
    amps = [1e-1, 1e-3, 1e-5, 0.0]
    table, _ = ws.perturbation_curve(cases, fields, amps, max_steps=100000)
    med = {e: float(np.median(table[e])) for e in amps}
    print("median steps by amplitude", med, "rest", np.median(table["rest"]))
    assert all(min(table[e]) > 0 for e in amps) and min(table["rest"]) > 0
    check = 1000
    assert med[1e-1] > med[1e-5]
    for a, b in zip(amps, amps[1:]):
        assert med[a] >= med[b] - check, (a, b, med)


def test_nonequilibrium_init_matches_the_steady_populations(mph):
    """From a converged cavity, the warm-start initialisation reproduces the
    solver's own steady populations: in the interior the stored (post-
    collision) non-equilibrium part f - feq agrees with the steady state's in
    sign and size, within the first-order Chapman-Enskog error."""
    from muphfasa_gb300 import warmstart as ws
    n, U, Re = 48, 0.08, 100.0
    c = {"kind": "cavity", "n": n, "Re": Re, "U": U, "tau": 0.5 + 3 * U * n / Re, "boxes": []}
    s = mph.Simulation(ws.case_desc(c, "f64x"))
    s.initialize()
    r = np.inf
    for _ in range(200):
        s.advance(900)
        s.residual()
        s.advance(100)
        r, _ = s.residual()
        if r < 1e-11:
            break
    assert r < 1e-11
    f_star = s.f().reshape(9, n, n)
    rho, u = s.update_macroscopic()
    t = mph.Simulation(ws.case_desc(c, "f64x"))
    t.initialize_neq(rho, u)
    f_init = t.f().reshape(9, n, n)
    cv, w, _ = mph.lattice_tables("D2Q9")
    R, Ux, Uy = rho.reshape(n, n), u[: n * n].reshape(n, n), u[n * n:].reshape(n, n)
    feq = np.stack([w[k] * R * (1 + 3 * (cv[k, 0] * Ux + cv[k, 1] * Uy) + 4.5 * (cv[k, 0] * Ux + cv[k, 1] * Uy) ** 2
                                - 1.5 * (Ux ** 2 + Uy ** 2)) for k in range(9)])
    inner = (slice(None), slice(4, -4), slice(4, -4))
    ns, ni = (f_star - feq)[inner], (f_init - feq)[inner]
    err = float(np.linalg.norm(ni - ns) / np.linalg.norm(ns))
    print("relative L2 of the initialised non-equilibrium part against the steady state:", err)
    assert err < 0.25


def test_consistent_start_lowers_the_floor(mph):
    """The consistent start (a few short runs, each followed by a reset of
    (rho, u) to the prescribed field that keeps the solver's own
    non-equilibrium part) leaves the prescribed moments in the stored
    populations to storage resolution (the moments of the streamed
    populations, which mph_batch_moments reports, equal them only at a steady
    state), and from the converged field itself it reaches 1e-8 in fewer
    steps than the feq + f_neq start, its own steps included."""
    from muphfasa_gb300 import warmstart as ws
    cases = _cases(ws, 32, 5, 4)
    st, fields, _, _ = ws.solve(cases, max_steps=100000, tol=1e-8)
    assert np.all(st > 0)
    b = ws._batch(cases, "f64x")
    for j, (rho, u) in enumerate(fields):
        b.initialize_neq(j, rho, u)
    spent = ws.consistent_start(b, cases, list(range(len(cases))), fields, steps=10, rounds=2)
    assert spent == 20
    for j, (rho, u) in enumerate(fields):
        r2, u2 = ws._moments_d2q9(b.f(j), cases[j]["n"])
        assert np.max(np.abs(r2 - rho)) < 1e-12 and np.max(np.abs(u2 - u)) < 1e-12
    b.close()
    plain, _, _, _ = ws.solve(cases, fields, max_steps=100000)
    cons, _, _, _ = ws.solve(cases, fields, max_steps=100000, consistent=(50, 4))
    print("steps from the converged field: feq + f_neq", plain, "consistent", cons)
    assert np.all(plain > 0) and np.all(cons > 0)
    assert np.median(cons) < np.median(plain)
