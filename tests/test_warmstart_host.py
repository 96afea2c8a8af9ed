"""Host-side pieces of the learned warm start (no device): the seeded case
draw (Re, U, tau, 0-3 solid boxes covering 5-20 % with a fluid margin), the
network inputs, and the target / prediction scaling round trip."""
import math

import numpy as np
import pytest

from muphfasa_gb300 import warmstart as ws


def test_draw_is_seeded_and_in_range():
    a = ws.draw_cases(60, seed=7)
    b = ws.draw_cases(60, seed=7)
    assert a == b
    assert ws.draw_cases(60, seed=8) != a
    for c in a:
        assert c["kind"] in ("cavity", "channel") and c["n"] == 128
        assert ws.RE[0] <= c["Re"] <= ws.RE[1] and ws.U[0] <= c["U"] <= ws.U[1]
        assert c["tau"] == pytest.approx(0.5 + 3.0 * c["U"] * c["n"] / c["Re"])
        assert c["tau"] > 0.5
        assert 0 <= len(c["boxes"]) <= 3
    assert {len(c["boxes"]) for c in a} == {0, 1, 2, 3}
    assert {c["kind"] for c in a} == {"cavity", "channel"}


def test_boxes_cover_a_bounded_fraction_with_a_fluid_margin():
    for c in ws.draw_cases(200, seed=11, sizes=(64, 128)):
        n = c["n"]
        m = ws.case_mask(c)
        assert m.shape == (n, n)
        if not c["boxes"]:
            assert m.sum() == 0
            continue
        cover = m.mean()
        assert 0.01 < cover < 0.26, cover  # 5-20 % drawn; boxes may overlap, sides round
        for x0, y0, w, h in c["boxes"]:
            assert w >= 2 and h >= 2
            assert x0 >= 3 and y0 >= 3 and x0 + w <= n - 3 and y0 + h <= n - 3
        assert m[:3].sum() == 0 and m[-3:].sum() == 0 and m[:, :3].sum() == 0 and m[:, -3:].sum() == 0


def test_case_description():
    cav, chan = None, None
    for c in ws.draw_cases(20, seed=3):
        if c["kind"] == "cavity" and cav is None:
            cav = c
        if c["kind"] == "channel" and chan is None:
            chan = c
    d = ws.case_desc(cav)
    assert (d.dim, d.q, d.n[0], d.n[1]) == (2, 9, cav["n"], cav["n"])
    assert d.omega == pytest.approx(1.0 / cav["tau"])
    d = ws.case_desc(chan, precision="f64")
    assert d.omega == pytest.approx(1.0 / chan["tau"])


def test_features():
    c = {"kind": "channel", "n": 16, "Re": 400.0, "U": 0.05, "tau": 0.5 + 3 * 0.05 * 16 / 400.0,
         "boxes": [(5, 6, 3, 2)]}
    f = ws.features(c)
    assert f.shape == (16, 16, 8) and f.dtype == np.float32
    assert f[..., 0].sum() == 6 and f[6, 5, 0] == 1 and f[7, 7, 0] == 1
    assert np.all(f[:, 0, 1] == 1) and f[..., 1].sum() == 16  # inflow column
    assert np.all(f[0, :, 2] == 1) and np.all(f[-1, :, 2] == 1)  # no-slip rows
    assert np.all(f[:, -1, 3] == 1) and f[..., 3].sum() == 16  # outlet column
    want = (math.log(400.0) - math.log(ws.RE[0])) / (math.log(ws.RE[1]) - math.log(ws.RE[0]))
    assert np.allclose(f[..., 4], want) and np.allclose(f[..., 5], 0.5)
    assert f[0, 0, 6] == pytest.approx(0.5 / 16) and f[0, -1, 6] == pytest.approx(15.5 / 16)
    assert f[0, 0, 7] == pytest.approx(0.5 / 16) and f[-1, 0, 7] == pytest.approx(15.5 / 16)
    c["kind"] = "cavity"
    f = ws.features(c)
    assert np.all(f[-1, :, 1] == 1) and f[..., 1].sum() == 16  # lid row
    assert f[..., 3].sum() == 0


def test_targets_and_prediction_round_trip():
    rng = np.random.default_rng(4)
    c = ws.draw_cases(1, seed=5)[0]
    n = c["n"]
    rho = 1.0 + 1e-3 * rng.standard_normal(n * n)
    u = 0.05 * rng.standard_normal(2 * n * n)
    t = ws.targets(c, rho, u)
    assert t.shape == (n, n, 3)
    r2, u2 = ws.fields_from_prediction(c, t)
    solid = ws.case_mask(c).reshape(-1).astype(bool)
    fluid = ~solid
    assert np.allclose(r2[fluid], rho[fluid], rtol=0, atol=1e-7 * ws.rho_scale(c) * 10 + 1e-12)
    assert np.allclose(u2[: n * n][fluid], u[: n * n][fluid], rtol=1e-6, atol=1e-9)
    assert np.allclose(u2[n * n:][fluid], u[n * n:][fluid], rtol=1e-6, atol=1e-9)
    assert np.all(r2[solid] == 1.0) and np.all(u2[: n * n][solid] == 0) and np.all(u2[n * n:][solid] == 0)


def test_consistent_start_moment_helpers():
    """The host arithmetic of the consistent start: the D2Q9 equilibrium of
    (rho, u) has exactly those moments (to rounding), and replacing the
    equilibrium part of a population set keeps its non-equilibrium part while
    its moments become the prescribed ones (what consistent_start uploads)."""
    n = 16
    rng = np.random.default_rng(3)
    rho = 1 + 0.01 * rng.standard_normal(n * n)
    u = 0.05 * rng.standard_normal(2 * n * n)
    feq = ws._feq_d2q9(rho, u, n)
    r2, u2 = ws._moments_d2q9(feq, n)
    assert np.max(np.abs(r2 - rho)) < 1e-14 and np.max(np.abs(u2 - u)) < 1e-14
    # a population set with a non-equilibrium part that carries no mass or momentum
    c, w, _ = __import__("muphfasa_gb300").lattice_tables("D2Q9")
    neq = 1e-3 * w[:, None] * (3 * c[:, 0:1] * c[:, 1:2]) * rng.standard_normal(n * n)[None, :]
    f = feq + neq
    rho_t, u_t = 1 + 0.02 * rng.standard_normal(n * n), 0.03 * rng.standard_normal(2 * n * n)
    rf, uf = ws._moments_d2q9(f, n)
    g = ws._feq_d2q9(rho_t, u_t, n) + (f - ws._feq_d2q9(rf, uf, n))
    r3, u3 = ws._moments_d2q9(g, n)
    assert np.max(np.abs(r3 - rho_t)) < 1e-13 and np.max(np.abs(u3 - u_t)) < 1e-13
    assert np.allclose(g - ws._feq_d2q9(rho_t, u_t, n), neq, atol=1e-15)
