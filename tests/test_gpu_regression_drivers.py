"""The reference's regression drivers and CI acceptance checks restated as
GPU tests on the library, driven through the inputs-file parser:

* lid2d (tests/regression/lid2d/main.cpp:45-54, 292-340): mass drift, KE
  spin-up and plateau, steady-state power balance and the three Marchi et
  al. (2009) centre-line extrema at 1 %;
* TGV-2D grid convergence (tests/regression/tgv2d/convergence.py, CI
  --n-list 32 64 128 --min-order 1.8): observed order of the inf-norm
  velocity error at the decay time nu k^2 t = 0.1;
* plane Couette, 2-D and 3-D over D3Q15 / D3Q19 / D3Q27
  (.github/workflows/couette-regression.yml: convergence*.py --min-order 1.8
  over 16 32 64, plot_couette*.py --max-profile-err 0.01
  --max-rate-rel-err 0.01): observed order at nu t / H^2 = 0.05, the
  start-up profile against the series solution over every 50-step snapshot,
  and the first-mode decay rate against pi^2 nu / H^2.

Errors are taken relative to the lattice reference velocity, which equals
the reference's physical-unit errors divided by its reference velocity."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# ---- lid-driven cavity -----------------------------------------------------
LID2D = """
grid.ncells = 64 64
sim.max_step = 20000
lbm.lattice_type = D2Q9
lbm.tau = 0.692
units.ref_length = 1.0
units.ref_velocity = 0.05
units.ref_density = 1.0
units.Re = 100.0
bc.lo_type = NoSlip NoSlip
bc.hi_type = NoSlip MovingWall
bc.hiy_Uwall = 0.05 0.0
geometry.prob_lo = 0.0 0.0
geometry.prob_hi = 1.0 1.0
amr.plot_int = 1000
"""

# Marchi, Suero & Araki (2009): grid-converged Re = 100 centre-line extrema
# (u / U_lid along x = 0.5; v / U_lid along y = 0.5), as the reference quotes them.
MARCHI = {"umin": -2.140417e-1, "vmax": 1.79572814e-1, "vmin": -2.53804e-1}


def _power_and_dissipation(ux, uy, u_lid, nu):
    """Lid power and viscous dissipation (lid2d/main.cpp:67-118): central
    differences with wall-reflected ghosts (2 u_wall - u), the lid shear from
    a quadratic through the wall and the two cells below it."""
    N = ux.shape[0]

    def ghosted(u, top):
        g = np.empty((N + 2, N + 2))
        g[1:-1, 1:-1] = u
        g[0, 1:-1] = -u[0]          # y = lo wall
        g[-1, 1:-1] = 2 * top - u[-1]  # y = hi (lid for u_x)
        g[1:-1, 0] = -u[:, 0]
        g[1:-1, -1] = -u[:, -1]
        return g

    gu, gv = ghosted(ux, u_lid), ghosted(uy, 0.0)
    dudx = 0.5 * (gu[1:-1, 2:] - gu[1:-1, :-2])
    dudy = 0.5 * (gu[2:, 1:-1] - gu[:-2, 1:-1])
    dvdx = 0.5 * (gv[1:-1, 2:] - gv[1:-1, :-2])
    dvdy = 0.5 * (gv[2:, 1:-1] - gv[:-2, 1:-1])
    eps = nu * float(np.sum(dudx ** 2 + dudy ** 2 + dvdx ** 2 + dvdy ** 2))
    d1 = ux[-1] - u_lid
    d2 = ux[-2] - u_lid
    b = (d2 - 3.0 * d1) / 1.5
    a = 2.0 * d1 - 0.5 * b
    power = u_lid * nu * float(np.sum(-a))
    return power, eps


def _extremum(f, sign):
    """Extremum of f sampled at (m + 1/2) / n with parabolic refinement
    (lid2d/main.cpp:122-140)."""
    n = len(f)
    m = int(np.argmax(sign * f))
    val, pos = f[m], (m + 0.5) / n
    if 0 < m < n - 1:
        den = f[m - 1] - 2.0 * f[m] + f[m + 1]
        if den != 0.0:
            delta = 0.5 * (f[m - 1] - f[m + 1]) / den
            val = f[m] - 0.25 * (f[m - 1] - f[m + 1]) * delta
            pos = (m + 0.5 + delta) / n
    return val, pos


def _centerline(ux, uy, u_lid):
    N = ux.shape[0]
    c0, c1 = N // 2 - 1, N // 2
    u_of_y = 0.5 * (ux[:, c0] + ux[:, c1]) / u_lid
    v_of_x = 0.5 * (uy[c0, :] + uy[c1, :]) / u_lid
    return {"umin": _extremum(u_of_y, -1)[0], "vmax": _extremum(v_of_x, +1)[0], "vmin": _extremum(v_of_x, -1)[0]}


@pytest.mark.parametrize("precision", ["f64", "f64x"])
def test_lid2d_regression_checks(precision, mph):
    d, info = mph.InputParser(text=LID2D).derive(precision)
    s = mph.Simulation(d, info)
    s.initialize()
    N = 64
    u_lid = d.face_U[3][0]
    nu = (1.0 / d.omega - 0.5) / 3.0
    assert abs(u_lid - 0.1) < 1e-12 and abs(nu - 0.064) < 1e-12
    hist = [{"mass": float(N * N), "ke": 0.0}]  # t = 0: the rest state itself
    done = 0
    for step in list(range(0, 20000, 1000)) + [20000]:
        s.advance(step + 1 - done)  # the driver's loop: advance, then sample after steps 0, 1000, ...
        done = step + 1
        rho, u = s.update_macroscopic()
        ux, uy = u[: N * N].reshape(N, N), u[N * N:].reshape(N, N)
        power, eps = _power_and_dissipation(ux, uy, u_lid, nu)
        hist.append({"mass": float(rho.sum()), "ke": 0.5 * float(np.sum(ux ** 2 + uy ** 2)),
                     "power": power, "eps": eps})
    m0 = hist[0]["mass"]
    drift = max(abs(h["mass"] - m0) / m0 for h in hist)
    dips = max((hist[i - 1]["ke"] - hist[i]["ke"]) / hist[i - 1]["ke"] for i in range(2, len(hist)))
    last = hist[-1]
    plateau = abs(last["ke"] - hist[-2]["ke"]) / last["ke"]
    balance = abs(last["power"] - last["eps"]) / abs(last["power"])
    ext = _centerline(ux, uy, u_lid)
    errs = {k: abs(ext[k] - MARCHI[k]) / abs(MARCHI[k]) for k in MARCHI}
    print(f"lid2d {precision}: drift {drift:.2e} dip {dips:.2e} plateau {plateau:.2e} balance {balance:.3f} "
          f"extrema {ext} rel err {errs}")
    assert drift < 1e-9                                   # kTolMass
    assert hist[0]["ke"] == 0.0 and last["ke"] > 0.0 and dips < 1e-3  # kTolMono
    assert plateau < 1e-4                                 # kTolPlateau
    assert balance < 0.20                                 # kTolBalance
    assert all(e < 0.01 for e in errs.values()), errs     # kTolBench


# ---- Taylor-Green vortex grid convergence ------------------------------------
TGV2D = """
grid.ncells = 64 64
sim.max_step = 2000
lbm.lattice_type = D2Q9
lbm.tau = 0.8
units.ref_length = 1.0
units.ref_velocity = 0.005
units.Re = 10
bc.lo_type = Periodic Periodic
bc.hi_type = Periodic Periodic
geometry.prob_lo = 0.0 0.0
geometry.prob_hi = 6.283185307179586 6.283185307179586
"""


def _tgv(N, u0, nu, t):
    """Analytic 2-D TGV of the reference's regression test (TgvAnalytic.H):
    u = -u0 cos kx sin ky e^{-2 nu k^2 t}, v = u0 sin kx cos ky e^{...},
    rho = 1 - u0^2 / (4 cs2) (cos 2kx + cos 2ky) e^{-4 nu k^2 t}."""
    k = 2.0 * math.pi / N
    x = np.arange(N) + 0.5
    X, Y = np.meshgrid(x, x, indexing="xy")  # [j][i]
    dec = math.exp(-2.0 * nu * k * k * t)
    u = -u0 * np.cos(k * X) * np.sin(k * Y) * dec
    v = u0 * np.sin(k * X) * np.cos(k * Y) * dec
    rho = 1.0 - 0.75 * u0 * u0 * (np.cos(2 * k * X) + np.cos(2 * k * Y)) * dec * dec
    return rho.ravel(), u.ravel(), v.ravel()


@pytest.mark.parametrize("precision", ["f64", "f64x"])
def test_tgv2d_grid_convergence_order(precision, mph):
    tau, target = 0.8, 0.1
    nu = (tau - 0.5) / 3.0
    rows = []
    for N in (32, 64, 128):
        k = 2.0 * math.pi / N
        step = max(1, round(target / (nu * k * k)))
        d, info = mph.InputParser(text=TGV2D, overrides=[f"grid.ncells={N} {N}", f"lbm.tau={tau}",
                                                          "units.ref_velocity=0.02"]).derive(precision)
        u0 = info.u_lat  # the lattice value of units.ref_velocity (initData)
        s = mph.Simulation(d, info)
        rho, ux, uy = _tgv(N, u0, nu, 0.0)
        s.initialize(rho, np.concatenate([ux, uy]))
        s.advance(step + 1)  # the driver writes plt<step> after steps 0 .. step
        _, u = s.update_macroscopic()
        _, ex, ey = _tgv(N, u0, nu, s.time())
        err = max(np.abs(u[: N * N] - ex).max(), np.abs(u[N * N:] - ey).max()) / u0
        rows.append((N, step, err))
    orders = [math.log(rows[i - 1][2] / rows[i][2]) / math.log(2.0) for i in (1, 2)]
    print(f"TGV-2D {precision}: {rows} orders {orders}")
    assert min(orders) >= 1.8


# ---- plane Couette -------------------------------------------------------------
COUETTE2D = """
grid.ncells = 4 32
sim.max_step = 5000
lbm.lattice_type = D2Q9
units.ref_length = 1.0
units.ref_velocity = 1.0
units.Re = 32.0
bc.lo_type = Periodic NoSlip
bc.hi_type = Periodic MovingWall
bc.hiy_Uwall = 1.0 0.0
geometry.prob_lo = 0.0 0.0
geometry.prob_hi = 0.125 1.0
"""

COUETTE3D = """
grid.ncells = 4 4 32
sim.max_step = 5000
lbm.lattice_type = D3Q19
units.ref_length = 1.0
units.ref_velocity = 1.0
units.Re = 32.0
bc.lo_type = Periodic Periodic NoSlip
bc.hi_type = Periodic Periodic MovingWall
bc.hiz_Uwall = 1. 0.0 0.0
geometry.prob_lo = 0.0 0.0 0.0
geometry.prob_hi = 0.125 0.125 1.0
"""


def _couette_series(y, H, U0, nu, t, n_terms=200):
    u = U0 * y / H
    for n in range(1, n_terms + 1):
        arg = -n * n * math.pi ** 2 * nu * t / H ** 2
        if arg < -50:
            break
        u = u + 2 * U0 * (-1) ** n / (n * math.pi) * np.sin(n * math.pi * y / H) * math.exp(arg)
    return u


def _couette_case(lattice):
    """(inputs text, wall-normal axis, grid override at H wall-normal cells):
    the periodic extent scales with H as in convergence*.py (4 cells at
    H = 32), keeping the lattice square on the fixed geometry."""
    if lattice == "D2Q9":
        return COUETTE2D, 1, (lambda H: f"grid.ncells={max(1, round(H * 4 / 32))} {H}"), 1
    return COUETTE3D, 2, (lambda H: f"grid.ncells={max(1, round(H * 4 / 32))} {max(1, round(H * 4 / 32))} {H}"), 3


def _wall_profile(mph, s, d, wall_dim, H):
    """u_x averaged over the periodic directions, per wall-normal cell."""
    _, u = s.update_macroscopic()
    n = [d.n[0], d.n[1], d.n[2] if d.dim == 3 else 1]
    ux = u[: n[0] * n[1] * n[2]].reshape(n[2], n[1], n[0])
    return ux.mean(axis=(0, 2)) if wall_dim == 1 else ux.mean(axis=(1, 2))


@pytest.mark.parametrize("lattice", ["D2Q9", "D3Q15", "D3Q19", "D3Q27"])
def test_couette_convergence_order(lattice, mph):
    text, wall_dim, ncells, _ = _couette_case(lattice)
    tau, target = 0.8, 0.05
    nu = (tau - 0.5) / 3.0
    rows = []
    for H in (16, 32, 64):
        step = max(1, round(target * H * H / nu))
        d, info = mph.InputParser(text=text, overrides=[ncells(H), f"lbm.tau={tau}",
                                                        f"lbm.lattice_type={lattice}"]).derive("f64")
        s = mph.Simulation(d, info)
        s.initialize()
        s.advance(step + 1)
        U0 = d.face_U[2 * wall_dim + 1][0]
        _, u = s.update_macroscopic()
        n = [d.n[0], d.n[1], d.n[2] if d.dim == 3 else 1]
        ux = u[: n[0] * n[1] * n[2]].reshape(n[2], n[1], n[0])
        y = np.arange(H) + 0.5
        an = _couette_series(y, H, U0, nu, s.time())
        an = an[None, :, None] if wall_dim == 1 else an[:, None, None]
        rows.append((H, step, float(np.abs(ux - an).max() / U0)))
    orders = [math.log(rows[i - 1][2] / rows[i][2]) / math.log(2.0) for i in (1, 2)]
    print(f"Couette {lattice}: {rows} orders {orders}")
    assert min(orders) >= 1.8


@pytest.mark.parametrize("lattice", ["D2Q9", "D3Q15", "D3Q19", "D3Q27"])
def test_couette_startup_profile_and_decay_rate(lattice, mph):
    text, wall_dim, _, _ = _couette_case(lattice)
    d, info = mph.InputParser(text=text, overrides=[f"lbm.lattice_type={lattice}"]).derive("f64")
    s = mph.Simulation(d, info)
    s.initialize()
    H = 32
    U0 = d.face_U[2 * wall_dim + 1][0]
    nu = (1.0 / d.omega - 0.5) / 3.0
    y = np.arange(H) + 0.5
    yn = y / H
    times, errs, log_a1 = [], [], []
    done = 0
    for step in range(0, 5001, 50):  # amr.plot_int = 50 up to sim.max_step = 5000
        s.advance(step + 1 - done)
        done = step + 1
        prof = _wall_profile(mph, s, d, wall_dim, H)
        t = s.time()
        times.append(t)
        errs.append(float(np.abs(prof - _couette_series(y, H, U0, nu, t)).max() / U0))
        a1 = float(np.sum((prof / U0 - yn) * np.sin(np.pi * yn)) * 2.0 / H)
        log_a1.append(math.log(abs(a1)) if abs(a1) > 1e-12 else float("nan"))
    la = np.array(log_a1)
    valid = np.where(~np.isnan(la))[0]
    skip = min(3, len(valid) // 4)
    idx = valid[skip:]
    slope = np.polyfit(np.array(times)[idx], la[idx], 1)[0]
    rate = -(math.pi ** 2) * nu / H ** 2
    prof_err = max(errs[1:])
    rate_err = abs(slope - rate) / abs(rate)
    print(f"Couette {lattice}: profile err {prof_err:.3e} rate rel err {rate_err:.3e}")
    assert prof_err < 0.01 and rate_err < 0.01
