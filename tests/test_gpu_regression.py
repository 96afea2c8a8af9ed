"""The reference's regression drivers (tests/regression/{couette, poiseuille}/
main.cpp) restated as GPU tests on the library: plane Couette start-up
against the series solution, body-force Poiseuille (periodic, and
Inflow / PressureOutlet with the corner-corrected inflow velocity) against
the parabola, with the reference's own acceptance limits where it states
them."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COUETTE = """
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

POISEUILLE = """
grid.ncells = 4 32
sim.max_step = 25600
lbm.lattice_type = D2Q9
units.ref_length = 0.5
units.ref_velocity = 1.0
units.Re = 16.0
forcing.accel = 0.125 0.0
bc.lo_type = Periodic NoSlip
bc.hi_type = Periodic NoSlip
geometry.prob_lo = 0.0 0.0
geometry.prob_hi = 0.125 1.0
"""

POISEUILLE_INFLOW = """
grid.ncells = 96 16
sim.max_step = 12000
lbm.lattice_type = D2Q9
lbm.tau = 0.8
units.ref_length = 0.5
units.ref_velocity = 1.0
units.Re = 16.0
units.ref_density = 1.0
forcing.accel = 5.4 0.0
bc.lo_type = Inflow NoSlip
bc.hi_type = PressureOutlet NoSlip
bc.lox_Uin = 0.408510638297872 0.0
geometry.prob_lo = 0.0 0.0
geometry.prob_hi = 1.0 0.1666666666666667
"""


def _couette_series(y, H, U0, nu, t, n_terms=200):
    u = U0 * y / H
    for n in range(1, n_terms + 1):
        arg = -n * n * math.pi ** 2 * nu * t / H ** 2
        if arg < -50:
            break
        u += 2 * U0 * (-1) ** n / (n * math.pi) * np.sin(n * math.pi * y / H) * math.exp(arg)
    return u


@pytest.mark.parametrize("precision", ["f64", "f64x"])
def test_couette_startup(precision, mph):
    d, info = mph.InputParser(text=COUETTE).derive(precision)
    s = mph.Simulation(d, info)
    s.initialize()
    H, U0, nu = 32.0, d.face_U[3][0], (1.0 / d.omega - 0.5) / 3.0
    y = np.arange(32) + 0.5
    errs = {}
    done = 0
    for step in (50, 500, 5000):
        s.advance(step + 1 - done)  # loop steps 0 .. step
        done = step + 1
        ux = s.update_macroscopic()[1][: 4 * 32].reshape(32, 4).mean(axis=1)
        errs[step] = float(np.max(np.abs(ux - _couette_series(y, H, U0, nu, s.time()))) / U0)
    print("Couette max |u - series| / U0:", errs)
    assert errs[5000] < 1e-3 and errs[500] < 2e-2 and errs[50] < 5e-2


@pytest.mark.parametrize("precision", ["f64", "f64x"])
def test_poiseuille_periodic(precision, mph):
    d, info = mph.InputParser(text=POISEUILLE).derive(precision)
    s = mph.Simulation(d, info)
    s.initialize()
    s.advance(25601)
    rho, u = s.update_macroscopic()
    H, F, nu = 32.0, d.force[0], (1.0 / d.omega - 0.5) / 3.0
    y = np.arange(32) + 0.5
    Umax = F * H * H / (8 * nu)
    ux = u[:128].reshape(32, 4)
    uy = u[128:].reshape(32, 4)
    ua = (F / (2 * nu) * y * (H - y))[:, None]
    assert np.max(np.abs(ux - ua)) / Umax < 1.5e-3            # test.max_rel_err (inputs)
    assert abs(ux.mean() - 2.0 / 3.0 * Umax) / Umax < 1.5e-3
    assert np.max(np.abs(uy)) / Umax < 1e-6                    # default test.max_transverse
    assert rho.max() - rho.min() < 1e-8                        # default test.max_rho_spread


def test_poiseuille_inflow_outflow(mph):
    d, info = mph.InputParser(text=POISEUILLE_INFLOW).derive("f64")
    s = mph.Simulation(d, info)
    s.initialize()
    s.advance(12001)
    rho, u = s.update_macroscopic()
    nx, ny = 96, 16
    H, F, nu = float(ny), d.force[0], (1.0 / d.omega - 0.5) / 3.0
    Umax = F * H * H / (8 * nu)
    Uin = d.face_U[0][0]
    assert abs(Uin - 2.0 / 3.0 * Umax * 3 * H / (3 * H - 1)) < 1e-6 * Umax
    i_lo, i_hi = round(0.5 * nx), round(0.8 * nx)           # test.window = 0.5 0.8
    y = np.arange(ny) + 0.5
    ux = u[: nx * ny].reshape(ny, nx)[:, i_lo:i_hi]
    uy = u[nx * ny:].reshape(ny, nx)[:, i_lo:i_hi]
    r = rho.reshape(ny, nx)[:, i_lo:i_hi]
    ua = (F / (2 * nu) * y * (H - y))[:, None]
    assert np.max(np.abs(ux - ua)) / Umax < 5e-3              # inputs: test.max_rel_err
    assert abs(ux.mean() - 2.0 / 3.0 * Umax) / Umax < 5e-3
    assert np.max(np.abs(uy)) / Umax < 4e-5                    # test.max_transverse
    assert r.max() - r.min() < 2e-5                            # test.max_rho_spread
