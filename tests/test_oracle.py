"""The CPU oracle against the golden fixtures produced by the reference's own
LBM sources, and the physics pins of the reference's unit tests
(tests/unit/test_lattice.cpp, test_equilibrium.cpp, test_forcing.cpp,
test_bc_corners.cpp, tests/regression/uniform_force/main.cpp)."""
import numpy as np
import pytest

import golden_cases as G


def _run_case(case, O, kind="port"):
    cfg = G.oracle_config(case, O)
    sim = O.OracleSim(cfg, kind)
    name = case["name"]
    if case["kind"] == "fields":
        r, u = sim.init_fields(G.arr(name, "rho0"), G.arr(name, "u0"))
        assert np.array_equal(r, G.arr(name, "rho_init"))
        assert np.array_equal(u, G.arr(name, "u_init"))
    else:
        sim.set_f(G.arr(name, "f0"))
        sim.fill_ghosts()
    assert np.array_equal(sim.get_f(), G.arr(name, "f_init"))
    sim.step(case["steps"], nthreads=2)
    return sim


@pytest.mark.parametrize("idx", range(48))
def test_oracle_matches_golden_bitwise(idx, oracle_mod):
    case = G.cases()[idx]
    sim = _run_case(case, oracle_mod)
    name = case["name"]
    assert np.array_equal(sim.get_f(), G.arr(name, "f_final"))
    # ghost layer too (NaN where the reference leaves a ghost population unset)
    assert np.array_equal(sim.get_f_ghost(), G.arr(name, "fg_final"), equal_nan=True)
    r, u = sim.moments()
    assert np.array_equal(r, G.arr(name, "rho_final"))
    assert np.array_equal(u, G.arr(name, "u_final"))


def test_oracle_matches_reference_build_directly(oracle_mod):
    O = oracle_mod
    if not O.ref_available():
        pytest.skip("reference-source build (oracle/_ref) not present on this host")
    rng = np.random.default_rng(3)
    for lat, n in (("D2Q9", (9, 7)), ("D3Q19", (4, 5, 6)), ("D3Q27", (5, 4, 3))):
        dim = O.LATTICE_DQ[lat][0]
        faces = ["Inflow", "PressureOutlet", "NoSlip", "MovingWall"] + (["Periodic", "Periodic"])
        U = [[0.0] * 3 for _ in range(6)]
        U[0][0] = 0.03
        U[3][0] = 0.07
        cfg = O.Config(lat, n, omega=1.3, faces=faces, face_rho=[1, 1.01, 1, 1, 1, 1], face_U=U,
                       force=(3e-5, -1e-5, 2e-5))
        a, b = O.OracleSim(cfg, "port"), O.OracleSim(cfg, "ref")
        N = a.N
        rho, u = 1 + 0.01 * rng.standard_normal(N), 0.03 * rng.standard_normal(dim * N)
        a.init_fields(rho, u)
        b.init_fields(rho, u)
        a.step(25, 3)
        b.step(25)
        assert np.array_equal(a.get_f(), b.get_f())


def test_reference_build_threaded_tiles_match_oracle(oracle_mod):
    """The reference build's OpenMP MFIter loops over 8-cell tiles (the form
    the reference arm of the benchmark times) give the restatement's bits:
    ragged last tiles along y and z, 4 threads over 9-12 tiles."""
    O = oracle_mod
    if not O.ref_available():
        pytest.skip("reference-source build (oracle/_ref) not present on this host")
    rng = np.random.default_rng(5)
    for lat, n in (("D2Q9", (13, 70)), ("D3Q19", (10, 21, 27)), ("D3Q27", (7, 17, 12))):
        dim = O.LATTICE_DQ[lat][0]
        faces = ["Periodic", "Periodic", "NoSlip", "MovingWall", "Periodic", "Periodic"]
        U = [[0.0] * 3 for _ in range(6)]
        U[3][0] = 0.05
        cfg = O.Config(lat, n, omega=1.6, faces=faces, face_U=U, force=(1e-5, 0.0, 0.0))
        a, b = O.OracleSim(cfg, "port"), O.OracleSim(cfg, "ref")
        N = a.N
        rho, u = 1 + 0.01 * rng.standard_normal(N), 0.02 * rng.standard_normal(dim * N)
        a.init_fields(rho, u)
        b.init_fields(rho, u)
        a.step(12, 2)
        b.step(12, 4)
        assert np.array_equal(a.get_f(), b.get_f()), lat


def _lattice(O, lat):
    """Velocity table of the oracle's lattice recovered through its moments:
    equilibrium populations at rho = 1, u = 0 are the weights."""
    dim, q = O.LATTICE_DQ[lat]
    n = (1, 1, 1) if dim == 3 else (1, 1)
    sim = O.OracleSim(O.Config(lat, n, omega=1.0), "port")
    sim.init_fields(np.ones(1), np.zeros(dim))
    return sim.get_f()


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q15", "D3Q19", "D3Q27"])
def test_weights_sum_to_one(lat, oracle_mod):
    # test_lattice.cpp: sum w = 1 (feq at rest equals w)
    w = _lattice(oracle_mod, lat)
    assert abs(w.sum() - 1.0) < 1e-15


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q15", "D3Q19", "D3Q27"])
def test_equilibrium_moments(lat, oracle_mod):
    # test_equilibrium.cpp:401-473: 20 random (rho, u); sum feq = rho and
    # sum c feq = rho u to 1e-12.  A one-cell periodic domain streams onto
    # itself, so its updateMacroscopic moments are those of the local feq.
    O = oracle_mod
    dim, q = O.LATTICE_DQ[lat]
    rng = np.random.default_rng(12345)
    n = (1, 1, 1) if dim == 3 else (1, 1)
    for _ in range(20):
        rho = np.array([1 + 0.1 * rng.uniform(-1, 1)])
        u = rng.uniform(-0.1, 0.1, dim)
        sim = O.OracleSim(O.Config(lat, n, omega=1.0), "port")
        sim.init_fields(rho, u)
        r2, u2 = sim.moments()
        assert abs(r2[0] - rho[0]) < 1e-12
        assert np.abs(u2 - u).max() < 1e-12


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
def test_uniform_force_regression(lat, oracle_mod):
    # tests/regression/uniform_force/main.cpp: periodic, quiescent start,
    # u_k = k F / rho after k steps, rho constant, to 1e-12.
    O = oracle_mod
    dim, q = O.LATTICE_DQ[lat]
    n = (8, 8, 8) if dim == 3 else (8, 8)
    F = (4e-4, -2e-4, 3e-4)[:dim] + (0.0,) * (3 - dim)
    sim = O.OracleSim(O.Config(lat, n, omega=1.25, force=F), "port")
    N = sim.N
    sim.init_fields(np.ones(N), np.zeros(dim * N))
    for k in range(1, 31):
        sim.step(1)
        if k % 5 == 0:
            rho, u = sim.moments()
            u = u.reshape(dim, N)
            for d in range(dim):
                assert np.abs(u[d] - k * F[d] / 1.0).max() < 1e-12
            assert np.abs(rho - 1.0).max() < 1e-12


def test_bc_corner_population_counts(oracle_mod):
    # test_bc_corners.cpp:531-548, 670-685: the D2Q9 (-1,-1) corner ghost
    # receives only the (1,1) population; the D3Q19 (-1,-1,-1) corner none.
    O = oracle_mod
    for lat, n, expect in (("D2Q9", (6, 6), 1), ("D3Q19", (4, 4, 4), 0)):
        dim, q = O.LATTICE_DQ[lat]
        cfg = O.Config(lat, n, omega=1.0, faces=["NoSlip"] * (2 * dim) + ["Periodic"] * (6 - 2 * dim))
        sim = O.OracleSim(cfg, "port")
        sim.set_f(np.random.default_rng(42).uniform(0.5, 1.5, q * sim.N))
        sim.fill_ghosts()
        g = sim.get_f_ghost().reshape(q, -1)
        corner = 0  # first ghost cell (-1,-1[,-1])
        assert int(np.isfinite(g[:, corner]).sum()) == expect


def test_bc_priority_and_conflicts(oracle_mod):
    # test_bc_corners.cpp:712-823 through the resolved table.
    O = oracle_mod
    cfg = O.Config("D2Q9", (4, 4), omega=1.0, faces=["NoSlip", "PressureOutlet", "NoSlip", "MovingWall", "Periodic", "Periodic"])
    rc, t, r, U = O.resolve_bc(cfg)
    assert rc == 0
    # class index = (code_x + 1) + 3 (code_y + 1)
    assert t[2 + 3 * 2] == O.BC["MovingWall"]      # MovingWall beats PressureOutlet
    assert t[0 + 3 * 2] == O.BC["NoSlip"]          # NoSlip beats MovingWall
    assert t[2 + 3 * 0] == O.BC["NoSlip"]          # NoSlip beats PressureOutlet
    bad = O.Config("D2Q9", (4, 4), omega=1.0, faces=["Inflow", "Outflow", "PressureOutlet", "NoSlip", "Periodic", "Periodic"])
    assert O.resolve_bc(bad)[0] != 0               # Outflow meets PressureOutlet at a corner
    two_moving = O.Config("D2Q9", (4, 4), omega=1.0, faces=["MovingWall", "NoSlip", "NoSlip", "MovingWall", "Periodic", "Periodic"])
    assert O.resolve_bc(two_moving)[0] != 0


# ---------------------------------------------------------------------------
# Interior obstacles (project-defined rule, no reference counterpart): a link
# whose upstream cell is solid bounces back (U = 0); solid cells hold f = w.
# ---------------------------------------------------------------------------
def _random_state(sim, seed, amp=0.02):
    rng = np.random.default_rng(seed)
    N, dim = sim.N, sim.cfg.dim
    sim.init_fields(1 + 0.01 * rng.standard_normal(N), amp * rng.standard_normal(dim * N))


def test_obstacles_all_fluid_mask_is_identity(oracle_mod):
    O = oracle_mod
    cfg = O.Config("D2Q9", (20, 14), omega=1.3, faces=["NoSlip", "NoSlip", "NoSlip", "MovingWall", "Periodic", "Periodic"],
                   face_U=[[0, 0, 0]] * 3 + [[0.05, 0, 0]] + [[0, 0, 0]] * 2)
    a, b = O.OracleSim(cfg, "port"), O.OracleSim(cfg, "port")
    _random_state(a, 1)
    _random_state(b, 1)
    b.set_obstacles(np.zeros(b.N, dtype=np.uint8))
    a.step(40)
    b.step(40)
    assert np.array_equal(a.get_f(), b.get_f())


@pytest.mark.parametrize("lat,n", [("D2Q9", (24, 20)), ("D3Q19", (12, 10, 8)), ("D3Q27", (10, 8, 8))])
def test_obstacles_conserve_fluid_mass(lat, n, oracle_mod):
    """Periodic box with a solid block: bounce-back at the block conserves the
    mass of the fluid cells."""
    O = oracle_mod
    sim = O.OracleSim(O.Config(lat, n, omega=1.2), "port")
    mask = np.zeros(n[::-1], dtype=np.uint8)
    if len(n) == 2:
        mask[5:11, 7:13] = 1
    else:
        mask[2:5, 3:6, 4:8] = 1
    _random_state(sim, 2)
    sim.set_obstacles(mask)
    fluid = mask.ravel() == 0
    q = sim.cfg.q
    m0 = sim.get_f().reshape(q, -1)[:, fluid].sum()
    sim.step(1)  # solid cells are set to the rest state on the first step
    m1 = sim.get_f().reshape(q, -1)[:, fluid].sum()
    s1 = sim.get_f().reshape(q, -1)[:, ~fluid]
    sim.step(300)
    m2 = sim.get_f().reshape(q, -1)[:, fluid].sum()
    assert abs(m2 - m1) < 1e-12 * m1
    assert abs(m1 - m0) < 1e-12 * m0
    s2 = sim.get_f().reshape(q, -1)[:, ~fluid]
    assert np.array_equal(s1, s2) and np.allclose(s2.sum(axis=0), 1.0, rtol=0, atol=1e-15)


def test_obstacle_plane_blocks_forced_flow(oracle_mod):
    """Periodic channel driven by a body force along x: a solid plane across
    the channel stops the mean flow; without it the flow accelerates."""
    O = oracle_mod
    n = (32, 12)
    cfg = O.Config("D2Q9", n, omega=1.0, force=(1e-5, 0.0, 0.0),
                   faces=["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic", "Periodic"])
    free, blocked = O.OracleSim(cfg, "port"), O.OracleSim(cfg, "port")
    for s in (free, blocked):
        s.init_fields(np.ones(s.N), np.zeros(2 * s.N))
    mask = np.zeros(n[::-1], dtype=np.uint8)
    mask[:, 16] = 1
    blocked.set_obstacles(mask)
    free.step(3000)
    blocked.step(3000)
    uf = free.moments()[1][: free.N].mean()
    fluid = mask.ravel() == 0
    ub = blocked.moments()[1][: blocked.N][fluid].mean()
    assert uf > 5e-4 and abs(ub) < 1e-3 * uf, (uf, ub)


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q15", "D3Q19", "D3Q27"])
def test_zero_force_path_is_bit_identical_to_unforced(lat, oracle_mod):
    # test_forcing.cpp: the forced kernel with F = 0 gives the unforced bits
    # (u gets + 0.5 * 0, the Guo term is exactly 0 and added as +0).
    O = oracle_mod
    dim, q = O.LATTICE_DQ[lat]
    n = (5, 4, 3) if dim == 3 else (6, 5)
    rng = np.random.default_rng(31)
    f0 = None
    out = []
    for force in (None, (0.0, 0.0, 0.0)):
        sim = O.OracleSim(O.Config(lat, n, omega=1.37, force=force), "port")
        if f0 is None:
            f0 = rng.uniform(0.5, 1.5, q * sim.N) / q
        sim.set_f(f0)
        sim.fill_ghosts()
        sim.step(7)
        out.append(sim.get_f())
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
def test_guo_step_moments(lat, oracle_mod):
    # test_forcing.cpp: one forced BGK step leaves the mass unchanged and adds
    # F to the momentum (a one-cell periodic domain streams onto itself, so the
    # step is the collision alone), from random non-equilibrium populations.
    O = oracle_mod
    dim, q = O.LATTICE_DQ[lat]
    n = (1, 1, 1) if dim == 3 else (1, 1)
    rng = np.random.default_rng(32)
    c = _velocities(O, lat)
    for _ in range(10):
        F = tuple(rng.uniform(-1e-3, 1e-3, dim)) + (0.0,) * (3 - dim)
        sim = O.OracleSim(O.Config(lat, n, omega=rng.uniform(0.6, 1.9), force=F), "port")
        f0 = _lattice(O, lat) * (1 + 0.05 * rng.standard_normal(q))
        sim.set_f(f0)
        sim.fill_ghosts()
        sim.step(1)
        f1 = sim.get_f()
        assert abs(f1.sum() - f0.sum()) < 1e-15
        assert np.abs(c.T @ f1 - c.T @ f0 - np.array(F[:dim])).max() < 1e-15


def _velocities(O, lat):
    """Velocity table of the oracle's lattice, recovered from streaming: on a
    3^D periodic box at rest, population n raised on one cell appears, after a
    pure-streaming step (omega = 0: no collision), at x + c_n."""
    dim, q = O.LATTICE_DQ[lat]
    n = (3, 3, 3) if dim == 3 else (3, 3)
    sim = O.OracleSim(O.Config(lat, n, omega=0.0), "port")
    N = sim.N
    c = np.zeros((q, dim))
    centre = 13 if dim == 3 else 4
    w = _lattice(O, lat)
    for k in range(q):
        f = np.repeat(w, N)
        f[k * N + centre] += 1.0
        sim.set_f(f)
        sim.fill_ghosts()
        sim.step(1)
        g = sim.get_f().reshape(q, N)[k]
        cell = int(np.argmax(g))
        coords = np.unravel_index(cell, tuple(reversed(n)))[::-1]
        base = np.unravel_index(centre, tuple(reversed(n)))[::-1]
        c[k] = np.array(coords) - np.array(base)
    return c


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q15", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("forced", [False, True])
def test_macroscopic_moments(lat, forced, oracle_mod):
    # test_macroscopic.cpp:59-158: rho = sum f, u = (sum c f [+ F / 2]) / rho,
    # on random populations (a one-cell periodic domain streams onto itself).
    O = oracle_mod
    dim, q = O.LATTICE_DQ[lat]
    n = (1, 1, 1) if dim == 3 else (1, 1)
    c = _velocities(O, lat)
    rng = np.random.default_rng(33)
    for _ in range(10):
        F = tuple(rng.uniform(-1e-3, 1e-3, dim)) + (0.0,) * (3 - dim) if forced else None
        sim = O.OracleSim(O.Config(lat, n, omega=1.0, force=F), "port")
        f = _lattice(O, lat) * rng.uniform(0.8, 1.2, q)
        sim.set_f(f)
        sim.fill_ghosts()
        rho, u = sim.moments()
        r = f.sum()
        j = c.T @ f + (0.5 * np.array(F[:dim]) if forced else 0.0)
        assert abs(rho[0] - r) < 1e-15
        assert np.abs(u - j / r).max() < 1e-16
