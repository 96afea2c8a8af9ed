"""Lattice invariants of the library's velocity sets (the checks of the
reference's test_lattice.cpp:21-112), read through the host-side table call
mph_lattice (no device needed), and the weights cross-checked against the
oracle's equilibrium at rest."""
import itertools

import numpy as np
import pytest

LATS = ["D2Q9", "D3Q15", "D3Q19", "D3Q27"]


def _tables(mph, lat):
    c, w, opp = mph.lattice_tables(lat)
    dim = mph.LATTICE_DQ[lat][0]
    return c[:, :dim], w, opp, dim


@pytest.mark.parametrize("lat", LATS)
def test_rest_population_first_and_velocities_distinct(lat, mph):
    c, w, opp, dim = _tables(mph, lat)
    q = len(w)
    assert np.all(c[0] == 0)
    assert len({tuple(v) for v in c}) == q
    assert np.all(np.abs(c) <= 1)


@pytest.mark.parametrize("lat", LATS)
def test_opposites(lat, mph):
    c, w, opp, dim = _tables(mph, lat)
    q = len(w)
    assert sorted(opp) == list(range(q))
    for n in range(q):
        assert np.all(c[opp[n]] == -c[n])
        assert opp[opp[n]] == n
        assert w[opp[n]] == w[n]
    assert opp[0] == 0


@pytest.mark.parametrize("lat", LATS)
def test_weight_and_velocity_moments(lat, mph):
    """sum w = 1, sum w c = 0, sum w c_a c_b = cs2 delta_ab with cs2 = 1/3,
    odd third moments vanish, and sum w c_a c_b c_c c_d = cs2^2 (d_ab d_cd +
    d_ac d_bd + d_ad d_bc) (isotropy needed by the second-order equilibrium)."""
    c, w, opp, dim = _tables(mph, lat)
    cs2 = 1.0 / 3.0
    assert abs(w.sum() - 1.0) < 1e-15
    assert np.all(w > 0)
    assert np.abs(w @ c).max() < 1e-15
    m2 = np.einsum("n,na,nb->ab", w, c, c)
    assert np.abs(m2 - cs2 * np.eye(dim)).max() < 1e-15
    m3 = np.einsum("n,na,nb,nc->abc", w, c, c, c)
    assert np.abs(m3).max() < 1e-15
    m4 = np.einsum("n,na,nb,nc,nd->abcd", w, c, c, c, c)
    d = np.eye(dim)
    want = cs2 * cs2 * (np.einsum("ab,cd->abcd", d, d) + np.einsum("ac,bd->abcd", d, d) +
                        np.einsum("ad,bc->abcd", d, d))
    assert np.abs(m4 - want).max() < 1e-15


@pytest.mark.parametrize("lat", LATS)
def test_weights_by_speed_class(lat, mph):
    """The published weights by |c|^2 class (rest, face, edge, corner)."""
    c, w, opp, dim = _tables(mph, lat)
    k = (c * c).sum(1)
    table = {"D2Q9": {0: 4 / 9, 1: 1 / 9, 2: 1 / 36},
             "D3Q15": {0: 2 / 9, 1: 1 / 9, 3: 1 / 72},
             "D3Q19": {0: 1 / 3, 1: 1 / 18, 2: 1 / 36},
             "D3Q27": {0: 8 / 27, 1: 2 / 27, 2: 1 / 54, 3: 1 / 216}}[lat]
    assert set(k.tolist()) == set(table)
    for kk, wk in table.items():
        assert np.all(np.abs(w[k == kk] - wk) < 1e-17)
    counts = {kk: int((k == kk).sum()) for kk in table}
    full = {kk: sum(1 for v in itertools.product((-1, 0, 1), repeat=dim) if sum(x * x for x in v) == kk)
            for kk in table}
    assert counts == full  # every velocity of each class present


@pytest.mark.parametrize("lat", LATS)
def test_weights_equal_oracle_rest_equilibrium(lat, mph, oracle_mod):
    """The oracle's equilibrium at rho = 1, u = 0 is its weight table; the
    library's table matches it bit for bit in the same population order."""
    O = oracle_mod
    dim, q = O.LATTICE_DQ[lat]
    n = (1, 1, 1) if dim == 3 else (1, 1)
    sim = O.OracleSim(O.Config(lat, n, omega=1.0), "port")
    sim.init_fields(np.ones(1), np.zeros(dim))
    w_oracle = sim.get_f()
    _, w, _, _ = _tables(mph, lat)
    assert np.array_equal(w, w_oracle)


@pytest.mark.parametrize("lat", LATS)
def test_velocities_equal_oracle_streaming(lat, mph, oracle_mod):
    """Population order: on a 3^D periodic box at rest, the oracle streams
    population n raised on one cell (omega = 0, no collision) to x + c_n with
    the library's c_n."""
    O = oracle_mod
    dim, q = O.LATTICE_DQ[lat]
    n = (3, 3, 3) if dim == 3 else (3, 3)
    c, w, _, _ = _tables(mph, lat)
    sim = O.OracleSim(O.Config(lat, n, omega=0.0), "port")
    N = sim.N
    centre = np.array([1] * dim)
    flat = lambda v: int(sum(int(v[a]) * 3 ** a for a in range(dim)))  # noqa: E731
    for k in range(q):
        f = np.repeat(w, N)
        f[k * N + flat(centre)] += 1.0
        sim.set_f(f)
        sim.fill_ghosts()
        sim.step(1)
        g = sim.get_f().reshape(q, N)[k]
        assert int(np.argmax(g)) == flat((centre + c[k]) % 3), k
