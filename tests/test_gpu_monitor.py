"""Steady-state residual norm (FP64 on the GPU) of single domains and batches:
the value against the same norm computed on the host from the downloaded
populations, the first-call and re-initialisation behaviour, agreement of
batch and single-domain residuals, and convergence of a small cavity."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

def _velocity(mph, desc, f):
    """u = (sum c f) / (sum f) of stored populations, FP64 on the host."""
    q, dim = desc.q, desc.dim
    lat = {9: "D2Q9", 15: "D3Q15", 19: "D3Q19", 27: "D3Q27"}[q]
    c = mph.lattice_tables(lat)[0].astype(np.float64)  # (q, 3)
    N = f.size // q
    F = f.reshape(q, N)
    rho = F.sum(axis=0)
    return np.stack([(c[:, d:d + 1] * F).sum(axis=0) / rho for d in range(dim)])


def _cavity(mph, n, tau, lid=0.1, precision="f64", lattice="D2Q9"):
    U = [[0.0] * 3 for _ in range(6)]
    U[3] = [lid, 0.0, 0.0]
    faces = ["NoSlip", "NoSlip", "NoSlip", "MovingWall", "Periodic", "Periodic"]
    return mph.make_desc(lattice, n, 1.0 / tau, faces=faces, face_U=U, precision=precision)


@pytest.mark.parametrize("precision", ["f64", "f32", "f16s", "f64x"])
def test_residual_matches_host_norm(precision, mph):
    d = _cavity(mph, (40, 36), 0.8, precision=precision)
    s = mph.Simulation(d)
    s.initialize()
    r0, n0 = s.residual()
    assert np.isinf(r0) and n0 == 0.0
    s.advance(50)
    u1 = _velocity(mph, d, s.f())
    r1, n1 = s.residual()
    s.advance(25)
    u2 = _velocity(mph, d, s.f())
    r2, n2 = s.residual()
    assert abs(n2 - np.linalg.norm(u2)) <= 1e-12 * np.linalg.norm(u2)
    ref = np.linalg.norm(u2 - u1) / np.linalg.norm(u2)
    assert abs(r2 - ref) <= 1e-10 * ref
    s.initialize()
    assert np.isinf(s.residual()[0])


@pytest.mark.parametrize("precision", ["f64", "f32", "bf16s", "f64x"])
def test_batch_residual_equals_single_domains(precision, mph):
    descs = [_cavity(mph, (17, 17), 0.7, precision=precision), _cavity(mph, (64, 48), 0.9, precision=precision),
             _cavity(mph, (33, 65), 0.6, 0.05, precision=precision)]
    b = mph.Batch(descs)
    singles = [mph.Simulation(x) for x in descs]
    for i, s in enumerate(singles):
        b.initialize(i)
        s.initialize()
    b.advance(40)
    r_b0, _ = b.residual()
    assert np.all(np.isinf(r_b0))
    for s in singles:
        s.advance(40)
        s.residual()
    b.advance(30)
    rb, nb = b.residual()
    for i, s in enumerate(singles):
        s.advance(30)
        r, n = s.residual()
        assert rb[i] == pytest.approx(r, rel=1e-12) and nb[i] == pytest.approx(n, rel=1e-12)


def test_small_cavity_reaches_residual_1e8(mph):
    """Re 100 cavity, 32 x 32, lid 0.1 (tau = 0.5 + 3 * 0.1 * 32 / 100): the
    residual over 100 steps falls below 1e-8 within 60k steps."""
    tau = 0.5 + 3 * 0.1 * 32 / 100.0
    s = mph.Simulation(_cavity(mph, (32, 32), tau))
    s.initialize()
    s.residual()
    steps = 0
    r = np.inf
    while steps < 60000 and not r < 1e-8:
        s.advance(100)
        steps += 100
        r, _ = s.residual()
    assert r < 1e-8, (steps, r)


def _neq_reference(mph, desc, rho, u, solid, tau):
    """NumPy restatement of the warm-start initialisation: feq + the
    post-collision first-order non-equilibrium part, -((tau - 1) w rho / cs2)
    (c c - cs2 I) : grad u."""
    c, w, _ = mph.lattice_tables("D2Q9")
    ny, nx = desc.n[1], desc.n[0]
    per = [desc.face_type[0] == mph.BC["Periodic"], desc.face_type[2] == mph.BC["Periodic"]]
    U = u.reshape(2, ny, nx)
    R = rho.reshape(ny, nx)
    S = solid.reshape(ny, nx).astype(bool)
    G = np.zeros((2, 2, ny, nx))  # G[a][b] = d_a u_b
    for a, (ax, n) in enumerate([(1, nx), (0, ny)]):
        for b in range(2):
            up = np.roll(U[b], -1, axis=ax)
            um = np.roll(U[b], 1, axis=ax)
            okp = ~np.roll(S, -1, axis=ax)
            okm = ~np.roll(S, 1, axis=ax)
            if not per[a]:
                idx = [slice(None)] * 2
                idx[ax] = -1
                okp[tuple(idx)] = False
                idx[ax] = 0
                okm[tuple(idx)] = False
            g = np.where(okp & okm, 0.5 * (up - um), np.where(okp, up - U[b], np.where(okm, U[b] - um, 0.0)))
            G[a, b] = g
    div = G[0, 0] + G[1, 1]
    usq = U[0] ** 2 + U[1] ** 2
    f = np.empty((9, ny, nx))
    for n in range(9):
        cu = c[n, 0] * U[0] + c[n, 1] * U[1]
        feq = w[n] * R * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * usq)
        cc = sum(c[n, a] * c[n, b] * G[a, b] for a in range(2) for b in range(2))
        f[n] = feq - 3.0 * (tau - 1.0) * w[n] * R * (cc - div / 3.0)
        f[n][S] = w[n]
    return f.reshape(9, -1)


def test_warm_start_initialisation_matches_restatement(mph):
    nx, ny = 36, 28
    U6 = [[0.0] * 3 for _ in range(6)]
    U6[3] = [0.05, 0, 0]
    tau = 0.7
    d = mph.make_desc("D2Q9", (nx, ny), 1 / tau, faces=["Periodic", "Periodic", "NoSlip", "MovingWall", "Periodic",
                                                        "Periodic"], face_U=U6, precision="f64")
    rng = np.random.default_rng(4)
    yy, xx = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    u = np.stack([0.03 * np.sin(2 * np.pi * xx / nx) * np.cos(np.pi * yy / ny),
                  0.02 * np.cos(2 * np.pi * xx / nx)]).reshape(-1)
    rho = 1 + 0.001 * rng.standard_normal(nx * ny)
    solid = np.zeros((ny, nx), np.uint8)
    solid[10:14, 5:9] = 1
    s = mph.Simulation(d)
    s.set_obstacles(solid)
    s.initialize_neq(rho, u)
    ref = _neq_reference(mph, d, rho, u, solid, tau)
    got = s.f()
    assert np.max(np.abs(got - ref.reshape(-1))) < 1e-14
    # f_neq carries no mass or momentum: the moments of the stored f are (rho, u)
    F = got.reshape(9, -1)
    fluid = solid.reshape(-1) == 0
    c, _, _ = mph.lattice_tables("D2Q9")
    assert np.allclose(F.sum(0)[fluid], rho[fluid], rtol=0, atol=1e-14)
    assert np.allclose((c[:, 0:1] * F).sum(0)[fluid], (rho * u[: nx * ny])[fluid], rtol=0, atol=1e-14)


@pytest.mark.parametrize("precision", ["f64", "f32", "f16s", "bf16s", "f64x"])
def test_native_state_round_trip_resumes_bit_for_bit(precision, mph):
    """mph_get_state / mph_set_state carry the storage format itself, so a
    run continued from a copy matches the uninterrupted run bit for bit."""
    import ctypes as C
    L = mph.lib()
    d = _cavity(mph, (24, 20), 0.7, precision=precision)
    a, b = mph.Simulation(d), mph.Simulation(d)
    a.initialize()
    a.advance(30)
    n = C.c_longlong()
    mph.check(L.mph_state_bytes(a._h, C.byref(n)))
    buf = (C.c_ubyte * n.value)()
    mph.check(L.mph_get_state(a._h, buf, n))
    mph.check(L.mph_set_state(b._h, buf, n))
    a.advance(25)
    b.advance(25)
    assert np.array_equal(a.f(), b.f())
    assert L.mph_set_state(b._h, buf, n.value - 1) != 0
