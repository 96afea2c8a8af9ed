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


@pytest.mark.parametrize("precision", ["f64", "f32", "bf16s"])
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
