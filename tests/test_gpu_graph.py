"""Small single domains advance in runs of steps replayed from CUDA graphs
(one graph per buffer the state starts in): the result equals plain
one-launch-per-step advances bit for bit across run remainders, odd step
counts, obstacle changes between advances (which re-capture) and the
fixed-point range flag."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair(mph, monkeypatch, desc_fn):
    monkeypatch.setenv("MPH_GRAPH_STEPS", "0")
    plain = mph.Simulation(desc_fn())
    monkeypatch.setenv("MPH_GRAPH_STEPS", "8")
    graphed = mph.Simulation(desc_fn())
    monkeypatch.delenv("MPH_GRAPH_STEPS")
    return plain, graphed


@pytest.mark.parametrize("precision", ["f64", "f64x", "f32", "f16s", "f16c", "f16w"])
def test_graph_runs_equal_plain_launches(precision, mph, monkeypatch):
    faces = ["NoSlip", "NoSlip", "NoSlip", "MovingWall", "Periodic", "Periodic"]
    U = [[0.0] * 3 for _ in range(6)]
    U[3] = [0.08, 0.0, 0.0]
    n = (96, 80)
    plain, graphed = _pair(mph, monkeypatch, lambda: mph.make_desc("D2Q9", n, 1.4, faces=faces, face_U=U,
                                                                     precision=precision))
    rng = np.random.default_rng(9)
    N = n[0] * n[1]
    rho, u = 1 + 0.01 * rng.standard_normal(N), 0.02 * rng.standard_normal(2 * N)
    for s in (plain, graphed):
        s.initialize(rho, u)
    mask = np.zeros((n[1], n[0]), np.uint8)
    mask[30:40, 20:35] = 1
    for k in (1, 19, 8, 3):
        plain.advance(k)
        graphed.advance(k)
    for s in (plain, graphed):
        s.set_obstacles(mask)
    for k in (17, 16):
        plain.advance(k)
        graphed.advance(k)
    assert plain.time() == graphed.time() == 64
    assert np.array_equal(plain.f(), graphed.f())


def test_graph_runs_3d_forced_and_timed(mph, monkeypatch):
    faces = ["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic", "Periodic"]
    plain, graphed = _pair(mph, monkeypatch, lambda: mph.make_desc("D3Q19", (24, 20, 16), 1.5, faces=faces,
                                                                     force=(1e-5, 0.0, 0.0), precision="f64x"))
    for s in (plain, graphed):
        s.initialize()
    plain.advance(41)
    graphed.advance_timed(41)
    assert np.array_equal(plain.f(), graphed.f())


def test_graph_runs_report_the_range_flag(mph, monkeypatch):
    """A near-vacuum state (set on the host) trips the fixed-point range flag
    inside a replayed run: the advance returns MPH_ERR_NONFINITE."""
    monkeypatch.setenv("MPH_GRAPH_STEPS", "8")
    s = mph.Simulation(mph.make_desc("D2Q9", (32, 32), 1.2, precision="f64x"))
    monkeypatch.delenv("MPH_GRAPH_STEPS")
    s.initialize(np.full(32 * 32, 1e-3), np.zeros(2 * 32 * 32))
    with pytest.raises(mph.MphError) as ei:
        s.advance(16)
    assert ei.value.code == 6
