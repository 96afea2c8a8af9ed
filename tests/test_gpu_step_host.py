"""mph_step_host over host buffers.  Domains of 32 MB of FP64 populations and
more take the slab pipeline (planes of the outermost axis uploaded, stepped
and downloaded in turn, both copy directions in flight at once); every case
here is above that size, and each must give the bits of the resident path
(set_f, advance, f) -- in place or into a second buffer, pageable or
page-locked, one step or several, with walls or periodic wrap across the
slab axis, slabs of one plane, and interior obstacles."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PREC = ["f64", "f64x", "f32", "f16s", "bf16s", "f16c", "f16w"]
CH3 = ["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic", "Periodic"]


def _state(mph, d, seed):
    """A developed state: initialized from random fields, advanced a few steps."""
    s = mph.Simulation(d)
    rng = np.random.default_rng(seed)
    N, dim = s.ncell, d.dim
    s.initialize(1.0 + 0.01 * rng.standard_normal(N), 0.03 * rng.standard_normal(dim * N))
    s.advance(3)
    return s


def _check(mph, d, nsteps, inplace, pinned, seed=1, mask=None):
    a = _state(mph, d, seed)
    b = mph.Simulation(d)
    if mask is not None:
        a.set_obstacles(mask)
        b.set_obstacles(mask)
    f0 = a.f()
    assert f0.size * 8 >= 32 << 20, "case below the pipeline size"
    a.set_f(f0)  # the FP64 view converted back, as step_host converts it
    a.advance(nsteps)
    want = a.f()
    bufs = []
    if pinned:
        bufs = [mph.PinnedArray(f0.size) for _ in range(1 if inplace else 2)]
        src = bufs[0].array
        dst = src if inplace else bufs[1].array
    else:
        src = np.empty_like(f0)
        dst = src if inplace else np.empty_like(f0)
    src[:] = f0
    b.step_host(src, dst, nsteps)
    ok = np.array_equal(dst, want)
    if not inplace:
        ok = ok and np.array_equal(src, f0)  # input untouched
    assert b.time() == nsteps
    got_resident = b.f()
    for p in bufs:
        p.close()
    assert ok
    assert np.array_equal(got_resident, want)  # the handle holds the result too


@pytest.mark.parametrize("precision", PREC)
@pytest.mark.parametrize("nsteps", [1, 3])
def test_channel_slabs_equal_resident(precision, nsteps, mph):
    d = mph.make_desc("D3Q19", (64, 64, 64), 1 / 0.6, faces=CH3, force=(1e-5, 0, 0), precision=precision)
    _check(mph, d, nsteps, inplace=True, pinned=True)


@pytest.mark.parametrize("precision", ["f64", "f64x", "f16s"])
def test_separate_pageable_buffers(precision, mph):
    d = mph.make_desc("D3Q19", (64, 64, 64), 1 / 0.6, faces=CH3, force=(1e-5, 0, 0), precision=precision)
    _check(mph, d, 2, inplace=False, pinned=False)


@pytest.mark.parametrize("precision", ["f64", "f64x", "f32"])
def test_one_plane_slabs_walls_across_slab_axis(precision, mph):
    """nz = 5: five slabs of one plane; z faces are walls (no wrap)."""
    U = [[0.0] * 3 for _ in range(6)]
    U[5] = [0.05, 0.02, 0.0]
    d = mph.make_desc("D3Q27", (256, 256, 5), 1.3, faces=["Periodic", "Periodic", "Periodic", "Periodic", "NoSlip",
                                                          "MovingWall"], face_U=U, precision=precision)
    _check(mph, d, 1, inplace=True, pinned=True, seed=2)
    _check(mph, d, 4, inplace=False, pinned=True, seed=3)


@pytest.mark.parametrize("precision", ["f64x", "bf16s"])
def test_three_slabs_periodic_wrap(precision, mph):
    """nz = 3: the fewest slabs the pipeline takes; every slab pulls across the wrap."""
    d = mph.make_desc("D3Q19", (320, 320, 3), 1.1, faces=["Periodic"] * 6, force=(0, 1e-5, 2e-6),
                      precision=precision)
    _check(mph, d, 1, inplace=True, pinned=True, seed=4)
    _check(mph, d, 2, inplace=True, pinned=False, seed=5)


@pytest.mark.parametrize("precision", ["f64", "f32", "f16s"])
def test_2d_row_slabs_open_boundaries(precision, mph):
    """D2Q9 slabs of rows (uneven: 600 rows over 16 slabs), inflow / pressure
    outlet along x, no-slip and moving walls along y."""
    U = [[0.0] * 3 for _ in range(6)]
    U[0] = [0.03, 0.0, 0.0]
    U[3] = [0.05, 0.0, 0.0]
    d = mph.make_desc("D2Q9", (1024, 600), 1.5, faces=["Inflow", "PressureOutlet", "NoSlip", "MovingWall",
                                                       "Periodic", "Periodic"], face_U=U,
                      face_rho=[1.0, 1.002, 1.0, 1.0, 1.0, 1.0], precision=precision)
    _check(mph, d, 1, inplace=True, pinned=True, seed=6)
    _check(mph, d, 3, inplace=False, pinned=True, seed=7)


@pytest.mark.parametrize("precision", ["f64x", "f16s", "f64"])
def test_obstacles_across_slab_edges(precision, mph):
    """A sphere that straddles slab boundaries (slabs of 4 planes)."""
    n = 64
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    mask = ((x - 30) ** 2 + (y - 33) ** 2 + (z - 31) ** 2) < 9 ** 2
    d = mph.make_desc("D3Q19", (n, n, n), 1 / 0.6, faces=CH3, force=(1e-5, 0, 0), precision=precision)
    _check(mph, d, 1, inplace=True, pinned=True, seed=8, mask=mask)
    _check(mph, d, 3, inplace=True, pinned=True, seed=9, mask=mask)


def test_pipeline_matches_oracle(mph, oracle_mod):
    """FP64 (reference operation order) through the pipeline against the oracle."""
    O = oracle_mod
    faces = ["Periodic", "Periodic", "NoSlip", "MovingWall", "Periodic", "Periodic"]
    U = [[0.0] * 3 for _ in range(6)]
    U[3] = [0.04, 0.0, 0.0]
    n = (64, 64, 64)
    cfg = O.Config("D3Q19", n, omega=1.25, faces=faces, face_U=U, face_rho=[1.0] * 6, force=(2e-6, 0, 0))
    o = O.OracleSim(cfg, "port")
    d = mph.make_desc("D3Q19", n, 1.25, faces=faces, face_U=U, force=(2e-6, 0, 0))
    s = _state(mph, d, 10)
    f0 = s.f()
    o.set_f(f0)
    o.fill_ghosts()  # the reference fills ghosts at the end of each step
    o.step(2, nthreads=4)
    b = mph.Simulation(d)
    buf = mph.PinnedArray(f0.size)
    buf.array[:] = f0
    b.step_host(buf.array, buf.array, 2)
    ok = np.array_equal(buf.array, o.get_f())
    buf.close()
    o.close()
    assert ok


def test_small_domain_takes_block_copies(mph):
    """Below 32 MB one block copy per direction: same bits."""
    d = mph.make_desc("D3Q19", (24, 20, 16), 1.4, faces=CH3, force=(1e-5, 0, 0), precision="f64x")
    a = _state(mph, d, 11)
    b = mph.Simulation(d)
    f0 = a.f()
    a.set_f(f0)
    a.advance(2)
    out = np.empty_like(f0)
    b.step_host(f0, out, 2)
    assert np.array_equal(out, a.f())


@pytest.mark.parametrize("slabs", ["0", "3", "5", "64"])
def test_slab_count_override(slabs, mph, monkeypatch):
    """MPH_STEP_HOST_SLABS: 0 forces the block copies, others the slab count
    (capped at the number of planes)."""
    monkeypatch.setenv("MPH_STEP_HOST_SLABS", slabs)
    d = mph.make_desc("D3Q19", (64, 64, 64), 1 / 0.6, faces=CH3, force=(1e-5, 0, 0), precision="f64x")
    _check(mph, d, 2, inplace=True, pinned=True, seed=12)
