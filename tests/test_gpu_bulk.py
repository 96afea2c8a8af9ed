"""The 16-bit pair step with its pull operands staged in shared memory by bulk
asynchronous copies (MPH_PAIR_KERNEL=bulk) against the direct pair kernel:
the same populations bit for bit after many steps, on every lattice, forced
and unforced, periodic and walled faces, inflow / outlet faces, chunks of one
row and of several rows, row lengths that are not multiples of 8 elements (so
the staged runs are widened to 16-byte boundaries and the array's last
elements are read directly), every stage count, and through the slab
pipeline of mph_step_host."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(mph, desc, bulk, stages=3, cells=512):
    keys = ("MPH_PAIR_KERNEL", "MPH_BULK_STAGES", "MPH_BULK_CELLS")
    old = {k: os.environ.get(k) for k in keys}
    try:
        os.environ["MPH_PAIR_KERNEL"] = "bulk" if bulk else "direct"
        os.environ["MPH_BULK_STAGES"] = str(stages)
        os.environ["MPH_BULK_CELLS"] = str(cells)
        return mph.Simulation(desc)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


CASES = [
    # lattice, n, faces, force, face U, face rho
    ("D2Q9", (64, 48), ["NoSlip", "NoSlip", "NoSlip", "MovingWall", "Periodic", "Periodic"], None,
     {3: [0.08, 0, 0]}, None),
    ("D2Q9", (34, 30), ["Periodic"] * 6, (1e-5, -2e-6, 0), None, None),
    ("D3Q19", (32, 20, 18), ["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic", "Periodic"], (2e-5, 0, 0),
     None, None),
    ("D3Q27", (22, 18, 14), ["Periodic"] * 6, None, None, None),
    ("D3Q15", (26, 12, 10), ["Inflow", "PressureOutlet", "NoSlip", "MovingWall", "NoSlip", "NoSlip"], None,
     {0: [0.03, 0, 0], 3: [0.05, 0, 0]}, [1, 1.01, 1, 1, 1, 1]),
    ("D3Q19", (24, 16, 12), ["Periodic", "Periodic", "Periodic", "Periodic", "NoSlip", "MovingWall"], None,
     {5: [0.04, 0.01, 0]}, None),
]


def _desc(mph, case, prec):
    lat, n, faces, force, U, rho = case
    face_U = [[0.0] * 3 for _ in range(6)]
    for k, v in (U or {}).items():
        face_U[k] = v
    return mph.make_desc(lat, n, 1.3, faces=faces, face_U=face_U, face_rho=rho, force=force, precision=prec)


def _init(s, n, dim, seed):
    rng = np.random.default_rng(seed)
    N = int(np.prod(n))
    s.initialize(1 + 0.01 * rng.standard_normal(N), 0.02 * rng.standard_normal(dim * N))


@pytest.mark.parametrize("prec", ["f16s", "bf16s", "f16c"])
@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}_{'x'.join(map(str, c[1]))}" for c in CASES])
def test_bulk_step_equals_direct_pair_step(case, prec, mph):
    d = _desc(mph, case, prec)
    dim = 2 if case[0] == "D2Q9" else 3
    a, b = _sim(mph, d, False), _sim(mph, d, True, stages=3, cells=2 * case[1][0])
    _init(a, case[1], dim, 7)
    _init(b, case[1], dim, 7)
    a.advance(41)
    b.advance(41)
    assert np.array_equal(a.f(), b.f())


@pytest.mark.parametrize("stages,cells", [(2, 2), (3, 100), (3, 512), (2, 4096)])
def test_bulk_step_every_stage_count_and_chunk_size(stages, cells, mph):
    case = CASES[2]
    d = _desc(mph, case, "f16s")
    a, b = _sim(mph, d, False), _sim(mph, d, True, stages=stages, cells=cells)
    _init(a, case[1], 3, 11)
    _init(b, case[1], 3, 11)
    a.advance(17)
    b.advance(17)
    assert np.array_equal(a.f(), b.f())


def test_bulk_step_large_channel_and_host_slabs(mph):
    """A 128^3 D3Q19 channel (rows of 128 cells, several rows per chunk),
    resident steps and the slab pipeline of mph_step_host (windows of planes)."""
    case = ("D3Q19", (128, 128, 128), ["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic", "Periodic"],
            (1e-6, 0, 0), None, None)
    d = _desc(mph, case, "f16s")
    a, b = _sim(mph, d, False), _sim(mph, d, True)
    _init(a, case[1], 3, 3)
    _init(b, case[1], 3, 3)
    a.advance(20)
    b.advance(20)
    fa = a.f()
    assert np.array_equal(fa, b.f())
    out_a, out_b = np.empty_like(fa), np.empty_like(fa)
    a.step_host(fa, out_a, 3)
    b.step_host(fa, out_b, 3)
    assert np.array_equal(out_a, out_b)


def test_bulk_step_rejects_bad_settings(mph):
    d = _desc(mph, CASES[0], "f16s")
    with pytest.raises(mph.MphError) as e:
        _sim(mph, d, True, stages=4)
    assert e.value.code == 1
