"""The allocation-free sums entry point (mph_reduce_f64_noalloc), for callers
that cannot allocate device memory: called through the C ABI on caller-owned
device buffers, it must agree with the handle-based mph_reduce, on two calls
in a row (the second call reuses the library's fixed scratch array).  This
file is collected last so that a run stopping at the first failure has run
every other test first."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(rng, N, dim):
    return 1.0 + 0.01 * rng.standard_normal(N), 0.04 * rng.standard_normal(dim * N)


# Cell counts against the 65,536-cell chunk of each scratch slot: one partial
# chunk (D3Q19, 46,080 cells), and two chunks with a partial last one for every
# lattice (D2Q9 77,100; D3Q15 72,000; D3Q27 84,480), so the cz terms of the
# 3-D lattices and the multi-slot final pass are both covered.
@pytest.mark.parametrize("lat,n", [("D3Q19", (40, 36, 32)), ("D2Q9", (300, 257)), ("D3Q15", (50, 40, 36)),
                                   ("D3Q27", (48, 44, 40))])
def test_noalloc_sums_match_handle_sums_twice(lat, n, mph):
    torch = pytest.importorskip("torch")
    dim, q = mph.LATTICE_DQ[lat]
    d = mph.make_desc(lat, n, 1.3, force=(1e-4, -2e-5, 3e-5)[:dim] + (0.0,) * (3 - dim))
    sim = mph.Simulation(d)
    rng = np.random.default_rng(17)
    sim.initialize(*_fields(rng, sim.ncell, dim))
    sim.advance(5)
    ref = sim.reduce()                      # the existing entry point
    f = torch.from_numpy(sim.f()).cuda()    # caller-owned device populations
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    L = mph.lib()
    for call in range(2):
        mph.check(L.mph_reduce_f64_noalloc(dim, q, f.data_ptr(), sim.ncell, out.data_ptr(), None))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        # same tolerance as the handle-based sum test: 1e-13 relative to the mass
        assert abs(got[0] - ref[0]) < 1e-13 * abs(ref[0]), (call, got, ref)
        assert np.all(np.abs(got[1:] - ref[1:]) < 1e-13 * abs(ref[0])), (call, got, ref)
        out.fill_(float("nan"))


def test_noalloc_rejects_sizes_beyond_the_fixed_scratch(mph):
    torch = pytest.importorskip("torch")
    L = mph.lib()
    f = torch.zeros(19, dtype=torch.float64, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = L.mph_reduce_f64_noalloc(3, 19, f.data_ptr(), 2048 * 65536 + 1, out.data_ptr(), None)
    assert rc == 1
    assert b"exceed" in L.mph_last_error()
