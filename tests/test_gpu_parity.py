"""CUDA step against the reference: bit-exact FP64 parity with the golden
fixtures (generated by the reference's own LBM sources) and with the CPU
oracle; tolerance parity for the refactored FP64, FP32 and shifted 16-bit
paths; moments, initial conditions, reductions, host-buffer step and the
plugin-level Array4 kernels."""
import ctypes as C

import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu


def _init(sim, case):
    name = case["name"]
    if case["kind"] == "fields":
        r, u = sim.initialize(G.arr(name, "rho0"), G.arr(name, "u0"))
        return r, u
    sim.set_f(G.arr(name, "f0"))
    return None, None


@pytest.mark.parametrize("idx", range(48))
def test_exact_step_matches_golden_bitwise(idx, mph):
    case = G.cases()[idx]
    name = case["name"]
    sim = mph.Simulation(G.product_desc(case, mph, "f64"))
    r, u = _init(sim, case)
    if r is not None:
        assert np.array_equal(r, G.arr(name, "rho_init"))
        assert np.array_equal(u, G.arr(name, "u_init"))
    assert np.array_equal(sim.f(), G.arr(name, "f_init"))
    sim.advance(case["steps"])
    assert np.array_equal(sim.f(), G.arr(name, "f_final"))
    rho, vel = sim.update_macroscopic()
    assert np.array_equal(rho, G.arr(name, "rho_final"))
    assert np.array_equal(vel, G.arr(name, "u_final"))
    assert sim.time() == case["steps"]


def _pair(mph, O, lattice, n, faces, omega, force=None, face_U=None, face_rho=None, precision="f64"):
    cfg = O.Config(lattice, n, omega=omega, faces=faces, face_U=face_U or [[0.0] * 3 for _ in range(6)],
                   face_rho=face_rho or [1.0] * 6, force=force)
    d = mph.make_desc(lattice, n, omega, faces=faces, face_U=cfg.face_U, face_rho=cfg.face_rho, force=force,
                      precision=precision)
    return O.OracleSim(cfg, "port"), mph.Simulation(d)


def _fields(rng, N, dim, amp=0.04):
    return 1.0 + 0.01 * rng.standard_normal(N), amp * rng.standard_normal(dim * N)


LONG = [
    ("D2Q9", (64, 48), ["Periodic"] * 6, 1.25, None, None, 500),
    ("D2Q9", (48, 40), ["NoSlip", "NoSlip", "NoSlip", "MovingWall", "Periodic", "Periodic"], 1.44, None,
     {3: [0.1, 0, 0]}, 800),
    ("D3Q19", (24, 20, 16), ["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic", "Periodic"], 1.0 / 0.6,
     (1e-5, 0.0, 0.0), None, 200),
    ("D3Q15", (16, 12, 10), ["Inflow", "PressureOutlet", "Periodic", "Periodic", "NoSlip", "NoSlip"], 1.25,
     (2e-5, 0, 0), {0: [0.02, 0, 0]}, 150),
    ("D3Q27", (12, 10, 14), ["Inflow", "Outflow", "NoSlip", "MovingWall", "Periodic", "Periodic"], 1.6,
     None, {0: [0.03, 0, 0], 3: [0.05, 0, 0.02]}, 150),
]


@pytest.mark.parametrize("case", LONG, ids=[f"{c[0]}_{c[6]}" for c in LONG])
def test_exact_long_runs_bitwise_vs_oracle(case, mph, oracle_mod):
    lat, n, faces, omega, force, U, steps = case
    face_U = [[0.0] * 3 for _ in range(6)]
    for k, v in (U or {}).items():
        face_U[k] = v
    o, s = _pair(mph, oracle_mod, lat, n, faces, omega, force, face_U)
    rng = np.random.default_rng(11)
    rho, u = _fields(rng, o.N, o.cfg.dim)
    ro, uo = o.init_fields(rho, u)
    rs, us = s.initialize(rho, u)
    assert np.array_equal(ro, rs) and np.array_equal(uo, us)
    o.step(steps, nthreads=8)
    s.advance(steps)
    assert np.array_equal(o.get_f(), s.f())
    mo, ms = o.moments(), s.update_macroscopic()
    assert np.array_equal(mo[0], ms[0]) and np.array_equal(mo[1], ms[1])


def _relerr(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


@pytest.mark.parametrize("prec", ["f64_fast", "f64x"])
@pytest.mark.parametrize("case", LONG, ids=[f"{c[0]}_{c[6]}" for c in LONG])
def test_fp64_accurate_paths_within_1e12(case, prec, mph, oracle_mod):
    lat, n, faces, omega, force, U, steps = case
    face_U = [[0.0] * 3 for _ in range(6)]
    for k, v in (U or {}).items():
        face_U[k] = v
    o, s = _pair(mph, oracle_mod, lat, n, faces, omega, force, face_U, precision=prec)
    rng = np.random.default_rng(12)
    rho, u = _fields(rng, o.N, o.cfg.dim)
    o.init_fields(rho, u)
    s.initialize(rho, u)
    o.step(steps, nthreads=8)
    s.advance(steps)
    err = _relerr(s.f(), o.get_f())
    print(f"{prec} max rel err in f after {steps} steps: {err:.3e}")
    assert err < 1e-12  # tolerance of the FP64 parity requirement
    ro, uo = o.moments()
    rs, us = s.update_macroscopic()
    assert np.max(np.abs(rs - ro)) < 1e-12 and np.max(np.abs(us - uo)) < 1e-12


@pytest.mark.parametrize("idx", range(48))
def test_f64x_golden_within_1e12(idx, mph):
    """The fixed-point path on the reference-generated fixtures (random
    initial populations included)."""
    case = G.cases()[idx]
    name = case["name"]
    sim = mph.Simulation(G.product_desc(case, mph, "f64x"))
    _init(sim, case)
    sim.advance(case["steps"])
    ref = G.arr(name, "f_final")
    err = float(np.max(np.abs(sim.f() - ref) / np.abs(ref)))
    assert err < 1e-12, err


PIPE = [
    ("D2Q9", (300, 37), ["Periodic"] * 6, 1.3, None, None),
    ("D2Q9", (257, 20), ["NoSlip", "NoSlip", "NoSlip", "MovingWall", "Periodic", "Periodic"], 1.5, None,
     {3: [0.08, 0, 0]}),
    ("D3Q19", (40, 24, 18), ["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic", "Periodic"], 1.6,
     (1e-5, 0.0, 0.0), None),
    ("D3Q15", (19, 12, 10), ["Inflow", "PressureOutlet", "Periodic", "Periodic", "NoSlip", "NoSlip"], 1.25,
     (2e-5, 0, 0), {0: [0.02, 0, 0]}),
    ("D3Q27", (270, 6, 5), ["Inflow", "Outflow", "NoSlip", "MovingWall", "Periodic", "Periodic"], 1.6, None,
     {0: [0.03, 0, 0], 3: [0.05, 0, 0.02]}),
]


@pytest.mark.parametrize("case", PIPE, ids=[f"{c[0]}_{c[1][0]}" for c in PIPE])
def test_f64x_pipelined_kernel_equals_direct_kernel(case, mph, monkeypatch):
    """The persistent cp.async kernel (MPH_F64X_KERNEL=pipe) and the default
    one-cell-per-thread kernel compute the same integers."""
    lat, n, faces, omega, force, U = case
    face_U = [[0.0] * 3 for _ in range(6)]
    for k, v in (U or {}).items():
        face_U[k] = v
    d = mph.make_desc(lat, n, omega, faces=faces, face_U=face_U, force=force, precision="f64x")
    rng = np.random.default_rng(13)
    N = int(np.prod(n))
    rho, u = _fields(rng, N, len(n))
    out = []
    for kernel in ("pipe", "direct"):
        monkeypatch.setenv("MPH_F64X_KERNEL", kernel)
        s = mph.Simulation(d)
        s.initialize(rho.copy(), u.copy())
        s.advance(37)
        out.append(s.f())
    assert np.array_equal(out[0], out[1])


def test_f64x_range_flag_reports_instead_of_wrapping(mph):
    """Fault injection on the host: a near-vacuum state (rho = 1e-3, below the
    fixed-point range) makes the step report MPH_ERR_NONFINITE, and keeps
    reporting it until a new state replaces the bad one; then the same handle
    steps normally."""
    d = mph.make_desc("D3Q19", (8, 8, 8), 1.2, precision="f64x")
    s = mph.Simulation(d)
    N = 8 * 8 * 8
    s.initialize(np.full(N, 1e-3), np.zeros(3 * N))
    with pytest.raises(mph.MphError) as e:
        s.advance(1)
    assert e.value.code == 6
    with pytest.raises(mph.MphError) as e:
        s.advance(1)
    assert e.value.code == 6
    s.initialize(np.ones(N), np.zeros(3 * N))
    s.advance(3)
    assert np.allclose(s.f().reshape(19, N).sum(axis=0), 1.0, atol=1e-14)


# Reduced precisions: velocity error relative to the FP64 oracle, L2 over the
# domain divided by the L2 norm of the oracle velocity, after up to 200 steps
# from a random (non-smooth) field.  Plain FP32 storage rounds f ~ w to 24 bits
# (measured 3e-6..8e-5); shifted FP16 / BF16 / the custom 1-4-11 format keep
# 11 / 8 / 12 bits of f - w (measured 1.9e-4..4.2e-4 / 1.4e-3..3.1e-3 /
# 9.0e-5..1.8e-4); the weight-scaled 1-3-12 format 13 bits of (f - w) / w.
TOL_LOWP = {"f32": 3e-4, "f16s": 3e-3, "bf16s": 1.5e-2, "f16c": 1e-3, "f16w": 1e-3}


@pytest.mark.parametrize("prec", ["f32", "f16s", "bf16s", "f16c", "f16w"])
@pytest.mark.parametrize("case", LONG[:3], ids=[f"{c[0]}_{c[6]}" for c in LONG[:3]])
def test_reduced_precision_velocity_error(case, prec, mph, oracle_mod):
    lat, n, faces, omega, force, U, steps = case
    face_U = [[0.0] * 3 for _ in range(6)]
    for k, v in (U or {}).items():
        face_U[k] = v
    o, s = _pair(mph, oracle_mod, lat, n, faces, omega, force, face_U, precision=prec)
    rng = np.random.default_rng(13)
    rho, u = _fields(rng, o.N, o.cfg.dim, amp=0.02)
    o.init_fields(rho, u)
    s.initialize(rho, u)
    steps = min(steps, 200)
    o.step(steps, nthreads=8)
    s.advance(steps)
    _, uo = o.moments()
    _, us = s.update_macroscopic()
    err = float(np.linalg.norm(us - uo) / np.linalg.norm(uo))
    print(f"{prec} velocity rel-L2 err after {steps} steps: {err:.3e}")
    assert err < TOL_LOWP[prec]


def test_reduce_sums(mph, oracle_mod):
    o, s = _pair(mph, oracle_mod, "D3Q19", (20, 18, 16), ["Periodic"] * 6, 1.3, (1e-4, 2e-5, -3e-5))
    rng = np.random.default_rng(5)
    rho, u = _fields(rng, o.N, 3)
    s.initialize(rho, u)
    s.advance(20)
    f = s.f().reshape(19, -1)
    red = s.reduce()
    assert abs(red[0] - f.sum()) / f.sum() < 1e-13
    # momentum through the moments of a uniform shift: compare against oracle
    o.init_fields(rho, u)
    o.step(20)
    fo = o.get_f().reshape(19, -1)
    assert abs(red[0] - fo.sum()) / fo.sum() < 1e-13


def test_step_host_equals_resident_steps(mph):
    d = mph.make_desc("D3Q19", (16, 12, 10), 1.4, faces=["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic",
                                                         "Periodic"], force=(1e-5, 0, 0))
    a, b = mph.Simulation(d), mph.Simulation(d)
    rng = np.random.default_rng(9)
    rho, u = _fields(rng, a.ncell, 3)
    a.initialize(rho, u)
    f0 = a.f()
    a.advance(7)
    out = np.empty_like(f0)
    b.step_host(f0, out, 7)
    assert np.array_equal(out, a.f())
    # the same through page-locked buffers from mph_host_alloc
    pin_in, pin_out = mph.PinnedArray(f0.size), mph.PinnedArray(f0.size)
    pin_in.array[:] = f0
    b.step_host(pin_in.array, pin_out.array, 7)
    assert np.array_equal(pin_out.array, out)
    pin_in.close()
    pin_out.close()


def _dev_a4(mph, torch, arr_ghost, q, ext):
    """A ghost-grown Array4 on the device, begin = -1 in each grown direction."""
    t = torch.from_numpy(arr_ghost.copy()).cuda()
    a = mph.Array4()
    a.p = t.data_ptr()
    gx, gy, gz = ext
    a.jstride, a.kstride, a.nstride = gx, gx * gy, gx * gy * gz
    return t, a


@pytest.mark.parametrize("lat,n,faces,force", [
    ("D2Q9", (10, 8), ["Inflow", "PressureOutlet", "NoSlip", "MovingWall", "Periodic", "Periodic"], None),
    ("D3Q19", (6, 5, 4), ["Periodic", "Periodic", "NoSlip", "MovingWall", "Outflow", "Inflow"], (1e-4, 0, 2e-5)),
    ("D3Q27", (5, 6, 4), ["Periodic"] * 6, (1e-4, -1e-4, 0)),
])
def test_plugin_array4_kernels_bitwise(lat, n, faces, force, mph, oracle_mod):
    torch = pytest.importorskip("torch")
    O = oracle_mod
    dim, q = O.LATTICE_DQ[lat]
    U = [[0.0] * 3 for _ in range(6)]
    U[0][0] = 0.02
    U[3][0] = 0.06
    U[5][2] = -0.01
    cfg = O.Config(lat, n, omega=1.3, faces=faces, face_U=U, force=force)
    o = O.OracleSim(cfg, "port")
    rng = np.random.default_rng(1)
    o.set_f(rng.uniform(0.5, 1.5, q * o.N) / q)
    o.fill_ghosts()
    g0 = o.get_f_ghost()
    o.step(1)
    g1 = o.get_f_ghost()
    ext = (n[0] + 2, n[1] + 2, (n[2] + 2) if dim == 3 else 1)
    tin, ain = _dev_a4(mph, torch, g0, q, ext)
    tout, aout = _dev_a4(mph, torch, np.full_like(g0, np.nan), q, ext)
    for a in (ain, aout):
        for d in range(3):
            a.begin[d] = -1 if d < dim else 0
            a.end[d] = (n[d] + 1) if d < dim else 1
        a.ncomp = q
    lo = (C.c_int * 3)(0, 0, 0)
    hi = (C.c_int * 3)(n[0] - 1, n[1] - 1, (n[2] - 1) if dim == 3 else 0)
    per = (C.c_int * 3)(*[int(d < dim and faces[2 * d] == "Periodic") for d in range(3)])
    F = (C.c_double * 3)(*(force or (0, 0, 0)))
    L = mph.lib()
    mph.check(L.mph_pull_collide_fused_arr(dim, q, lo, hi, C.byref(ain), C.byref(aout), 1.3,
                                           F if force else None, None))
    mph.check(L.mph_periodic_fill_arr(dim, q, lo, hi, per, C.byref(aout), None))
    d = mph.make_desc(lat, n, 1.3, faces=faces, face_U=U)
    tab = (mph.ResolvedBC * 27)()
    mph.check(L.mph_resolve_bc(C.byref(d), tab))
    mph.check(L.mph_bc_fill_arr(dim, q, lo, hi, per, tab, C.byref(aout), None))
    torch.cuda.synchronize()
    got = tout.cpu().numpy()
    assert np.array_equal(got, g1, equal_nan=True)


def test_plugin_rejects_too_small_array(mph):
    L = mph.lib()
    a = mph.Array4()
    a.p = 16
    a.jstride, a.kstride, a.nstride = 4, 16, 16
    for d in range(3):
        a.begin[d] = 0
        a.end[d] = 4 if d < 2 else 1
    a.ncomp = 9
    lo = (C.c_int * 3)(0, 0, 0)
    hi = (C.c_int * 3)(3, 3, 0)
    assert L.mph_pull_collide_fused_arr(2, 9, lo, hi, C.byref(a), C.byref(a), 1.0, None, None) == 1


@pytest.mark.parametrize("precision", ["f64", "f64x", "f32", "f16s", "f16c", "f16w"])
@pytest.mark.parametrize("lat,n", [("D2Q9", (20, 16)), ("D3Q19", (12, 10, 8)), ("D3Q27", (10, 8, 6))])
def test_zero_force_is_bit_identical_to_unforced(lat, n, precision, mph):
    """The forced kernels with F = 0 reproduce the unforced ones bit for bit
    (the reference's F = 0 identity of the Guo path, test_forcing.cpp) where
    the arithmetic is explicitly rounded (FP64 reference order, fixed point,
    shifted 16-bit); the FP32 path leaves FMA contraction to the compiler, so
    its two instantiations agree to rounding."""
    faces = ["Periodic", "Periodic", "NoSlip", "MovingWall", "Periodic", "Periodic"]
    U = [[0.0] * 3 for _ in range(6)]
    U[3] = [0.05, 0.0, 0.0]
    kw = dict(faces=faces, face_U=U, precision=precision)
    a = mph.Simulation(mph.make_desc(lat, n, 1.3, **kw))
    b = mph.Simulation(mph.make_desc(lat, n, 1.3, force=(0.0, 0.0, 0.0), **kw))
    rng = np.random.default_rng(3)
    # the weight-scaled 16-bit format holds populations within w +- p (|u| up
    # to about 0.1): random velocities of standard deviation 0.02 stay inside
    rho, u = _fields(rng, a.ncell, len(n), amp=0.02 if precision == "f16w" else 0.04)
    a.initialize(rho.copy(), u.copy())
    b.initialize(rho.copy(), u.copy())
    a.advance(23)
    b.advance(23)
    if precision == "f32":
        assert np.max(np.abs(a.f() - b.f())) <= 1e-6
    else:
        assert np.array_equal(a.f(), b.f())
