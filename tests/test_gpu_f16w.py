"""The weight-scaled 16-bit storage of MPH_PREC_F16W ((f - w) / p, p the power
of two nearest to w, as sign, 3 exponent bits biased by 8, 12 mantissa
bits) against a NumPy restatement from its definition: the stored bits of
mph_set_f are the format's rounding of the FP32 deviation f - w, the FP64
view of mph_get_f decodes them exactly (power-of-two scales), the rounding
error stays within half a unit in the last place (2^-13 relative for
normals, 2^-20 absolute for subnormals, in units of p), magnitudes from
1 - 2^-14 up saturate at the largest value, and a step whose stores saturate
reports MPH_ERR_NONFINITE instead of continuing silently."""
import numpy as np
import pytest

from f16w_ref import decode_ref, pscale, round_ref

pytestmark = pytest.mark.gpu


def _sim(mph, n=(256, 64), lat="D2Q9", **kw):
    return mph.Simulation(mph.make_desc(lat, n, 1.0, precision="f16w", **kw))


def test_f16w_storage_bits_and_values(mph):
    s = _sim(mph)
    _, w, _ = mph.lattice_tables("D2Q9")
    N = 256 * 64
    W = np.repeat(w, N)
    P = pscale(W)
    assert np.all((0.75 * W <= P) & (P <= 1.125 * W))
    rng = np.random.default_rng(4)
    # deviations over the whole range: normals, subnormals, zero, both signs,
    # values near ties of the 12-bit rounding, values that saturate
    mag = np.exp2(rng.uniform(-25.0, 0.3, 9 * N))
    x = np.where(rng.random(9 * N) < 0.5, -mag, mag)
    x[:64] = 0.0
    x[64:128] = (1.0 + (2 * np.arange(64) + 1) / 8192.0) * np.exp2(rng.integers(-7, 0, 64))
    f = W + P * x
    with pytest.raises(mph.MphError) as e:  # the saturating values are reported, and stored saturated
        s.set_f(f)
    assert e.value.code == 6
    nbytes = 2 * 9 * N
    raw = np.empty(nbytes, np.uint8)
    mph.check(mph.lib().mph_get_state(s._h, raw.ctypes.data, nbytes))
    bits = raw.view(np.uint16).astype(np.uint32)
    # the device's FP32 steps: g = f32(f) - f32(w), then v = g 2^-119 / p (an
    # FP32 product: exact, except that below 2^-30 p it lands on the FP32
    # subnormal grid before the 12-bit rounding), rounded on the grid of x
    W32 = W.astype(np.float32)
    g32 = (f.astype(np.float32) - W32).astype(np.float32)
    xr = g32.astype(np.float64) / P
    v32 = (g32 * (2.0 ** -119 / P).astype(np.float32)).astype(np.float32)
    ref = round_ref(v32.astype(np.float64) * 2.0 ** 119)
    assert np.array_equal(bits, ref), np.flatnonzero(bits != ref)[:10]
    # decoding: g = x p exactly, then f32(g + f32(w))
    xd = decode_ref(bits)
    fv = ((xd * P).astype(np.float32) + W32).astype(np.float64)
    assert np.array_equal(s.f(), fv)
    # saturation and rounding error in units of p (the largest value is 1 - 2^-13)
    assert np.all((bits[np.abs(xr) >= 1.0] & 0x7FFF) == 0x7FFF)
    fin = np.abs(xr) < 1.0 - 2.0 ** -13
    err = np.abs(xd - xr)
    normal = np.abs(xr) >= 2.0 ** -7
    # half a unit of the 13-bit significand or of the subnormal step
    lim = np.where(normal, np.abs(xr) * 2.0 ** -13, 2.0 ** -20)
    assert np.all(err[fin] <= lim[fin])


def test_f16w_saturating_upload_and_init_report_nonfinite(mph):
    """Populations outside the format's range are reported where they are
    stored: mph_set_f and mph_init_fields return MPH_ERR_NONFINITE (the state
    is kept, saturated), the steps keep reporting it, and a state within the
    range clears it."""
    n = (32, 16)
    N = n[0] * n[1]
    s = _sim(mph, n=n, faces=["Periodic"] * 6)
    _, w, _ = mph.lattice_tables("D2Q9")
    f = np.repeat(w, N).copy()
    f[N + 5] = 2.5 * w[1]          # (f - w) / p = 1.33: beyond the largest value
    with pytest.raises(mph.MphError) as e:
        s.set_f(f)
    assert e.value.code == 6
    with pytest.raises(mph.MphError) as e:
        s.advance(1)
    assert e.value.code == 6
    s.set_f(np.repeat(w, N))
    s.advance(2)
    with pytest.raises(mph.MphError) as e:  # u = 0.5 along x: (f - w) / p of the population along it is 2.0
        s.initialize(np.ones(N), np.concatenate([np.full(N, 0.5), np.zeros(N)]))
    assert e.value.code == 6
    s.initialize(np.ones(N), np.zeros(2 * N))
    s.advance(2)


def test_f16w_saturating_step_reports_nonfinite(mph):
    """A uniform flow at u = 0.2 ((f - w) / w = 0.72 for the population along
    the flow, p = 9 w / 8) accelerated by a body force of 0.05 per step passes
    u = 0.29, where that population's deviation reaches p: the step's stores
    saturate and the handle reports MPH_ERR_NONFINITE (code 6) instead of
    continuing.  Without the force the same flow steps normally."""
    N = 64 * 32
    u = np.concatenate([np.full(N, 0.2), np.zeros(N)])
    for force in (None, (0.05, 0.0, 0.0)):
        s = _sim(mph, n=(64, 32), faces=["Periodic"] * 6, force=force)
        s.initialize(np.ones(N), u.copy())
        if force:
            with pytest.raises(mph.MphError) as e:
                s.advance(8)
            assert e.value.code == 6
            # a new state clears the status: from rest the forced flow stays in range
            s.initialize(np.ones(N), np.zeros(2 * N))
            s.advance(2)
        else:
            s.advance(8)
            _, uu = s.update_macroscopic()
            assert abs(uu[:N].mean() - 0.2) < 1e-4


def test_f16w_error_below_f16c_on_a_shear_wave(mph):
    """A decaying shear wave (u0 = 0.05) on a periodic D3Q19 domain, 400
    steps: the velocity error against the FP64-accurate fixed-point run is
    below that of the 1-4-11 format, whose significand has one bit less
    (measured 2.2e-4 against 3.8e-4)."""
    n = (64, 48, 32)
    N = int(np.prod(n))
    y = (np.arange(n[1]) + 0.5) / n[1]
    ux = 0.05 * np.sin(2 * np.pi * y)[None, :, None] * np.ones((n[2], 1, n[0]))   # [z][y][x]
    u = np.concatenate([ux.reshape(-1), np.zeros(N), np.zeros(N)])
    rho = 1 + 1e-3 * np.cos(2 * np.pi * y)[None, :, None] * np.ones((n[2], 1, n[0]))
    out = {}
    for p in ("f64x", "f16c", "f16w"):
        s = mph.Simulation(mph.make_desc("D3Q19", n, 1.0 / 0.55, faces=["Periodic"] * 6, precision=p))
        s.initialize(rho.reshape(-1).copy(), u.copy())
        s.advance(400)
        out[p] = s.update_macroscopic()[1]
        s.close()
    ref = out["f64x"]
    err = {p: float(np.linalg.norm(out[p] - ref) / np.linalg.norm(ref)) for p in ("f16c", "f16w")}
    print("shear wave velocity error after 400 steps:", err)
    assert err["f16w"] < 0.8 * err["f16c"] and err["f16w"] < 3e-4


def test_f16w_batch_flags_the_saturating_domain(mph):
    """In a batch, the weight-scaled storage flags the domain whose stores
    saturate (a forced flow driven past the range) and the advance reports
    MPH_ERR_NONFINITE; the other domains step on, equal to single handles,
    and re-initialising the flagged domain clears its flag."""
    n = (64, 32)
    N = n[0] * n[1]
    descs = [mph.make_desc("D2Q9", n, 1.0, faces=["Periodic"] * 6, force=(f, 0.0, 0.0), precision="f16w")
             for f in (1e-5, 0.05, 2e-5)]
    b = mph.Batch(descs)
    u = np.concatenate([np.full(N, 0.2), np.zeros(N)])
    for d in range(3):
        b.initialize(d, np.ones(N), u.copy())
    with pytest.raises(mph.MphError) as e:
        b.advance(8)
    assert e.value.code == 6
    assert list(b.range_flags()) == [False, True, False]
    for d in (0, 2):
        s = mph.Simulation(descs[d])
        s.initialize(np.ones(N), u.copy())
        s.advance(8)
        assert np.array_equal(b.f(d), s.f())
    b.initialize(1, np.ones(N), np.zeros(2 * N))
    assert not b.range_flags().any()
    # an upload outside the range names its domain too
    _, w, _ = mph.lattice_tables("D2Q9")
    f = np.repeat(w, N).copy()
    f[3] = 3.0 * w[0]
    with pytest.raises(mph.MphError) as e:
        b.set_f(2, f)
    assert e.value.code == 6
    assert list(b.range_flags()) == [False, False, True]
