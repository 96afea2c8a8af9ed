"""The custom 16-bit storage format of MPH_PREC_F16C (f - w as sign, 4
exponent bits biased by 16, 11 mantissa bits) against a NumPy restatement
from its definition: stored bits of mph_set_f equal the format's rounding of
the FP32 deviation, the FP64 view of mph_get_f decodes them exactly, and the
rounding error stays within half a unit in the last place (2^-12 relative
for normals, 2^-27 absolute for subnormals); magnitudes of 1 and more
saturate at the largest value, 1 - 2^-12."""
import numpy as np
import pytest

from f16c_ref import decode_ref, encode_ref

pytestmark = pytest.mark.gpu


def test_f16c_storage_bits_and_values(mph):
    d = mph.make_desc("D2Q9", (256, 64), 1.0, precision="f16c")
    s = mph.Simulation(d)
    _, w, _ = mph.lattice_tables("D2Q9")
    N = 256 * 64
    rng = np.random.default_rng(4)
    # deviations over the whole range: normals, subnormals, zero, both signs,
    # values near ties of the 11-bit rounding, and values that saturate
    mag = np.exp2(rng.uniform(-32.0, 1.2, 9 * N))
    g = np.where(rng.random(9 * N) < 0.5, -mag, mag)
    g[:64] = 0.0
    g[64:128] = (1.0 + (2 * np.arange(64) + 1) / 4096.0) * np.exp2(rng.integers(-14, 0, 64))
    f = g + np.repeat(w, N)
    s.set_f(f)
    nbytes = 2 * 9 * N
    raw = np.empty(nbytes, np.uint8)
    mph.check(mph.lib().mph_get_state(s._h, raw.ctypes.data, nbytes))
    bits = raw.view(np.uint16).astype(np.uint32)
    # the device stores the FP32 deviation of the FP32 population
    g32 = (f.astype(np.float32) - np.repeat(w.astype(np.float32), N)).astype(np.float32)
    ref = encode_ref(g32)
    # double rounding through the FP32 rebias can move a subnormal by one unit
    diff = np.abs(bits.astype(np.int64) - ref.astype(np.int64))
    normal = np.abs(g32) >= 2.0 ** -15
    assert np.all(diff[normal] == 0), np.flatnonzero(diff[normal])[:10]
    assert np.all(diff[~normal] <= 1)
    # decoding: the FP64 view is decode(bits) + w rounded through FP32
    got = s.f() - np.repeat(w, N)
    dec = decode_ref(bits)
    dv = (dec.astype(np.float32) + np.repeat(w.astype(np.float32), N)).astype(np.float64) - np.repeat(w, N)
    assert np.array_equal(got, dv)
    # rounding error bounds where the value is representable (the largest
    # value is 2^-1 (2 - 2^-11) = 1 - 2^-12; from 1 - 2^-13 on it saturates)
    assert np.all((bits[np.abs(g32) >= 1.0] & 0x7FFF) == 0x7FFF)
    fin = np.abs(g32) < 1.0 - 2.0 ** -13
    err = np.abs(dec - g32.astype(np.float64))
    lim = np.where(normal, np.abs(g32) * 2.0 ** -12, 2.0 ** -27) * (1 + 1e-12) + np.where(normal, 0, 2.0 ** -26)
    assert np.all(err[fin] <= lim[fin])
