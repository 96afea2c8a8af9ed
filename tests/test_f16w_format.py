"""The conversion steps of the weight-scaled 16-bit format (MPH_PREC_F16W) on
the CPU, against the format's definition (`f16w_ref`): the device encodes an
FP32 deviation g with one FP32 multiply by 2^(8-127) / p and rounds the FP32
bits to nearest even at bit 11 (saturating above 0x7FFF), and decodes by
placing the 15 magnitude bits at FP32 bit 11 and multiplying by p 2^(127-8).
Restated here operation by operation in NumPy's IEEE FP32 (subnormals kept),
the steps must give the definition's codes for every tie of the 12-bit
rounding in every binade, values one FP32 unit either side of the ties,
subnormals down to the FP32 subnormal range, the saturation boundary and
random values; the GPU test checks the device against the same definition."""
import numpy as np

from f16w_ref import decode_ref, pscale, round_ref

W = {"D2Q9": [4 / 9, 1 / 9, 1 / 36], "D3Q15": [2 / 9, 1 / 9, 1 / 72], "D3Q19": [1 / 3, 1 / 18, 1 / 36],
     "D3Q27": [8 / 27, 2 / 27, 1 / 54, 1 / 216]}


def encode_steps(g32, p):
    """The device's encode of FP32 deviations g32 for scale p: (codes, saturated)."""
    v32 = (g32 * np.float32(2.0 ** -119 / p)).astype(np.float32)
    u = v32.view(np.uint32).astype(np.uint64)
    a = u & 0x7FFFFFFF
    r = (a + 0x3FF + ((a >> 11) & 1)) >> 11
    code = ((u >> 16) & 0x8000) | np.minimum(r, 0x7FFF)
    return code.astype(np.uint32), r > 0x7FFF


def decode_steps(h, p):
    """The device's decode of codes h for scale p (FP32 g)."""
    h = h.astype(np.uint64)
    bits = (((h & 0x8000) << 16) | ((h & 0x7FFF) << 11)).astype(np.uint32)
    return (bits.view(np.float32) * np.float32(p * 2.0 ** 119)).astype(np.float32)


def _values(rng):
    xs = []
    for e in range(-7, 0):  # every 12-bit tie of each normal binade, and its FP32 neighbours
        ulp = 2.0 ** (e - 12)
        t = 2.0 ** e + (np.arange(4096) + 0.5) * ulp
        xs += [t, np.nextafter(t, 0), np.nextafter(t, 2)]
    t = (np.arange(4096) + 0.5) * 2.0 ** -19  # subnormal ties
    xs += [t, np.nextafter(t, 0), np.nextafter(t, 1)]
    xs.append(np.exp2(rng.uniform(-32.0, 0.2, 200000)))
    xs.append(np.array([0.0, 1.0 - 2.0 ** -13, 1.0 - 2.0 ** -14, 1.0 - 2.0 ** -15, 1.0, 1.5, 2.0 ** -7, 2.0 ** -30]))
    x = np.concatenate(xs)
    return np.concatenate([x, -x])


def test_encode_steps_equal_the_definition():
    rng = np.random.default_rng(12)
    x = _values(rng)
    for lat, ws in W.items():
        for w in ws:
            p = float(pscale(w))
            assert 0.75 * w <= p <= 1.125 * w, (lat, w)
            g32 = (x * p).astype(np.float32)          # FP32 deviations
            code, sat = encode_steps(g32, p)
            # the definition, applied to the FP32 product the device rounds
            v32 = (g32 * np.float32(2.0 ** -119 / p)).astype(np.float32)
            ref = round_ref(v32.astype(np.float64) * 2.0 ** 119)
            assert np.array_equal(code, ref), (lat, w, np.flatnonzero(code != ref)[:5])
            # the scaling multiply is exact wherever the product is an FP32 normal
            # (|x| >= 2^-7); below, it lands on the FP32 subnormal grid (2^-30 in
            # units of p), finer than the format's steps of 2^-19
            xr = g32.astype(np.float64) / p
            exact = np.abs(xr) >= 2.0 ** -7
            assert np.array_equal(v32.astype(np.float64)[exact] * 2.0 ** 119, xr[exact])
            assert np.all(np.abs(v32.astype(np.float64) * 2.0 ** 119 - xr) <= 2.0 ** -31)
            # saturation is flagged exactly where the rounded magnitude passes the largest value
            assert np.array_equal(sat, np.abs(xr) >= 1.0 - 2.0 ** -14)


def test_decode_steps_invert_exactly():
    h = np.arange(1 << 16, dtype=np.uint32)
    for ws in W.values():
        for w in ws:
            p = float(pscale(w))
            g = decode_steps(h, p).astype(np.float64)
            assert np.array_equal(g, decode_ref(h) * p)
            # encoding the decoded values gives the codes back (negative zero aside)
            code, sat = encode_steps(decode_steps(h, p), p)
            keep = (h & 0x7FFF) != 0
            assert np.array_equal(code[keep], h[keep]) and not sat.any()


def test_ties_round_to_even():
    """Exact ties of the 12-bit rounding go to the even code (no bias): the
    tie between mantissas k and k + 1 of a binade rounds to the even one, and
    the last tie of a binade carries into the next binade (mantissa 0), or
    saturates in the top binade."""
    p = float(pscale(1 / 9))
    k = np.arange(4096)
    for e in range(-7, 0):
        x = 2.0 ** e + (k + 0.5) * 2.0 ** (e - 12)
        code, sat = encode_steps((x * p).astype(np.float32), p)
        expect = np.where(k % 2 == 0, k, k + 1)
        assert np.array_equal(code[:-1] & 0xFFF, expect[:-1])
        assert np.all((code[:-1] >> 12) == e + 8)
        assert code[-1] == (0x7FFF if e == -1 else (e + 9) << 12)
        assert sat[-1] == (e == -1) and not sat[:-1].any()
