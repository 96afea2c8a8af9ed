"""The conversion steps of the 1-4-11 16-bit format (MPH_PREC_F16C) on the
CPU, against the format's definition (`f16c_ref`): the device encodes an FP32
deviation g with one FP32 multiply by 2^(16-127) and rounds the FP32 bits to
nearest even at bit 12 (saturating above 0x7FFF), and decodes by placing the
15 magnitude bits at FP32 bit 12 and multiplying by 2^(127-16).  Restated here
operation by operation in NumPy's IEEE FP32 (subnormals kept), the steps give
the definition's codes for every tie of the 11-bit rounding in every binade
and values one FP32 unit either side; below 2^-15 the multiply lands on the
FP32 subnormal grid first (2^-38, finer than the format's 2^-26 steps), which
can move a value onto a tie: one code at most, as the GPU test allows."""
import numpy as np

from f16c_ref import decode_ref, encode_ref


def encode_steps(g32):
    v32 = (g32 * np.float32(2.0 ** -111)).astype(np.float32)
    u = v32.view(np.uint32).astype(np.uint64)
    a = u & 0x7FFFFFFF
    r = (a + 0x7FF + ((a >> 12) & 1)) >> 12
    return (((u >> 16) & 0x8000) | np.minimum(r, 0x7FFF)).astype(np.uint32), v32


def decode_steps(h):
    h = h.astype(np.uint64)
    bits = (((h & 0x8000) << 16) | ((h & 0x7FFF) << 12)).astype(np.uint32)
    return (bits.view(np.float32) * np.float32(2.0 ** 111)).astype(np.float32)


def test_encode_steps_equal_the_definition():
    rng = np.random.default_rng(21)
    xs = []
    for e in range(-15, 0):
        t = 2.0 ** e + (np.arange(2048) + 0.5) * 2.0 ** (e - 11)
        xs += [t, np.nextafter(t, 0), np.nextafter(t, 2)]
    xs.append(np.exp2(rng.uniform(-40.0, 0.2, 200000)))
    xs.append(np.array([0.0, 1.0 - 2.0 ** -12, 1.0 - 2.0 ** -13, 1.0, 1.5, 2.0 ** -15, 2.0 ** -26]))
    g = np.concatenate(xs)
    g32 = np.concatenate([g, -g]).astype(np.float32)
    code, v32 = encode_steps(g32)
    # exactly the definition applied to the FP32 product the device rounds
    assert np.array_equal(code, encode_ref((v32.astype(np.float64) * 2.0 ** 111)))
    # and to g itself wherever that product is an FP32 normal; one code at most below
    direct = encode_ref(g32)
    normal = np.abs(g32.astype(np.float64)) >= 2.0 ** -15
    assert np.array_equal(code[normal], direct[normal])
    assert np.max(np.abs(code.astype(np.int64) - direct.astype(np.int64))) <= 1


def test_decode_steps_invert_exactly():
    h = np.arange(1 << 16, dtype=np.uint32)
    g = decode_steps(h)
    assert np.array_equal(g.astype(np.float64), decode_ref(h))
    code, _ = encode_steps(g)
    keep = (h & 0x7FFF) != 0
    assert np.array_equal(code[keep], h[keep])
