"""NumPy restatement of the 1-4-11 16-bit format of MPH_PREC_F16C from its
definition (shared by the CPU and GPU tests): f - w as sign, 4 exponent bits
biased by 16 and 11 mantissa bits; v = 2^(e - 16) (1 + m / 2^11) for
e = 1..15, multiples of 2^-26 below 2^-15, round to nearest with ties to
even, saturation at 1 - 2^-12."""
import numpy as np


def encode_ref(g32):
    """Round FP32 deviations to the 1-4-11 format (nearest, ties to even),
    from the value definition v = 2^(e - 16) (1 + m / 2^11), e = 1..15, and
    v = 2^-15 m / 2^11 for e = 0; magnitudes beyond the largest saturate."""
    g = g32.astype(np.float64)
    a = np.abs(g)
    mant, ex = np.frexp(a)           # a = mant 2^ex, mant in [0.5, 1)
    e = ex.astype(np.int64) - 1      # a = (2 mant) 2^e
    normal = (a >= 2.0 ** -15)
    sub = (a > 0) & ~normal
    # normals: significand rounded to 11 fraction bits
    sig = 2.0 * mant - 1.0                      # [0, 1), exact
    m = np.rint(sig * 2048.0).astype(np.int64)  # rint rounds half to even
    carry = m == 2048
    e2 = np.where(carry, e + 1, e)
    m2 = np.where(carry, 0, m)
    code_n = ((e2 + 16) << 11) | m2
    code_n = np.where(e2 + 16 > 15, 0x7FFF, code_n)
    # subnormals: multiples of 2^-26 (a result of 2048 is the smallest normal)
    code_s = np.rint(a / 2.0 ** -26).astype(np.int64)
    out = np.where(normal, code_n, np.where(sub, code_s, 0)).astype(np.uint32)
    out |= np.where(np.signbit(g), 0x8000, 0).astype(np.uint32)
    return out


def decode_ref(h):
    h = h.astype(np.int64)
    e, m = (h >> 11) & 0xF, h & 0x7FF
    v = np.where(e > 0, np.exp2(e - 16.0) * (1.0 + m / 2048.0), m * 2.0 ** -26)
    return np.where(h & 0x8000, -v, v)
