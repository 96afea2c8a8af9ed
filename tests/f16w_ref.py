"""NumPy restatement of the weight-scaled 16-bit format of MPH_PREC_F16W from
its definition (shared by the CPU and GPU tests): x = (f - w) / p, p the
power of two nearest to w, as sign, 3 exponent bits biased by 8 and 12
mantissa bits; x = 2^(e - 8) (1 + m / 2^12) for e = 1..7, multiples of 2^-19
below 2^-7, round to nearest with ties to even, saturation at 1 - 2^-13."""
import numpy as np


def pscale(w):
    """The power of two nearest to w (no weight lies near a tie)."""
    return np.exp2(np.round(np.log2(w)))


def round_ref(xs):
    """Round x (float64, exact) to the 1-3-12 grid (nearest, ties to even):
    x = 2^(e - 8) (1 + m / 2^12), e = 1..7, and multiples of 2^-19 below
    2^-7; magnitudes beyond the largest saturate.  Returns codes."""
    x = np.abs(xs)
    mant, ex = np.frexp(x)
    e = ex.astype(np.int64) - 1                  # x = (2 mant) 2^e
    normal = x >= 2.0 ** -7
    m = np.rint((2.0 * mant - 1.0) * 4096.0).astype(np.int64)
    carry = m == 4096
    e2 = np.where(carry, e + 1, e)
    m2 = np.where(carry, 0, m)
    code_n = np.where(e2 + 8 > 7, 0x7FFF, ((e2 + 8) << 12) | m2)
    code_s = np.rint(x / 2.0 ** -19).astype(np.int64)   # 4096 is the smallest normal
    code = np.where(normal, code_n, code_s).astype(np.uint32)
    return code | np.where(np.signbit(xs), 0x8000, 0).astype(np.uint32)


def decode_ref(h):
    """x of each code (float64, exact)."""
    h = h.astype(np.int64)
    e, m = (h >> 12) & 0x7, h & 0xFFF
    x = np.where(e > 0, np.exp2(e - 8.0) * (1.0 + m / 4096.0), m * 2.0 ** -19)
    return np.where(h & 0x8000, -x, x)
