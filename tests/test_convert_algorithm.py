"""The integer-pipe binary32 <-> binary64 conversions of the FP32-mixed kernels
(openmhd_gb300/csrc/omhd_fastmath.h: narrow_f64, widen_f32), their bit
manipulation restated step for step in numpy and checked on the host against
numpy's IEEE conversions (round to nearest even), without a GPU.  The device
functions themselves are checked the same way on the GPU by
tests/test_gpu_convert.py; this file pins the algorithm."""
import numpy as np

from test_gpu_convert import TINY32, _doubles, _floats

U32 = np.uint64(0xFFFFFFFF)


def narrow(x: np.ndarray) -> np.ndarray:
    """narrow_f64 on 64-bit patterns: add half an ulp of the result minus one
    plus the kept lowest bit, drop 29 bits, rebias 1023 -> 127; |x| >= 2^128
    -> inf, |x| < 2^-126 -> zero, NaN -> quiet NaN; sign kept."""
    b = x.view(np.uint64)
    hi, lo = b >> np.uint64(32), b & U32
    ahi = hi & np.uint64(0x7FFFFFFF)
    a = (ahi << np.uint64(32)) | lo
    r = a + (np.uint64(0x0FFFFFFF) + ((lo >> np.uint64(29)) & np.uint64(1)))
    f = (((r >> np.uint64(29)) & U32) - np.uint64(896 << 23)) & U32
    f = np.where(ahi >= 0x47F00000, np.uint64(0x7F800000), f)
    f = np.where(ahi < 0x38100000, np.uint64(0), f)
    f = np.where(a > np.uint64(0x7FF0000000000000), np.uint64(0x7FC00000), f)
    return (f | (hi & np.uint64(0x80000000))).astype(np.uint32).view(np.float32)


def widen(f: np.ndarray) -> np.ndarray:
    """widen_f32 on 32-bit patterns: rebias the exponent in the high word
    (twice for inf/NaN), move the three low mantissa bits to the low word;
    subnormals -> signed zero."""
    u = f.view(np.uint32).astype(np.uint64)
    mag = u & np.uint64(0x7FFFFFFF)
    hi = ((mag >> np.uint64(3)) + np.where(mag >= 0x7F800000, np.uint64(0x70000000), np.uint64(0x38000000))) & U32
    lo = (u << np.uint64(29)) & U32
    z = mag < 0x00800000
    hi, lo = np.where(z, np.uint64(0), hi), np.where(z, np.uint64(0), lo)
    return (((hi | (u & np.uint64(0x80000000))) << np.uint64(32)) | lo).view(np.float64)


def test_narrow_algorithm_matches_ieee():
    x = _doubles(np.random.default_rng(7))
    got = narrow(x)
    nan = np.isnan(x)
    small = ~nan & (np.abs(x) < TINY32)
    big = ~nan & ~small
    with np.errstate(over="ignore"):
        want = x[big].astype(np.float32)
    assert np.array_equal(want.view(np.uint32), got[big].view(np.uint32))
    assert np.all(got[small] == 0) and np.all(np.signbit(got[small]) == np.signbit(x[small]))
    assert np.all(np.isnan(got[nan]))


def test_widen_algorithm_is_exact():
    f = _floats(np.random.default_rng(8))
    got = widen(f)
    nan = np.isnan(f)
    sub = ~nan & (f != 0) & (np.abs(f) < np.finfo(np.float32).tiny)
    rest = ~nan & ~sub
    assert np.array_equal(f[rest].astype(np.float64).view(np.uint64), got[rest].view(np.uint64))
    assert np.all(got[sub] == 0) and np.all(np.signbit(got[sub]) == np.signbit(f[sub]))
    assert np.all(np.isnan(got[nan])) and np.all(np.signbit(got[nan]) == np.signbit(f[nan]))
