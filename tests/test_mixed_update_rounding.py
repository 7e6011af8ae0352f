"""Why the FP32-mixed update accumulates in plain binary64, without compensated
summation, shown on the host (no GPU).

The FP32-mixed stage kernels (openmhd_gb300/csrc/omhd_fused2d.cuh,
phase_update; omhd_fused3d.cuh, the plane update) widen each binary32 face
flux to binary64 and form, per variable, F(i-1/2) - F(i+1/2) (+ G(j-1/2) -
G(j+1/2)), scale it by dt/dx and add it to the state: the operation order of
rk.f90:26-35 (rk_tvd21) and rk.f90:56-66 (rk_tvd22) of the reference's
2D_basic.  Two facts make compensated summation of that update unnecessary:

1. the difference of two binary32 numbers whose exponents differ by at most
   29 is exact in binary64 (the 24-bit significands span at most 53 bits), so
   the flux differences themselves carry no rounding; at a larger gap the one
   rounding is relative to the larger flux;
2. what is rounded -- dt/dx times the difference, the x + y sum, U + d -- is a
   few binary64 ulps per stage, which over a long run stays five to six
   orders of magnitude below the rounding of the face fluxes to binary32
   that sets the mixed path's error (6e5 in the third test).  A Kahan residual carried across steps would remove only the
   former, and would need a second binary64 state array.
"""
import numpy as np


def _two_sum_error(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """The rounding error of a + b in binary64 (Knuth's TwoSum, exact for
    finite operands): zero exactly when a + b is representable."""
    s = a + b
    bb = s - a
    return (a - (s - bb)) + (b - bb)


def _binary32_pairs(rng, n: int, gap: int):
    """n binary32 pairs (a, b): a with a random exponent in [-40, 40), b with
    the exponent gap below it, random significands and signs."""
    ma = rng.integers(1 << 23, 1 << 24, n).astype(np.float64)
    mb = rng.integers(1 << 23, 1 << 24, n).astype(np.float64)
    ea = rng.integers(-40, 40, n)
    sa = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    sb = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    a = (sa * np.ldexp(ma, ea - 23)).astype(np.float32)
    b = (sb * np.ldexp(mb, ea - gap - 23)).astype(np.float32)
    return a.astype(np.float64), b.astype(np.float64)


def test_binary32_flux_differences_are_exact_in_binary64():
    rng = np.random.default_rng(11)
    for gap in range(0, 30):
        a, b = _binary32_pairs(rng, 50_000, gap)
        assert np.count_nonzero(_two_sum_error(a, -b)) == 0, gap


def test_exactness_ends_at_an_exponent_gap_of_30():
    # 2^30 (1 + 2^-23) - (-(1 + 2^-23)) has set bits from 2^30 down to 2^-23: 54
    # bits, one more than binary64 holds; the bound of the first test is tight
    a = np.float64(np.float32(2.0**30 * (1 + 2.0**-23)))
    b = np.float64(np.float32(-(1 + 2.0**-23)))
    assert _two_sum_error(np.array([a]), np.array([-b]))[0] != 0
    rng = np.random.default_rng(12)
    a, b = _binary32_pairs(rng, 50_000, 30)
    assert np.count_nonzero(_two_sum_error(a, -b)) > 0


def _dd_add(hi: np.ndarray, lo: np.ndarray, x: np.ndarray):
    """(hi + lo) + x in double-double arithmetic (TwoSum, then renormalise):
    an accumulation that loses nothing a compensated sum could recover."""
    s = hi + x
    bb = s - hi
    e = (hi - (s - bb)) + (x - bb) + lo
    h = s + e
    return h, e - (h - s)


def test_update_roundings_stay_far_below_the_binary32_face_rounding():
    """2000 TVD-RK2 steps of the kernels' update arithmetic on 4096 cells with
    random face fluxes (fresh each stage, |F| <= 1e-2 against a state of order
    1) and dt/dx = dt/dy = 0.2: the state accumulated in plain binary64, as the
    kernels do, against (a) the same updates accumulated in double-double --
    all that compensated summation could recover -- and (b) plain binary64
    from the unrounded binary64 fluxes -- the binary32 face rounding."""
    rng = np.random.default_rng(13)
    n, steps = 4096, 2000
    dtx = dty = 0.2
    u0 = rng.uniform(0.5, 1.5, n)
    u_plain, u_f64 = u0.copy(), u0.copy()
    acc_hi, acc_lo = u0.copy(), np.zeros(n)

    def update(F, G):
        # FX(i-1/2) - FX(i+1/2) and FY(j-1/2) - FY(j+1/2), then the dx != dy
        # form of the kernels' update: dtx * dF + dty * (gm - gp)
        return dtx * (F[0] - F[1]) + dty * (G[0] - G[1])

    for _ in range(steps):
        start = (u_plain.copy(), u_f64.copy(), acc_hi.copy(), acc_lo.copy())
        for stage in (1, 2):
            F = rng.uniform(-1.0, 1.0, (2, n)) * 1e-2
            G = rng.uniform(-1.0, 1.0, (2, n)) * 1e-2
            d32 = update(F.astype(np.float32).astype(np.float64), G.astype(np.float32).astype(np.float64))
            d64 = update(F, G)
            acc_hi, acc_lo = _dd_add(acc_hi, acc_lo, d32)
            if stage == 1:  # rk_tvd21: U* = U + d
                u_plain = u_plain + d32
                u_f64 = u_f64 + d64
            else:  # rk_tvd22: U = (U0 + U* + d) / 2
                u_plain = 0.5 * (start[0] + u_plain + d32)
                u_f64 = 0.5 * (start[1] + u_f64 + d64)
                acc_hi, acc_lo = _dd_add(acc_hi, acc_lo, start[2])
                acc_hi, acc_lo = _dd_add(acc_hi, acc_lo, start[3])
                acc_hi, acc_lo = 0.5 * acc_hi, 0.5 * acc_lo

    scale = np.mean(np.abs(u_f64))
    recoverable = np.mean(np.abs((u_plain - acc_hi) - acc_lo)) / scale
    face_rounding = np.mean(np.abs(u_plain - u_f64)) / scale
    assert recoverable < 1e-14
    assert face_rounding > 1e-10
    assert face_rounding > 1e4 * recoverable
